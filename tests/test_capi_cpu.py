"""The C-ABI library builds, loads and exports every symbol include/rubix_gb300.h
declares; argument validation runs on the host (no GPU work in these tests)."""

import ctypes
import os
import re

import pytest

from rubix_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rubix_gb300.h")


def header_functions():
    txt = open(HEADER).read()
    return re.findall(r"RUBIX_API\s+(?:const\s+)?\w+\**\s+(rubix_\w+)\s*\(", txt)


def test_header_lists_entry_points():
    names = header_functions()
    for expected in ("rubix_spaxel_assign", "rubix_spaxel_sort", "rubix_cube_fwd",
                     "rubix_psf_fwd", "rubix_lsf_fwd", "rubix_last_error"):
        assert expected in names


def test_library_exports_every_header_symbol(rubix_lib):
    names = header_functions()
    missing = [n for n in names if not hasattr(rubix_lib, n)]
    assert not missing, f"not exported: {missing}"
    unbound = [n for n in names if n not in _lib.SIGNATURES]
    assert not unbound, f"no ctypes signature for: {unbound}"


def test_abi_version_and_workspace_queries(rubix_lib):
    assert rubix_lib.rubix_abi_version() == 1
    a = _lib.query("rubix_spaxel_sort_workspace_size", 1000, 625)
    b = _lib.query("rubix_spaxel_sort_workspace_size", 100000, 625)
    assert 0 < a < b
    c = _lib.query("rubix_cube_workspace_size", 10000, 625, 3721, 6, 20, 1000)
    d = _lib.query("rubix_cube_workspace_size", 100000, 625, 3721, 6, 20, 1000)
    assert 0 < c < d
    assert _lib.query("rubix_cube_workspace_size", -1, 625, 3721, 6, 20, 1000) == 0


@pytest.mark.parametrize("call,code,msg", [
    (lambda h: h.rubix_spaxel_assign(None, -1, 3, None, 2, None, None), -1, "n < 0"),
    (lambda h: h.rubix_spaxel_assign(None, 10, 3, None, 1, None, None), -2, "two edges"),
    (lambda h: h.rubix_psf_fwd(None, None, 4, 4, 8, 8, 8, None, 0, None, 3, None), -2,
     "kernel sizes"),
    (lambda h: h.rubix_lsf_fwd(None, None, 4, 8, 8, 8, None, 0, 0, None), -2, "n_taps"),
    (lambda h: h.rubix_cube_fwd(None, None, None, None, 1, 5, 10, None, 8, None, None, None,
                                None, 3, 2, None, None, 4, 10, None, 0, 0, None, 8, None, 0,
                                None), -2, ">= 2 metallicities"),
    (lambda h: h.rubix_cube_fwd(None, None, None, None, 2, 5, 10, None, 5000, None, None, None,
                                None, 3, 2, None, None, 4, 10, None, 0, 0, None, 5000, None, 0,
                                None), -2, "n_wave_t"),
    # The pointer arguments below are placeholders (256): each call is refused on the host
    # before any of them is used.
    (lambda h: h.rubix_cube_fwd_noalloc(*[256] * 4, 6, 221, 1221, 256, 3721, *[256] * 4, 3, 2,
                                        256, 256, 22500, 1_000_000_000, None, 0, 0, 256, 3721,
                                        None), -3, "static array"),
    # the same argument checks, hence the same codes, as rubix_cube_fwd
    (lambda h: h.rubix_cube_fwd_noalloc(*[256] * 4, 6, 221, 1221, 256, 3721, *[256] * 4, 3, 2,
                                        256, 256, 22500, 1 << 31, None, 0, 0, 256, 3721, None),
     -2, "bad n"),
    (lambda h: h.rubix_cube_fwd_noalloc(None, None, None, None, 6, 221, 1221, None, 3721, None,
                                        None, None, None, 3, 2, None, None, 22500, 10, None, 0,
                                        0, None, 3721, None), -1, "null pointer"),
    (lambda h: h.rubix_cube_fwd(None, None, None, None, 6, 221, 1221, None, 3721, None, None,
                                None, None, 3, 2, None, None, 22500, 10, None, 0, 0, None, 3721,
                                None, 0, None), -1, "null pointer"),
    (lambda h: h.rubix_cube_noalloc_status(None, None), -1, "null pointer"),
    (lambda h: h.rubix_psf_status(None, None), -1, "null pointer"),
    (lambda h: h.rubix_psf_dot_dtaps(None, 8, None, 8, 4, 4, 8, None, None, 15, None, None, 0,
                                     None), -1, "null output"),
    (lambda h: h.rubix_psf_dot_dtaps(None, 8, None, 8, 4, 4, 8, None, None, 23, None, None, 0,
                                     None), -6, "odd and <= 21"),
    (lambda h: h.rubix_lsf_dot_dtaps(None, 4, 8, 8, None, 8, None, 40, 0, None, None, 0, None),
     -6, "n_taps must be in"),
    (lambda h: h.rubix_lsf_dot_dtaps(None, 4, 8, 8, None, 8, None, 5, 2, None, None, 0, None),
     -1, "null output"),
    (lambda h: h.rubix_cube_fwd_dust(None, None, None, None, 6, 221, 1221, None, 3721, None,
                                     None, None, None, 3, 2, None, None, None, None, 22500, 10,
                                     None, 0, 0, None, 3721, None, 0, None), -1,
     "null A_V or extinction exponent"),
    (lambda h: h.rubix_dust_av(None, 3, None, None, 10, None, 3, None, 10, 0, 4, None, None, 0,
                               None), -2, "n_segments"),
    (lambda h: h.rubix_dust_av(None, 3, None, None, 10, None, 3, None, 10, 25, 16, None, None,
                               0, None), -2, "n_segments <= pa_limit"),
    (lambda h: h.rubix_dust_gas_extinction(None, None, 5, 0, 7, 10, None, 1, 1.0, 1.0, None,
                                           None), -1, "H/O columns"),
    (lambda h: h.rubix_fits_cube_layout(None, 4, 70000, 8, 8, None, None), -2,
     "65535 columns"),
    (lambda h: h.rubix_fits_cube_layout(None, 4, 4, 8, 4, None, None), -2, "spaxel_stride"),
    (lambda h: h.rubix_orient_filter_assign(None, None, 10, None, None, None, None, 1, 0, None,
                                            None, None, None, None, None), -2, "two edges"),
    (lambda h: h.rubix_orient_filter_assign(None, None, 10, None, None, None, None, 26, 9, None,
                                            None, None, None, None, None), -1,
     "n_fields must be in [0, 8]"),
    (lambda h: h.rubix_orient_filter_assign(None, None, 10, None, None, None, None, 26, 1, None,
                                            None, None, None, None, None), -1,
     "null field arrays"),
])
def test_host_side_validation(rubix_lib, call, code, msg):
    rc = call(rubix_lib)
    assert rc == code
    assert msg in rubix_lib.rubix_last_error().decode()


def test_ops_refuse_cpu_tensors(rubix_lib):
    import torch

    from rubix_gb300 import ops

    with pytest.raises(ValueError, match="CUDA"):
        ops.spaxel_assign(torch.zeros(3, 3), torch.zeros(4))
    with pytest.raises(ValueError, match="CUDA"):
        ops.psf_forward(torch.zeros(2, 2, 2), [1.0])
