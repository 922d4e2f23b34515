"""rubix_cube_fwd_noalloc: the allocation-free variant of the fused cube kernel.

It is meant for callers that cannot allocate device memory when they render (a host
that owns all GPU memory through its own pool, a loop that must stay out of the
allocator), so it takes its scratch from a static device array instead of a caller
workspace.  These tests call it through the C ABI and compare its cube with the one
rubix_cube_fwd produces from the same inputs -- bit for bit, since both run the same
deterministic kernel -- twice in a row (the second call finds the first call's
leftovers in the shared array), read the device error word of each call through
rubix_cube_noalloc_status, compare one cube with the float64 oracle, and check that a
problem too large for the array is refused before any GPU work.

This file is named so that pytest collects it last.
"""

import ctypes

import numpy as np
import pytest

import oracle
from helpers import CUBE_RTOL, assert_cube_close, to_dev, workload

pytestmark = pytest.mark.gpu

_vp, _i32, _i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
_ARGTYPES = [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _i32,
             _vp, _vp, _vp, _vp, _i64, _i32,
             _vp, _vp, _i32, _i64, _vp, _i32, _i32, _vp, _i64, _vp]
RUBIX_E_WORKSPACE = -3


def _bind(lib):
    fn = lib.rubix_cube_fwd_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = _ARGTYPES
    st = lib.rubix_cube_noalloc_status
    st.restype = ctypes.c_int
    st.argtypes = [ctypes.POINTER(ctypes.c_int), _vp]
    return fn, st


def _inputs():
    import torch

    from rubix_gb300 import ops

    w = workload("small")
    p = w.particles
    d = {k: to_dev(getattr(p, k)) for k in ("coords", "velocity", "mass", "metallicity", "age")}
    ssp = {"flux": to_dev(w.ssp.flux), "met": to_dev(w.ssp.metallicity),
           "age": to_dev(w.ssp.age), "wz": to_dev(w.wave_z), "wt": to_dev(w.wave_t)}
    edges = to_dev(w.edges)
    nseg = w.sbin * w.sbin
    perm, offs = ops.spaxel_sort(ops.spaxel_assign(d["coords"], edges), nseg,
                                 ops.aperture_mask(d["coords"], edges))
    torch.cuda.synchronize()
    return w, d, ssp, perm, offs, nseg


def _call(fn, w, d, ssp, perm, offs, nseg, out, n=None):
    import torch

    nz, na, nw = w.ssp.flux.shape
    L = w.wave_t.size
    return fn(ssp["flux"].data_ptr(), ssp["met"].data_ptr(), ssp["age"].data_ptr(),
              ssp["wz"].data_ptr(), nz, na, nw, ssp["wt"].data_ptr(), L,
              d["mass"].data_ptr(), d["metallicity"].data_ptr(), d["age"].data_ptr(),
              d["velocity"].data_ptr(), 3, 2, perm.data_ptr(), offs.data_ptr(), nseg,
              d["mass"].numel() if n is None else n, None, 0, 0, out.data_ptr(), L,
              torch.cuda.current_stream().cuda_stream)


def test_noalloc_matches_workspace_entry_point_twice(rubix_lib):
    import torch

    from rubix_gb300 import ops

    w, d, ssp, perm, offs, nseg = _inputs()
    ref = ops.cube_forward(ssp["flux"], ssp["met"], ssp["age"], ssp["wz"], ssp["wt"], d["mass"],
                           d["metallicity"], d["age"], d["velocity"], 2, perm, offs, nseg,
                           check=True)
    torch.cuda.synchronize()
    fn, status = _bind(rubix_lib)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out = torch.full((nseg, w.wave_t.size), float("nan"), dtype=torch.float32, device="cuda")
        rc = _call(fn, w, d, ssp, perm, offs, nseg, out)
        assert rc == 0, rubix_lib.rubix_last_error().decode()
        err = ctypes.c_int(-1)
        rc = status(ctypes.byref(err), stream)
        assert rc == 0 and err.value == 0, rubix_lib.rubix_last_error().decode()
        torch.cuda.synchronize()
        n_diff = int((out != ref).sum())
        assert torch.equal(out, ref), f"call {call}: {n_diff} elements differ from rubix_cube_fwd"
    # the same cube against the float64 oracle (spaxel sum before PSF and LSF)
    p = w.particles
    want = oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                              w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux,
                              w.ssp.wavelength, w.dist_z, w.wave_t)["cube"]
    assert_cube_close(out.cpu().numpy().reshape(want.shape), want, rtol=CUBE_RTOL,
                      what="no-alloc cube vs oracle")


def test_noalloc_rejects_problem_beyond_static_scratch(rubix_lib):
    import torch

    w, d, ssp, perm, offs, nseg = _inputs()
    fn, _ = _bind(rubix_lib)
    out = torch.empty((nseg, w.wave_t.size), dtype=torch.float32, device="cuda")
    # 10^9 particles need far more scratch than the static array holds; the call is
    # refused on the host before any pointer is used.
    rc = _call(fn, w, d, ssp, perm, offs, nseg, out, n=1_000_000_000)
    assert rc == RUBIX_E_WORKSPACE
    assert b"static array" in rubix_lib.rubix_last_error()
