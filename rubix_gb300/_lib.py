"""ctypes binding of ``librubix_gb300.so`` (the C ABI declared in include/rubix_gb300.h).

The library is the only compute path of this package: there is no CPU or eager
PyTorch fallback.  If the shared object is missing, ``lib()`` raises with the
command that builds it.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import _build

_c = ctypes
_vp = _c.c_void_p
_i32 = _c.c_int32
_i64 = _c.c_int64
_sz = _c.c_size_t
_f32p = _c.c_void_p  # device pointers travel as void*

RUBIX_OK = 0
ERROR_NAMES = {
    -1: "RUBIX_E_INVALID",
    -2: "RUBIX_E_SHAPE",
    -3: "RUBIX_E_WORKSPACE",
    -4: "RUBIX_E_CUDA",
    -5: "RUBIX_E_DEVICE",
    -6: "RUBIX_E_UNSUPPORTED",
}

# name -> (restype, argtypes); mirrors include/rubix_gb300.h
SIGNATURES = {
    "rubix_abi_version": (_c.c_int, []),
    "rubix_last_error": (_c.c_char_p, []),
    "rubix_aperture_mask": (_c.c_int, [_vp, _i64, _i64, _vp, _i32, _vp, _vp]),
    "rubix_spaxel_assign": (_c.c_int, [_vp, _i64, _i64, _vp, _i32, _vp, _vp]),
    "rubix_spaxel_sort_workspace_size": (_sz, [_i64, _i32]),
    "rubix_spaxel_sort": (_c.c_int, [_vp, _vp, _i64, _i32, _vp, _vp, _vp, _sz, _vp]),
    "rubix_cube_workspace_size": (_sz, [_i64, _i32, _i32, _i32, _i32, _i32]),
    "rubix_cube_status": (_c.c_int, [_vp, _c.POINTER(_c.c_int), _vp]),
    "rubix_cube_fwd": (
        _c.c_int,
        [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _i32,
         _vp, _vp, _vp, _vp, _i64, _i32,
         _vp, _vp, _i32, _i64, _vp, _i32, _i32, _vp, _i64, _vp, _sz, _vp],
    ),
    "rubix_cube_fwd_dust": (
        _c.c_int,
        [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _i32,
         _vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp,
         _vp, _vp, _i32, _i64, _vp, _i32, _i32, _vp, _i64, _vp, _sz, _vp],
    ),
    "rubix_dust_gas_extinction": (_c.c_int, [_vp, _vp, _i64, _i32, _i32, _i64, _vp, _i32,
                                             _c.c_float, _c.c_float, _vp, _vp]),
    "rubix_dust_apply_rows": (_c.c_int, [_vp, _i64, _i32, _i64, _vp, _vp, _vp]),
    "rubix_fits_cube_layout": (_c.c_int, [_vp, _i32, _i32, _i32, _i64, _vp, _vp]),
    "rubix_psf_fwd_dtaps": (_c.c_int, [_vp, _vp, _i32, _i32, _i32, _i64, _i64, _vp, _i32,
                                       _vp, _i32, _vp]),
    "rubix_lsf_fwd_dtaps": (_c.c_int, [_vp, _vp, _i64, _i32, _i64, _i64, _vp, _i32, _i32,
                                       _vp]),
    "rubix_gauss_taps": (_c.c_int, [_vp, _vp, _i32, _vp, _vp, _vp, _i32, _vp]),
    "rubix_dust_av_workspace_size": (_sz, [_i64, _i32]),
    "rubix_dust_av": (_c.c_int, [_vp, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _i64, _i32, _i32,
                                 _vp, _vp, _sz, _vp]),
    "rubix_cube_fwd_noalloc": (
        _c.c_int,
        [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _i32,
         _vp, _vp, _vp, _vp, _i64, _i32,
         _vp, _vp, _i32, _i64, _vp, _i32, _i32, _vp, _i64, _vp],
    ),
    "rubix_cube_noalloc_status": (_c.c_int, [_c.POINTER(_c.c_int), _vp]),
    "rubix_ssp_lookup": (_c.c_int, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "rubix_mask_zero": (_c.c_int, [_vp, _i64, _i32, _i64, _vp, _vp]),
    "rubix_scale_rows": (_c.c_int, [_vp, _i64, _vp, _i64, _i32, _vp, _i64, _vp]),
    "rubix_resample_rows": (
        _c.c_int, [_vp, _i64, _vp, _i32, _vp, _i64, _i32, _i64, _vp, _i32, _vp, _i64, _vp]
    ),
    "rubix_segment_sum_rows": (_c.c_int, [_vp, _i64, _i32, _vp, _vp, _i32, _vp, _i64, _vp]),
    "rubix_psf_fwd": (
        _c.c_int, [_vp, _vp, _i32, _i32, _i32, _i64, _i64, _vp, _i32, _vp, _i32, _vp]
    ),
    "rubix_psf_status": (_c.c_int, [_c.POINTER(_c.c_int), _vp]),
    "rubix_fused_dot_workspace_size": (_sz, []),
    "rubix_psf_dot_dtaps": (
        _c.c_int, [_vp, _i64, _vp, _i64, _i32, _i32, _i32, _vp, _vp, _i32, _vp, _vp, _sz, _vp]
    ),
    "rubix_lsf_dot_dtaps": (
        _c.c_int, [_vp, _i64, _i32, _i64, _vp, _i64, _vp, _i32, _i32, _vp, _vp, _sz, _vp]
    ),
    "rubix_lsf_fwd": (_c.c_int, [_vp, _vp, _i64, _i32, _i64, _i64, _vp, _i32, _i32, _vp]),
    "rubix_cube_bwd_workspace_size": (_sz, [_i64, _i32, _i32, _i32, _i32, _i32]),
    "rubix_cube_bwd": (
        _c.c_int,
        [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _i32,
         _vp, _vp, _vp, _vp, _i64, _i32,
         _vp, _vp, _i32, _i64,
         _vp, _i64, _vp, _vp, _vp, _vp,
         _vp, _sz, _vp],
    ),
    "rubix_cube_bwd_dust": (
        _c.c_int,
        [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _i32,
         _vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp,
         _vp, _vp, _i32, _i64,
         _vp, _i64, _vp, _vp, _vp, _vp,
         _vp, _sz, _vp],
    ),
    "rubix_cube_bwd_dust_av": (
        _c.c_int,
        [_vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _i32,
         _vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp,
         _vp, _vp, _i32, _i64,
         _vp, _i64, _vp, _vp, _vp, _vp, _vp,
         _vp, _sz, _vp],
    ),
    "rubix_dust_av_bwd_workspace_size": (_sz, [_i64, _i32, _i64]),
    "rubix_dust_av_bwd": (_c.c_int, [_vp, _i64, _vp, _vp, _i64, _vp, _i64, _vp, _i64, _i32,
                                     _i32, _vp, _vp, _vp, _vp, _sz, _vp]),
    "rubix_dust_gas_extinction_bwd": (_c.c_int, [_vp, _vp, _i64, _i32, _i32, _i64, _vp, _i32,
                                                 _c.c_float, _c.c_float, _vp, _vp, _vp, _vp,
                                                 _vp]),
    "rubix_ragged_assign": (_c.c_int, [_vp, _i64, _i64, _vp, _i32, _vp, _vp, _vp, _vp, _vp,
                                       _vp, _vp]),
    "rubix_ragged_psf_fwd": (_c.c_int, [_vp, _vp, _i32, _i64, _i64, _i32, _vp, _vp, _vp, _i32,
                                        _vp, _i32, _vp]),
    "rubix_segmented_dot_workspace_size": (_sz, [_i32]),
    "rubix_segmented_dot": (_c.c_int, [_vp, _vp, _vp, _i32, _vp, _vp, _sz, _vp]),
    "rubix_inertia_workspace_size": (_sz, []),
    "rubix_inertia_tensor": (_c.c_int, [_vp, _i64, _i64, _vp, _c.c_float, _vp, _vp, _sz, _vp]),
    "rubix_rotate_vectors": (_c.c_int, [_vp, _vp, _i64, _i64, _i64, _vp, _vp]),
    "rubix_orient_filter_assign": (
        _c.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp]
    ),
    "rubix_flux_image": (_c.c_int, [_vp, _i64, _i32, _i64, _vp, _vp]),
    "rubix_noise_median_workspace_size": (_sz, []),
    "rubix_noise_median": (_c.c_int, [_vp, _i64, _vp, _vp, _sz, _vp]),
    "rubix_apply_noise": (_c.c_int, [_vp, _i64, _i32, _i64, _vp, _vp, _c.c_float, _i32,
                                     _c.c_uint64, _vp]),
    "rubix_philox4x32_10": (_c.c_int, [_vp, _vp, _vp]),
    "rubix_cube_tuning_set": (_c.c_int, [_i32, _vp]),
    "rubix_cube_tuning_get": (_c.c_int, [_i32, _vp]),
    "rubix_dot_workspace_size": (_sz, []),
    "rubix_dot": (_c.c_int, [_vp, _vp, _i64, _vp, _vp, _sz, _vp]),
}

_lock = threading.Lock()
_lib = None


class RubixError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, func: str, code: int, message: str):
        self.code = code
        self.func = func
        super().__init__(f"{func} -> {ERROR_NAMES.get(code, code)}: {message}")


def library_path() -> str:
    return _build.LIB_PATH


def lib():
    """Load the shared library once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"rubix_gb300 CUDA library not found at {path}; build it with "
                "`python -m rubix_gb300._build` (or __graft_entry__.build())"
            )
        h = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
        return _lib


def call(name: str, *args) -> None:
    """Call a status-returning entry point and raise RubixError on failure."""
    h = lib()
    rc = getattr(h, name)(*args)
    if rc != RUBIX_OK:
        msg = h.rubix_last_error()
        raise RubixError(name, rc, msg.decode() if msg else "")


def query(name: str, *args) -> int:
    return int(getattr(lib(), name)(*args))
