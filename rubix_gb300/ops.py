"""Torch-facing wrappers of the C ABI: one function per kernel entry point.

Tensors must live on a CUDA device; they are passed to the library as raw device
pointers together with the current torch stream.  Workspaces come from torch's
caching allocator, so the library itself never allocates.  Every function raises
(``ValueError`` for bad arguments, ``RubixError`` for a failing C-ABI call) and none
has a CPU path.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib

__all__ = [
    "aperture_mask",
    "spaxel_assign",
    "spaxel_sort",
    "cube_forward",
    "psf_forward",
    "lsf_forward",
    "cube_backward",
    "dot",
    "flux_image",
    "noise_median",
    "apply_noise_",
    "dust_gas_extinction",
    "dust_av",
    "dust_apply_rows_",
    "fits_cube_layout",
    "workspace",
]


# Number of this library's kernels launched through these wrappers (per process).
LAUNCHES = {"count": 0}


def _count(k: int) -> None:
    LAUNCHES["count"] += int(k)


def _sort_passes(n_segments: int) -> int:
    bits = max(1, int(n_segments).bit_length())
    return (bits + 7) // 8


def _stream(dev: torch.device) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


def _check_cuda(name: str, t: torch.Tensor, dtype=None) -> None:
    if not isinstance(t, torch.Tensor):
        raise ValueError(f"{name} must be a torch.Tensor, got {type(t).__name__}")
    if t.device.type != "cuda":
        raise ValueError(f"{name} must be a CUDA tensor (rubix_gb300 has no CPU path)")
    if dtype is not None and t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")


def _contig(name: str, t: torch.Tensor, dtype) -> torch.Tensor:
    _check_cuda(name, t, None)
    if t.dtype != dtype:
        t = t.to(dtype)
    return t.contiguous()


def workspace(nbytes: int, device) -> torch.Tensor:
    """A device scratch buffer of at least ``nbytes`` bytes (256-byte aligned)."""
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


def _ptr(t):
    return None if t is None else t.data_ptr()


def aperture_mask(coords: torch.Tensor, edges: torch.Tensor) -> torch.Tensor:
    """uint8 mask of particles inside [min(edges), max(edges)]^2 (x, y columns)."""
    coords = _contig("coords", coords, torch.float32)
    edges = _contig("edges", edges, torch.float32)
    n = coords.shape[0]
    out = torch.empty(n, dtype=torch.uint8, device=coords.device)
    stride = coords.shape[1] if coords.dim() == 2 else 1
    _lib.call("rubix_aperture_mask", _ptr(coords), n, stride, _ptr(edges), edges.numel(),
              _ptr(out), _stream(coords.device))
    _count(1 if n > 0 else 0)
    return out


def spaxel_assign(coords: torch.Tensor, edges: torch.Tensor) -> torch.Tensor:
    """int32 flat spaxel index ix + nb*iy (square_spaxel_assignment semantics)."""
    coords = _contig("coords", coords, torch.float32)
    edges = _contig("edges", edges, torch.float32)
    if coords.dim() != 2 or coords.shape[1] < 2:
        raise ValueError(f"coords must be (n, >=2), got {tuple(coords.shape)}")
    n = coords.shape[0]
    out = torch.empty(n, dtype=torch.int32, device=coords.device)
    _lib.call("rubix_spaxel_assign", _ptr(coords), n, coords.shape[1], _ptr(edges),
              edges.numel(), _ptr(out), _stream(coords.device))
    _count(1 if n > 0 else 0)
    return out


def spaxel_sort(idx: torch.Tensor, n_segments: int, keep: torch.Tensor | None = None):
    """Stable sort by spaxel; returns (perm int32 [n], seg_offsets int32 [n_segments+1])."""
    idx = _contig("idx", idx, torch.int32)
    if keep is not None:
        keep = _contig("keep", keep, torch.uint8)
        if keep.numel() != idx.numel():
            raise ValueError("keep must have one entry per particle")
    n = idx.numel()
    dev = idx.device
    perm = torch.empty(n, dtype=torch.int32, device=dev)
    offs = torch.empty(int(n_segments) + 1, dtype=torch.int32, device=dev)
    nbytes = _lib.query("rubix_spaxel_sort_workspace_size", n, int(n_segments))
    ws = workspace(nbytes, dev)
    _lib.call("rubix_spaxel_sort", _ptr(idx), _ptr(keep), n, int(n_segments), _ptr(perm),
              _ptr(offs), _ptr(ws), ws.numel(), _stream(dev))
    _count(2 + 3 * _sort_passes(n_segments) if n > 0 else 0)
    return perm, offs


def cube_forward(ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z, wave_t, mass, metallicity,
                 age, velocity, vel_component, perm, seg_offsets, n_segments, out=None,
                 lsf_taps=None, lsf_crop=0, check=False, dust_av=None, dust_exponent=None):
    """Fused lookup + mass + Doppler/resample + per-spaxel sum -> cube [n_segments, L].

    ``lsf_taps`` (optional) adds the LSF convolution along wavelength of every finished
    spectrum.  ``dust_av`` ([n], A_V per particle) with ``dust_exponent`` ([L],
    -0.4 log2(10) A(lambda)/A(V)) multiplies every resampled spectrum by its dust
    transmission before the sum.  ``check=True`` synchronises the stream and raises if
    the kernel reported a device error (a timed-out shared-memory copy wait)."""
    ssp_flux = _contig("ssp_flux", ssp_flux, torch.float32)
    if ssp_flux.dim() != 3:
        raise ValueError("ssp_flux must be [n_met, n_age, n_wave]")
    nz, na, nw = ssp_flux.shape
    ssp_metallicity = _contig("ssp_metallicity", ssp_metallicity, torch.float32)
    ssp_age = _contig("ssp_age", ssp_age, torch.float32)
    ssp_wave_z = _contig("ssp_wave_z", ssp_wave_z, torch.float32)
    wave_t = _contig("wave_t", wave_t, torch.float32)
    if ssp_metallicity.numel() != nz or ssp_age.numel() != na or ssp_wave_z.numel() != nw:
        raise ValueError("SSP grid sizes do not match ssp_flux")
    mass = _contig("mass", mass, torch.float32).reshape(-1)
    metallicity = _contig("metallicity", metallicity, torch.float32).reshape(-1)
    age = _contig("age", age, torch.float32).reshape(-1)
    velocity = _contig("velocity", velocity, torch.float32)
    n = mass.numel()
    if metallicity.numel() != n or age.numel() != n or velocity.shape[0] != n:
        raise ValueError("particle arrays must all have the same length")
    vstride = velocity.shape[1] if velocity.dim() == 2 else 1
    perm = _contig("perm", perm, torch.int32)
    seg_offsets = _contig("seg_offsets", seg_offsets, torch.int32)
    L = wave_t.numel()
    dev = mass.device
    if out is None:
        out = torch.empty((int(n_segments), L), dtype=torch.float32, device=dev)
    else:
        _check_cuda("out", out, torch.float32)
        if out.dim() != 2 or out.shape[0] != n_segments or out.shape[1] < L or out.stride(1) != 1:
            raise ValueError("out must be [n_segments, >=L] with unit stride along wavelength")
    lsf = None if lsf_taps is None else _host_taps(lsf_taps)
    nbytes = _lib.query("rubix_cube_workspace_size", n, int(n_segments), L, nz, na, nw)
    ws = workspace(nbytes, dev)
    lsf_args = (None if lsf is None else lsf.ctypes.data, 0 if lsf is None else lsf.size,
                int(lsf_crop))
    if (dust_av is None) != (dust_exponent is None):
        raise ValueError("dust_av and dust_exponent go together")
    if dust_av is None:
        _lib.call("rubix_cube_fwd", _ptr(ssp_flux), _ptr(ssp_metallicity), _ptr(ssp_age),
                  _ptr(ssp_wave_z), nz, na, nw, _ptr(wave_t), L, _ptr(mass), _ptr(metallicity),
                  _ptr(age), _ptr(velocity), vstride, int(vel_component), _ptr(perm),
                  _ptr(seg_offsets), int(n_segments), n, *lsf_args, _ptr(out), out.stride(0),
                  _ptr(ws), ws.numel(), _stream(dev))
    else:
        dust_av = _contig("dust_av", dust_av, torch.float32).reshape(-1)
        dust_exponent = _contig("dust_exponent", dust_exponent, torch.float32).reshape(-1)
        if dust_av.numel() != n or dust_exponent.numel() != L:
            raise ValueError("dust_av must be [n] and dust_exponent [L]")
        _lib.call("rubix_cube_fwd_dust", _ptr(ssp_flux), _ptr(ssp_metallicity),
                  _ptr(ssp_age), _ptr(ssp_wave_z), nz, na, nw, _ptr(wave_t), L, _ptr(mass),
                  _ptr(metallicity), _ptr(age), _ptr(velocity), vstride, int(vel_component),
                  _ptr(dust_av), _ptr(dust_exponent), _ptr(perm), _ptr(seg_offsets),
                  int(n_segments), n, *lsf_args, _ptr(out), out.stride(0), _ptr(ws),
                  ws.numel(), _stream(dev))
    # setup, corner table, prefix, count, scans (one launch), fill, main (+ gather)
    _count((7 + (1 if n > 0 else 0)) if n_segments > 0 else 0)
    if check and n_segments > 0:
        import ctypes

        err = ctypes.c_int(0)
        _lib.call("rubix_cube_status", _ptr(ws), ctypes.byref(err), _stream(dev))
    return out


def cube_backward(ssp_flux, ssp_metallicity, ssp_age, ssp_wave_z, wave_t, mass, metallicity,
                  age, velocity, vel_component, perm, seg_offsets, n_segments, adj,
                  dust_av=None, dust_exponent=None, av_grad=False):
    """Gradients (mass, metallicity, age, v_los) of <adj, cube> with cube the output of
    ``cube_forward`` without LSF (with the same ``dust_av`` / ``dust_exponent``);
    ``adj`` is [n_segments, >=L].  Four [n] tensors, zero for particles outside the
    sorted set; with ``av_grad`` (dust only) a fifth, dL/dA_V of every particle."""
    ssp_flux = _contig("ssp_flux", ssp_flux, torch.float32)
    nz, na, nw = ssp_flux.shape
    ssp_metallicity = _contig("ssp_metallicity", ssp_metallicity, torch.float32)
    ssp_age = _contig("ssp_age", ssp_age, torch.float32)
    ssp_wave_z = _contig("ssp_wave_z", ssp_wave_z, torch.float32)
    wave_t = _contig("wave_t", wave_t, torch.float32)
    mass = _contig("mass", mass, torch.float32).reshape(-1)
    metallicity = _contig("metallicity", metallicity, torch.float32).reshape(-1)
    age = _contig("age", age, torch.float32).reshape(-1)
    velocity = _contig("velocity", velocity, torch.float32)
    n = mass.numel()
    if metallicity.numel() != n or age.numel() != n or velocity.shape[0] != n:
        raise ValueError("particle arrays must all have the same length")
    vstride = velocity.shape[1] if velocity.dim() == 2 else 1
    perm = _contig("perm", perm, torch.int32)
    seg_offsets = _contig("seg_offsets", seg_offsets, torch.int32)
    L = wave_t.numel()
    _check_cuda("adj", adj, torch.float32)
    if adj.dim() != 2 or adj.shape[0] != n_segments or adj.shape[1] < L or adj.stride(1) != 1:
        adj = adj.reshape(int(n_segments), -1).contiguous()
    dev = mass.device
    if av_grad and dust_av is None:
        raise ValueError("av_grad needs dust_av and dust_exponent")
    grads = [torch.empty(n, dtype=torch.float32, device=dev) for _ in range(5 if av_grad else 4)]
    nbytes = _lib.query("rubix_cube_bwd_workspace_size", n, int(n_segments), L, nz, na, nw)
    ws = workspace(nbytes, dev)
    if (dust_av is None) != (dust_exponent is None):
        raise ValueError("dust_av and dust_exponent go together")
    if dust_av is None:
        _lib.call("rubix_cube_bwd", _ptr(ssp_flux), _ptr(ssp_metallicity), _ptr(ssp_age),
                  _ptr(ssp_wave_z), nz, na, nw, _ptr(wave_t), L, _ptr(mass), _ptr(metallicity),
                  _ptr(age), _ptr(velocity), vstride, int(vel_component), _ptr(perm),
                  _ptr(seg_offsets), int(n_segments), n, _ptr(adj), adj.stride(0),
                  *[_ptr(g) for g in grads], _ptr(ws), ws.numel(), _stream(dev))
    else:
        dust_av = _contig("dust_av", dust_av, torch.float32).reshape(-1)
        dust_exponent = _contig("dust_exponent", dust_exponent, torch.float32).reshape(-1)
        if dust_av.numel() != n or dust_exponent.numel() != L:
            raise ValueError("dust_av must be [n] and dust_exponent [L]")
        _lib.call("rubix_cube_bwd_dust_av" if av_grad else "rubix_cube_bwd_dust",
                  _ptr(ssp_flux), _ptr(ssp_metallicity), _ptr(ssp_age),
                  _ptr(ssp_wave_z), nz, na, nw, _ptr(wave_t), L, _ptr(mass), _ptr(metallicity),
                  _ptr(age), _ptr(velocity), vstride, int(vel_component), _ptr(dust_av),
                  _ptr(dust_exponent), _ptr(perm), _ptr(seg_offsets), int(n_segments), n,
                  _ptr(adj), adj.stride(0), *[_ptr(g) for g in grads], _ptr(ws), ws.numel(),
                  _stream(dev))
    # setup, corner table, prefix, count, scans (one launch), fill, adjoint (+ gather)
    _count((7 + (1 if n > 0 else 0)) if (n_segments > 0 and n > 0) else 0)
    return tuple(grads)


def dot(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Deterministic sum(a * b) of two float32 CUDA tensors of equal size, as a 0-d
    float64 tensor on the device."""
    _check_cuda("a", a, torch.float32)
    _check_cuda("b", b, torch.float32)
    if a.numel() != b.numel():
        raise ValueError("dot: sizes differ")
    a = a.contiguous().reshape(-1)
    b = b.contiguous().reshape(-1)
    out = torch.empty((), dtype=torch.float64, device=a.device)
    ws = workspace(_lib.query("rubix_dot_workspace_size"), a.device)
    _lib.call("rubix_dot", _ptr(a), _ptr(b), a.numel(), _ptr(out), _ptr(ws), ws.numel(),
              _stream(a.device))
    _count(1)
    return out


def psf_dot(cube: torch.Tensor, taps_y: torch.Tensor, taps_x: torch.Tensor,
            w: torch.Tensor) -> torch.Tensor:
    """sum(w * psf_forward(cube, taps_y, taps_x)) as a 0-d float64 device tensor, the
    convolution never written (device taps, odd count <= 21; the same arithmetic per
    element as psf_forward with device taps, a deterministic fixed-order sum)."""
    _check_cuda("cube", cube, torch.float32)
    _check_cuda("w", w, torch.float32)
    if cube.dim() != 3 or cube.stride(2) != 1 or cube.stride(0) != cube.shape[1] * cube.stride(1):
        cube = cube.contiguous()
    if w.shape != cube.shape:
        raise ValueError("psf_dot: w must have the cube's shape")
    if w.stride(2) != 1 or w.stride(0) != w.shape[1] * w.stride(1):
        w = w.contiguous()
    ny, nx, L = cube.shape
    ty = _contig("taps_y", taps_y, torch.float32).reshape(-1)
    tx = _contig("taps_x", taps_x, torch.float32).reshape(-1)
    if ty.numel() != tx.numel():
        raise ValueError("psf_dot: taps_y and taps_x must have the same length")
    out = torch.empty((), dtype=torch.float64, device=cube.device)
    ws = workspace(_lib.query("rubix_fused_dot_workspace_size"), cube.device)
    _lib.call("rubix_psf_dot_dtaps", _ptr(cube), cube.stride(1), _ptr(w), w.stride(1), ny, nx,
              L, _ptr(ty), _ptr(tx), ty.numel(), _ptr(out), _ptr(ws), ws.numel(),
              _stream(cube.device))
    _count(1)
    return out


def lsf_dot(cube: torch.Tensor, taps: torch.Tensor, crop: int, w: torch.Tensor) -> torch.Tensor:
    """sum(w * lsf_forward(cube, taps, crop)) over rows [..., L] as a 0-d float64 device
    tensor, the convolution never written (device taps, at most 28; the arithmetic of
    lsf_forward per element, a deterministic fixed-order sum)."""
    _check_cuda("cube", cube, torch.float32)
    _check_cuda("w", w, torch.float32)
    L = cube.shape[-1]
    rows = cube.reshape(-1, L)
    if rows.stride(1) != 1:
        rows = rows.contiguous()
    wr = w.reshape(-1, L)
    if wr.shape != rows.shape:
        raise ValueError("lsf_dot: w must have the cube's shape")
    if wr.stride(1) != 1:
        wr = wr.contiguous()
    t = _contig("taps", taps, torch.float32).reshape(-1)
    out = torch.empty((), dtype=torch.float64, device=cube.device)
    ws = workspace(_lib.query("rubix_fused_dot_workspace_size"), cube.device)
    _lib.call("rubix_lsf_dot_dtaps", _ptr(rows), rows.shape[0], L, rows.stride(0), _ptr(wr),
              wr.stride(0), _ptr(t), t.numel(), int(crop), _ptr(out), _ptr(ws), ws.numel(),
              _stream(cube.device))
    _count(1)
    return out


def inertia_tensor(coords: torch.Tensor, mass: torch.Tensor, halfmass_radius: float) -> torch.Tensor:
    """[3, 3] float64 moment-of-inertia tensor of the particles within the radius, with
    rubix's index padding (particle 0 once more per particle outside)."""
    coords = _contig("coords", coords, torch.float32)
    mass = _contig("mass", mass, torch.float32).reshape(-1)
    c = coords.reshape(-1, coords.shape[-1])
    out = torch.empty((3, 3), dtype=torch.float64, device=c.device)
    ws = workspace(_lib.query("rubix_inertia_workspace_size"), c.device)
    _lib.call("rubix_inertia_tensor", _ptr(c), c.shape[0], c.stride(0), _ptr(mass),
              float(halfmass_radius), _ptr(out), _ptr(ws), ws.numel(), _stream(c.device))
    _count(2)
    return out


def rotate_vectors(x: torch.Tensor, matrix, out=None) -> torch.Tensor:
    """x [..., 3] times the 3x3 float64 matrix (row vectors), float32 result."""
    x = _contig("x", x, torch.float32)
    m = np.ascontiguousarray(np.asarray(matrix, dtype=np.float64).reshape(3, 3))
    rows = x.reshape(-1, 3)
    if out is None:
        out = torch.empty_like(rows)
    o = out.reshape(-1, 3)
    _lib.call("rubix_rotate_vectors", _ptr(rows), _ptr(o), rows.shape[0], rows.stride(0),
              o.stride(0), m.ctypes.data, _stream(x.device))
    _count(1 if rows.shape[0] > 0 else 0)
    return out.reshape(x.shape)


def orient_filter_assign(coords, velocity, matrix, edges, fields=(), mask=True,
                         out_coords=None, out_velocity=None):
    """rotate_galaxy + filter_particles + spaxel_assignment in one launch.

    coords, velocity: [n, 3] float32 (velocity used only with ``matrix``); matrix: 3x3
    (host) or None; fields: float32 tensors with n rows, copied with the particles
    outside the aperture set to 0.  Returns (coords_out, velocity_out, fields_out, mask
    uint8 or None, idx int32); without ``matrix`` coords_out / velocity_out are None."""
    import ctypes

    coords = _contig("coords", coords, torch.float32)
    n = coords.shape[0]
    if coords.dim() != 2 or coords.shape[1] != 3:
        raise ValueError(f"coords must be (n, 3), got {tuple(coords.shape)}")
    edges = _contig("edges", edges, torch.float32)
    dev = coords.device
    m = None
    if matrix is not None:
        m = np.ascontiguousarray(np.asarray(matrix, dtype=np.float64).reshape(3, 3))
        velocity = _contig("velocity", velocity, torch.float32)
        if tuple(velocity.shape) != (n, 3):
            raise ValueError("velocity must be (n, 3) like coords")
        out_coords = torch.empty_like(coords) if out_coords is None else out_coords
        out_velocity = torch.empty_like(velocity) if out_velocity is None else out_velocity
    fields = [_contig("field", f, torch.float32) for f in fields]
    if len(fields) > 8:
        raise ValueError("at most 8 fields per launch")
    widths = []
    for f in fields:
        w = f.numel() // max(n, 1) if n else 1
        if n and f.numel() != n * w:
            raise ValueError("every field needs one row per particle")
        widths.append(max(w, 1))
    outs = [torch.empty_like(f) for f in fields]
    mask_t = torch.empty(n, dtype=torch.uint8, device=dev) if (mask or fields) else None
    idx = torch.empty(n, dtype=torch.int32, device=dev)
    k = len(fields)
    fin = (ctypes.c_void_p * max(k, 1))(*[f.data_ptr() for f in fields])
    fout = (ctypes.c_void_p * max(k, 1))(*[o.data_ptr() for o in outs])
    fw = (ctypes.c_int32 * max(k, 1))(*widths)
    _lib.call("rubix_orient_filter_assign", _ptr(coords), _ptr(velocity) if m is not None else None,
              n, None if m is None else m.ctypes.data, _ptr(out_coords) if m is not None else None,
              _ptr(out_velocity) if m is not None else None, _ptr(edges), edges.numel(), k,
              ctypes.addressof(fin), ctypes.addressof(fout), ctypes.addressof(fw),
              _ptr(mask_t) if mask_t is not None else None, _ptr(idx), _stream(dev))
    _count(1 if n > 0 else 0)
    return (out_coords if m is not None else None, out_velocity if m is not None else None,
            outs, mask_t, idx)


def flux_image(cube: torch.Tensor) -> torch.Tensor:
    """[..., L] -> [...] float32: sum over the last axis (the flux image of a cube)."""
    _check_cuda("cube", cube, torch.float32)
    L = cube.shape[-1]
    rows = cube.reshape(-1, L)
    if rows.stride(-1) != 1:
        rows = rows.contiguous()
    out = torch.empty(rows.shape[0], dtype=torch.float32, device=cube.device)
    _lib.call("rubix_flux_image", _ptr(rows), rows.shape[0], L, rows.stride(0), _ptr(out),
              _stream(cube.device))
    _count(1 if rows.shape[0] > 0 else 0)
    return out.view(cube.shape[:-1])


def noise_median(flux: torch.Tensor) -> torch.Tensor:
    """0-d float32: median of `flux`, or 0 when any value is <= 0 (rubix's
    nan_to_num(jnp.median(where(flux > 0, flux, nan))))."""
    _check_cuda("flux", flux, torch.float32)
    f = flux.contiguous().reshape(-1)
    out = torch.empty((), dtype=torch.float32, device=f.device)
    ws = workspace(_lib.query("rubix_noise_median_workspace_size"), f.device)
    _lib.call("rubix_noise_median", _ptr(f), f.numel(), _ptr(out), _ptr(ws), ws.numel(),
              _stream(f.device))
    # one block-wide select up to 2^20 values; else init, 8 x (histogram, pick), finish
    _count(1 if f.numel() <= (1 << 20) else 2 + 16 * (f.numel() > 0))
    return out


def apply_noise_(cube: torch.Tensor, signal_to_noise: float, distribution: str = "normal",
                 seed: int = 0, flux=None, median=None) -> torch.Tensor:
    """In place: cube += cube * z * sqrt(median) / s2n / sqrt(flux) per spaxel (rubix's
    calculate_noise_cube), z from Philox4x32-10 keyed by `seed`."""
    _check_cuda("cube", cube, torch.float32)
    if not cube.is_contiguous():
        raise ValueError("cube must be contiguous")
    dist = {"normal": 0, "uniform": 1}.get(distribution)
    if dist is None:
        raise ValueError(f"Invalid noise type: {distribution}. Supported types: "
                         "['normal', 'uniform']")
    L = cube.shape[-1]
    rows = cube.view(-1, L)
    flux = flux_image(cube).reshape(-1) if flux is None else flux.reshape(-1)
    median = noise_median(flux) if median is None else median
    _lib.call("rubix_apply_noise", _ptr(rows), rows.shape[0], L, rows.stride(0), _ptr(flux),
              _ptr(median), float(signal_to_noise), dist, int(seed) & (2**64 - 1),
              _stream(cube.device))
    _count(1 if rows.numel() > 0 else 0)
    return cube


def philox4x32_10(counter, key) -> list:
    """One Philox4x32-10 block computed by the library on the host (no GPU needed)."""
    import ctypes

    c = (ctypes.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in counter])
    k = (ctypes.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (ctypes.c_uint32 * 4)()
    _lib.call("rubix_philox4x32_10", ctypes.addressof(c), ctypes.addressof(k),
              ctypes.addressof(o))
    return [int(x) for x in o]


def _host_taps(t) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(t, dtype=np.float32).reshape(-1))
    return a


def _is_device_taps(t) -> bool:
    return isinstance(t, torch.Tensor) and t.is_cuda


def psf_forward(cube: torch.Tensor, taps_y, taps_x=None, out=None) -> torch.Tensor:
    """Separable 'same' convolution of every wavelength plane of cube [ny, nx, L].  Taps
    on the host (array-like) or, both, as float32 CUDA tensors (no host copy)."""
    _check_cuda("cube", cube, torch.float32)
    if cube.dim() != 3 or cube.stride(2) != 1 or cube.stride(0) != cube.shape[1] * cube.stride(1):
        cube = cube.contiguous()
    ny, nx, L = cube.shape
    if out is None:
        out = torch.empty((ny, nx, L), dtype=torch.float32, device=cube.device)
    if _is_device_taps(taps_y):
        ty = _contig("taps_y", taps_y, torch.float32).reshape(-1)
        tx = ty if taps_x is None else _contig("taps_x", taps_x, torch.float32).reshape(-1)
        _lib.call("rubix_psf_fwd_dtaps", _ptr(cube), _ptr(out), ny, nx, L, cube.stride(1),
                  out.stride(1), _ptr(ty), ty.numel(), _ptr(tx), tx.numel(),
                  _stream(cube.device))
        _count(1 if cube.numel() > 0 else 0)
        return out
    ty = _host_taps(taps_y)
    tx = ty if taps_x is None else _host_taps(taps_x)
    _lib.call("rubix_psf_fwd", _ptr(cube), _ptr(out), ny, nx, L, cube.stride(1), out.stride(1),
              ty.ctypes.data, ty.size, tx.ctypes.data, tx.size, _stream(cube.device))
    _count(1 if cube.numel() > 0 else 0)
    return out


def psf_status(device=None) -> int:
    """Device error word of the TMA-staged PSF: 1 if a staged-row wait ran out since the
    last read (reading clears it), else 0.  Synchronises the current stream."""
    import ctypes

    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    v = ctypes.c_int(0)
    _lib.lib().rubix_psf_status(ctypes.byref(v), _stream(dev))
    return int(v.value)


def lsf_forward(cube: torch.Tensor, taps, crop: int, out=None) -> torch.Tensor:
    """Full 1-D convolution along the last axis cropped to [crop, L + crop)."""
    _check_cuda("cube", cube, torch.float32)
    if cube.stride(-1) != 1:
        cube = cube.contiguous()
    L = cube.shape[-1]
    rows = cube.reshape(-1, L) if cube.is_contiguous() else cube.contiguous().reshape(-1, L)
    if out is None:
        out = torch.empty(cube.shape, dtype=torch.float32, device=cube.device)
    orow = out.view(-1, L)
    if _is_device_taps(taps):
        k = _contig("taps", taps, torch.float32).reshape(-1)
        _lib.call("rubix_lsf_fwd_dtaps", _ptr(rows), _ptr(orow), rows.shape[0], L,
                  rows.stride(0), orow.stride(0), _ptr(k), k.numel(), int(crop),
                  _stream(cube.device))
        _count(1 if cube.numel() > 0 else 0)
        return out
    k = _host_taps(taps)
    _lib.call("rubix_lsf_fwd", _ptr(rows), _ptr(orow), rows.shape[0], L, rows.stride(0),
              orow.stride(0), k.ctypes.data, k.size, int(crop), _stream(cube.device))
    _count(1 if cube.numel() > 0 else 0)
    return out


# ------------------------------------------------------------------ materialised steps
def ssp_lookup(ssp_flux, ssp_metallicity, ssp_age, metallicity, age, mass=None):
    """[n, n_wave] bilinear SSP lookup (times mass when given)."""
    ssp_flux = _contig("ssp_flux", ssp_flux, torch.float32)
    nz, na, nw = ssp_flux.shape
    zg = _contig("ssp_metallicity", ssp_metallicity, torch.float32)
    ag = _contig("ssp_age", ssp_age, torch.float32)
    metallicity = _contig("metallicity", metallicity, torch.float32).reshape(-1)
    age = _contig("age", age, torch.float32).reshape(-1)
    if mass is not None:
        mass = _contig("mass", mass, torch.float32).reshape(-1)
    n = metallicity.numel()
    out = torch.empty((n, nw), dtype=torch.float32, device=metallicity.device)
    _lib.call("rubix_ssp_lookup", _ptr(ssp_flux), _ptr(zg), _ptr(ag), nz, na, nw,
              _ptr(metallicity), _ptr(age), _ptr(mass), n, _ptr(out), nw,
              _stream(metallicity.device))
    _count(1 if n > 0 else 0)
    return out


def scale_rows(rows, mass):
    """rows[i, :] * mass[i]."""
    rows = _contig("rows", rows, torch.float32)
    mass = _contig("mass", mass, torch.float32).reshape(-1)
    n, nw = rows.shape
    out = torch.empty_like(rows)
    _lib.call("rubix_scale_rows", _ptr(rows), nw, _ptr(mass), n, nw, _ptr(out), nw,
              _stream(rows.device))
    _count(1 if rows.numel() > 0 else 0)
    return out


def resample_rows(spectra, ssp_wave_z, velocity, vel_component, wave_t):
    """resample_spectrum of each row on its Doppler-shifted grid -> [n, L]."""
    spectra = _contig("spectra", spectra, torch.float32)
    wz = _contig("ssp_wave_z", ssp_wave_z, torch.float32)
    velocity = _contig("velocity", velocity, torch.float32)
    wave_t = _contig("wave_t", wave_t, torch.float32)
    n, nw = spectra.shape
    L = wave_t.numel()
    vstride = velocity.shape[1] if velocity.dim() == 2 else 1
    out = torch.empty((n, L), dtype=torch.float32, device=spectra.device)
    _lib.call("rubix_resample_rows", _ptr(spectra), nw, _ptr(wz), nw, _ptr(velocity), vstride,
              int(vel_component), n, _ptr(wave_t), L, _ptr(out), L, _stream(spectra.device))
    _count(1 if n > 0 else 0)
    return out


def segment_sum_rows(rows, perm, seg_offsets, n_segments):
    """Per-spaxel ordered sum of given rows -> [n_segments, L]."""
    rows = _contig("rows", rows, torch.float32)
    perm = _contig("perm", perm, torch.int32)
    seg_offsets = _contig("seg_offsets", seg_offsets, torch.int32)
    L = rows.shape[1]
    out = torch.empty((int(n_segments), L), dtype=torch.float32, device=rows.device)
    _lib.call("rubix_segment_sum_rows", _ptr(rows), L, L, _ptr(perm), _ptr(seg_offsets),
              int(n_segments), _ptr(out), L, _stream(rows.device))
    _count(1 if n_segments > 0 else 0)
    return out


def mask_zero_(values, mask):
    """In place: values[i, ...] = 0 where mask[i] == 0 (float32, contiguous rows)."""
    _check_cuda("values", values, torch.float32)
    if not values.is_contiguous():
        raise ValueError("values must be contiguous")
    mask = _contig("mask", mask, torch.uint8).reshape(-1)
    n = mask.numel()
    width = values.numel() // max(n, 1) if n else 0
    if n and values.numel() != n * width:
        raise ValueError("values must have one row per mask entry")
    _lib.call("rubix_mask_zero", _ptr(values), n, width, width, _ptr(mask), _stream(values.device))
    _count(1 if values.numel() > 0 else 0)
    return values


def dust_gas_extinction(mass, metals, dgr_params, broken: bool, scale: float,
                        spaxel_area: float, h_col: int = 0, o_col: int = 4) -> torch.Tensor:
    """Per-cell extinction of the gas [n] float32: mass * dust-to-gas ratio of
    12 + log10(O/(16 H)) * scale / spaxel_area (``rubix_dust_gas_extinction``)."""
    mass = _contig("mass", mass, torch.float32).reshape(-1)
    metals = _contig("metals", metals, torch.float32)
    n = mass.numel()
    rows = metals.reshape(n, -1) if n > 0 else metals.reshape(0, max(h_col, o_col) + 1)
    prm = np.ascontiguousarray(np.asarray(dgr_params, dtype=np.float32).reshape(6))
    out = torch.empty(n, dtype=torch.float32, device=mass.device)
    _lib.call("rubix_dust_gas_extinction", _ptr(mass), _ptr(rows), rows.shape[1], int(h_col),
              int(o_col), n, prm.ctypes.data, 1 if broken else 0, float(scale),
              float(spaxel_area), _ptr(out), _stream(mass.device))
    _count(1 if n > 0 else 0)
    return out


def dust_av(gas_coords, gas_pa, gas_ext, star_coords, star_pa, n_segments: int,
            pa_limit: int) -> torch.Tensor:
    """A_V [n_stars] float32 of every star (``rubix_dust_av``): rubix's interpolated
    cumulative dust column of the star's spaxel at the star's z."""
    star_coords = _contig("star_coords", star_coords, torch.float32).reshape(-1, 3)
    star_pa = _contig("star_pa", star_pa, torch.int32).reshape(-1)
    gas_coords = _contig("gas_coords", gas_coords, torch.float32).reshape(-1, 3)
    gas_pa = _contig("gas_pa", gas_pa, torch.int32).reshape(-1)
    gas_ext = _contig("gas_ext", gas_ext, torch.float32).reshape(-1)
    ns, ng = star_coords.shape[0], gas_coords.shape[0]
    if star_pa.numel() != ns or gas_pa.numel() != ng or gas_ext.numel() != ng:
        raise ValueError("per-star / per-cell arrays must match the coordinates")
    dev = star_coords.device
    out = torch.empty(ns, dtype=torch.float32, device=dev)
    ws = workspace(_lib.query("rubix_dust_av_workspace_size", ng, int(n_segments)), dev)
    _lib.call("rubix_dust_av", _ptr(gas_coords), 3, _ptr(gas_pa), _ptr(gas_ext), ng,
              _ptr(star_coords), 3, _ptr(star_pa), ns, int(n_segments), int(pa_limit),
              _ptr(out), _ptr(ws), ws.numel(), _stream(dev))
    if ns > 0:
        k = 1  # star pass
        if ng > 0:
            # z sort, assignment sort, G sort (4 + P + 4 radix passes of 3 launches each)
            # plus the key, offset, cumulative-sum, node, run and scan passes
            k += 36 + 3 * _key_passes(int(pa_limit) - 1)
            if pa_limit > n_segments:
                k += 14 + 3 * _key_passes(int(n_segments) - 1)
        _count(k)
    return out


def dust_av_backward(gas_coords, gas_pa, gas_ext, star_coords, star_pa, n_segments: int,
                     pa_limit: int, grad_av):
    """Adjoint of ``dust_av`` (``rubix_dust_av_bwd``): from dL/dA_V of every star, the
    stars' dL/dz [n_stars] and the cells' dL/d ext [n_gas] (gas heights held fixed)."""
    star_coords = _contig("star_coords", star_coords, torch.float32).reshape(-1, 3)
    star_pa = _contig("star_pa", star_pa, torch.int32).reshape(-1)
    gas_coords = _contig("gas_coords", gas_coords, torch.float32).reshape(-1, 3)
    gas_pa = _contig("gas_pa", gas_pa, torch.int32).reshape(-1)
    gas_ext = _contig("gas_ext", gas_ext, torch.float32).reshape(-1)
    grad_av = _contig("grad_av", grad_av, torch.float32).reshape(-1)
    ns, ng = star_coords.shape[0], gas_coords.shape[0]
    if star_pa.numel() != ns or grad_av.numel() != ns or gas_pa.numel() != ng \
            or gas_ext.numel() != ng:
        raise ValueError("per-star / per-cell arrays must match the coordinates")
    dev = star_coords.device
    gz = torch.empty(ns, dtype=torch.float32, device=dev)
    gext = torch.empty(ng, dtype=torch.float32, device=dev)
    ws = workspace(_lib.query("rubix_dust_av_bwd_workspace_size", ng, int(n_segments), ns),
                   dev)
    _lib.call("rubix_dust_av_bwd", _ptr(gas_coords), 3, _ptr(gas_pa), _ptr(gas_ext), ng,
              _ptr(star_coords), 3, _ptr(star_pa), ns, int(n_segments), int(pa_limit),
              _ptr(grad_av), _ptr(gz), _ptr(gext), _ptr(ws), ws.numel(), _stream(dev))
    if ns > 0:
        k = 1
        if ng > 0:
            # the forward's setup passes, then the record sort and three reduction passes
            k += 36 + 3 * _key_passes(int(pa_limit) - 1) + 3 + 3 * _key_passes(ng)
            if pa_limit > n_segments:
                k += 14 + 3 * _key_passes(int(n_segments) - 1)
        _count(k)
    return gz, gext


def dust_gas_extinction_backward(mass, metals, dgr_params, broken: bool, scale: float,
                                 spaxel_area: float, grad_ext, h_col: int = 0,
                                 o_col: int = 4):
    """Adjoint of ``dust_gas_extinction``: (dL/d mass [n], dL/d metals [n, columns], the
    latter non-zero in the hydrogen and oxygen columns only)."""
    mass = _contig("mass", mass, torch.float32).reshape(-1)
    metals = _contig("metals", metals, torch.float32)
    grad_ext = _contig("grad_ext", grad_ext, torch.float32).reshape(-1)
    n = mass.numel()
    rows = metals.reshape(n, -1) if n > 0 else metals.reshape(0, max(h_col, o_col) + 1)
    prm = np.ascontiguousarray(np.asarray(dgr_params, dtype=np.float32).reshape(6))
    dev = mass.device
    gm = torch.empty(n, dtype=torch.float32, device=dev)
    gh = torch.empty(n, dtype=torch.float32, device=dev)
    go = torch.empty(n, dtype=torch.float32, device=dev)
    _lib.call("rubix_dust_gas_extinction_bwd", _ptr(mass), _ptr(rows), rows.shape[1],
              int(h_col), int(o_col), n, prm.ctypes.data, 1 if broken else 0, float(scale),
              float(spaxel_area), _ptr(grad_ext), _ptr(gm), _ptr(gh), _ptr(go), _stream(dev))
    _count(1 if n > 0 else 0)
    gmet = torch.zeros_like(rows)
    gmet[:, h_col] = gh
    gmet[:, o_col] = go
    return gm, gmet.view_as(metals)


def dust_apply_rows_(rows: torch.Tensor, av, exponent) -> torch.Tensor:
    """In place: rows [n, L] *= 2^(exponent[t] * av[i]) (``rubix_dust_apply_rows``)."""
    _check_cuda("rows", rows, torch.float32)
    if rows.dim() != 2 or rows.stride(1) != 1:
        raise ValueError("rows must be [n, L] with unit stride along wavelength")
    av = _contig("av", av, torch.float32).reshape(-1)
    exponent = _contig("exponent", exponent, torch.float32).reshape(-1)
    n, L = rows.shape
    if av.numel() != n or exponent.numel() != L:
        raise ValueError("av must be [n] and exponent [L]")
    _lib.call("rubix_dust_apply_rows", _ptr(rows), n, L, rows.stride(0), _ptr(av),
              _ptr(exponent), _stream(rows.device))
    _count(1 if n * L > 0 else 0)
    return rows


def fits_cube_layout(cube: torch.Tensor, out=None) -> torch.Tensor:
    """cube [A, B, L] float32 -> int32 [L, B, A] holding big-endian float32 bit patterns
    (the bytes of ``cube.T`` in a FITS file), ``rubix_fits_cube_layout``."""
    _check_cuda("cube", cube, torch.float32)
    if cube.dim() != 3 or cube.stride(2) != 1 or cube.stride(0) != cube.shape[1] * cube.stride(1):
        cube = cube.contiguous()
    A, B, L = (int(x) for x in cube.shape)
    if out is None:
        out = torch.empty((L, B, A), dtype=torch.int32, device=cube.device)
    _lib.call("rubix_fits_cube_layout", _ptr(cube), A, B, L, cube.stride(1), _ptr(out),
              _stream(cube.device))
    _count(1 if A * B * L > 0 else 0)
    return out


def gauss_taps(sigma: torch.Tensor, x, reversed_pad: bool = False):
    """(taps, dtaps/dsigma, reversed taps) float32 CUDA tensors of the normalised Gaussian
    at positions ``x`` (host array) for a sigma held on the device (0-d tensor): no
    synchronisation (``rubix_gauss_taps``).  The reversed taps get a trailing zero when
    ``reversed_pad``."""
    _check_cuda("sigma", sigma, None)
    sg = sigma.detach().to(torch.float64).reshape(1).contiguous()
    xs = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1))
    m = xs.size
    dev = sg.device
    taps = torch.empty(m, dtype=torch.float32, device=dev)
    dtaps = torch.empty(m, dtype=torch.float32, device=dev)
    rtaps = torch.empty(m + (1 if reversed_pad else 0), dtype=torch.float32, device=dev)
    _lib.call("rubix_gauss_taps", _ptr(sg), xs.ctypes.data, m, _ptr(taps), _ptr(dtaps),
              _ptr(rtaps), 1 if reversed_pad else 0, _stream(dev))
    _count(1)
    return taps, dtaps, rtaps


def _key_passes(max_key: int) -> int:
    return (max(int(max_key), 0).bit_length() + 7) // 8
