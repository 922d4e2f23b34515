"""NumPy restatement of rubix's particle -> IFU datacube path, float64 arithmetic.

TEST INFRASTRUCTURE ONLY.  The product package never imports this module; tests,
``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use it as the checker and
as the timed CPU baseline.

Every function cites the rubix source it restates (``path:line`` relative to the rubix
project root).  The reference is JAX code computing in float32; this module keeps the
reference's discrete decisions on the float32 values the reference materialises and
does the arithmetic in float64:

* spatial bin edges, digitize, aperture mask: float32 inputs, exact comparisons;
* the SSP wavelength after the cosmological shift is the float32 product
  ``fl32(fl32(1+z) * lambda_ssp)`` (spectra/ifu.py:66-80, core/ifu.py:261);
* the Doppler-shifted grid is the float32 grid ``fl32(lambda_z * fl32(exp(v/c)))``
  (spectra/ifu.py:190).  The in-range mask and the interpolation brackets of the
  resampling (spectra/ifu.py:241-251) are taken on that float32 grid; interpolation
  weights, sums and the flux-conservation ratio are computed in float64.

Parity status.  The reference cannot be imported here (JAX, interpax and friends are
absent), so the restatement is pinned by the reference's own known-answer tests for
this path (tests/test_spectra_ifu.py, tests/test_telescope_utils.py,
tests/test_telescope_psf.py, tests/test_telescope_psf_kernels.py,
tests/test_telescope_lsf.py, tests/test_core_ifu.py), restated in
``tests/test_oracle_known_answers.py``.  The SSP lookup calls the third-party
``interpax.interp2d`` (unpinned in rubix's pyproject.toml, not vendored); its
``method="linear"`` branch is restated here from interpax's published algorithm and
is not covered by any reference test (the reference tests use ``method="cubic"`` on a
template file that is not shipped).
"""

from __future__ import annotations

import math

import numpy as np

SPEED_OF_LIGHT = 299792.458  # km/s, rubix/config/rubix_config.yml:8
FLT_MAX = float(np.finfo(np.float32).max)
VELOCITY_AXIS = {"x": 0, "y": 1, "z": 2}  # spectra/ifu.py:106-142

__all__ = [
    "SPEED_OF_LIGHT",
    "calculate_spatial_bin_edges",
    "calculate_wave_seq",
    "square_spaxel_assignment",
    "mask_particles_outside_aperture",
    "filter_particles",
    "interp2d_linear",
    "cosmological_doppler_shift",
    "doppler_factor32",
    "velocity_doppler_shift32",
    "calculate_diff",
    "resample_spectrum",
    "resample_spectra",
    "calculate_cube",
    "gaussian_kernel_2d",
    "apply_psf",
    "lsf_kernel",
    "apply_lsf",
    "particle_spectra",
    "render_cube",
    "angular_scale",
]


# ----------------------------------------------------------------------------------
# Telescope grids
# ----------------------------------------------------------------------------------
def calculate_wave_seq(wave_range, wave_res):
    """telescope/utils.py:42-53 (``jnp.arange`` over Python floats -> float32)."""
    return np.arange(wave_range[0], wave_range[1], wave_res, dtype=np.float32)


def calculate_spatial_bin_edges(fov, spatial_bins, ang_size):
    """telescope/utils.py:12-37 with ``cosmology.angular_scale(dist_z)`` = ``ang_size``.

    With the real cosmology ``ang_size`` is a float32 JAX scalar, so the aperture and
    bin size are float32; a plain Python float (the reference's own test mocks the
    cosmology with one, tests/test_telescope_utils.py:88-89) keeps them in float64.
    ``jnp.arange`` materialises float32 values either way, and the float ``arange``
    can yield ``spatial_bins + 1`` or ``spatial_bins + 2`` edges.
    """
    if isinstance(ang_size, float) and not isinstance(ang_size, np.floating):
        aperture = ang_size * fov
        bin_size = aperture / float(spatial_bins)
        start, stop = -aperture / 2, aperture / 2 + bin_size
    else:
        aperture = np.float32(np.float32(ang_size) * np.float32(fov))
        bin_size = np.float32(aperture / np.float32(spatial_bins))
        start = np.float32(-aperture / np.float32(2))
        stop = np.float32(aperture / np.float32(2) + bin_size)
    edges = np.arange(start, stop, bin_size, dtype=np.float32)
    return edges, bin_size


def angular_scale(z, Om0=0.3075, w0=-1.0, wa=0.0, h=0.6774):
    """cosmology/base.py:290-314 (kpc/arcsec), flat wCDM, trapezoid on 256 nodes.

    Defaults are PLANCK15 (cosmology/__init__.py:3).  Computed in float64 and
    rounded to float32 once.
    """
    ztab = np.linspace(0.0, z, 256)
    a = 1.0 / (1.0 + ztab)
    rho_de = a ** (-3.0 * (1.0 + w0 + wa)) * np.exp(-3.0 * wa * (1.0 - a))
    ez = np.sqrt(Om0 * (1.0 + ztab) ** 3 + (1.0 - Om0) * rho_de)
    integ = np.sum(np.diff(ztab) * (1.0 / ez[1:] + 1.0 / ez[:-1]) / 2.0)
    d_c = integ * 2.99792458e8 * 1e-5 / h  # Mpc (cosmology/base.py:137)
    d_a = d_c / (1.0 + z)
    return np.float32(d_a * (np.pi / (180 * 60 * 60)) * 1e3)


# ----------------------------------------------------------------------------------
# Spaxel assignment and aperture filter
# ----------------------------------------------------------------------------------
def _digitize(x, edges):
    """``jnp.digitize(x, edges)`` (right=False) for ascending edges = count of edges <= x.

    NaN sorts last in JAX's searchsorted comparator, giving ``len(edges)``.
    """
    x = np.asarray(x, dtype=np.float32)
    out = np.searchsorted(edges, x, side="right").astype(np.int64)
    return out


def square_spaxel_assignment(coords, edges):
    """telescope/utils.py:138-152: ``ix + nb*iy`` with ``nb = len(edges)-1``, int32."""
    coords = np.asarray(coords, dtype=np.float32)
    edges = np.asarray(edges, dtype=np.float32)
    nb = len(edges) - 1
    ix = np.clip(_digitize(coords[:, 0], edges) - 1, 0, nb - 1)
    iy = np.clip(_digitize(coords[:, 1], edges) - 1, 0, nb - 1)
    return (ix + nb * iy).astype(np.int32)


def mask_particles_outside_aperture(coords, edges):
    """telescope/utils.py:170-178: inclusive box ``[min(edges), max(edges)]^2`` in x, y."""
    coords = np.asarray(coords, dtype=np.float32)
    lo = np.float32(np.min(edges))
    hi = np.float32(np.max(edges))
    m = (coords[:, 0] >= lo) & (coords[:, 0] <= hi)
    m &= (coords[:, 1] >= lo) & (coords[:, 1] <= hi)
    return m


def filter_particles(coords, edges, **arrays):
    """core/telescope.py:151-175: zero every non-coordinate/velocity array outside."""
    mask = mask_particles_outside_aperture(coords, edges)
    out = {}
    for k, v in arrays.items():
        v = np.asarray(v)
        m = mask.reshape(mask.shape + (1,) * (v.ndim - 1))
        out[k] = np.where(m, v, np.zeros((), dtype=v.dtype))
    return mask, out


# ----------------------------------------------------------------------------------
# SSP lookup: interpax.interp2d(method="linear", extrap=0), spectra/ssp/grid.py:113-120
# ----------------------------------------------------------------------------------
def interp2d_linear(xq, yq, x, y, f, query_dtype=np.float32):
    """Bilinear interpolation of ``f[x, y, :]`` at ``(xq, yq)``; 0 outside the box.

    Restates interpax's linear branch: cell ``i = clip(searchsorted(x, xq, 'right'),
    1, nx-1)`` (and likewise ``j``), weights ``tx = (xq-x[i-1])/(x[i]-x[i-1])``,
    ``ty`` likewise, and ``extrap=0`` returning 0 where ``xq < x[0]``, ``xq > x[-1]``,
    ``yq < y[0]`` or ``yq > y[-1]`` (boundaries inclusive).  In rubix ``x`` is the
    metallicity grid and ``y`` the age grid (grid.py:113-120; flux layout [Z, age, lambda]).
    """
    xq = np.asarray(xq, dtype=query_dtype).astype(np.float64)
    yq = np.asarray(yq, dtype=query_dtype).astype(np.float64)
    x = np.asarray(x, dtype=np.float32).astype(np.float64)
    y = np.asarray(y, dtype=np.float32).astype(np.float64)
    f = np.asarray(f, dtype=np.float32).astype(np.float64)
    i = np.clip(np.searchsorted(x, xq, side="right"), 1, len(x) - 1)
    j = np.clip(np.searchsorted(y, yq, side="right"), 1, len(y) - 1)
    dx = x[i] - x[i - 1]
    dy = y[j] - y[j - 1]
    tx = np.where(dx == 0, 0.0, (xq - x[i - 1]) / np.where(dx == 0, 1.0, dx))
    ty = np.where(dy == 0, 0.0, (yq - y[j - 1]) / np.where(dy == 0, 1.0, dy))
    tx = tx[:, None]
    ty = ty[:, None]
    fq = (
        (1 - tx) * (1 - ty) * f[i - 1, j - 1]
        + tx * (1 - ty) * f[i, j - 1]
        + (1 - tx) * ty * f[i - 1, j]
        + tx * ty * f[i, j]
    )
    outside = (xq < x[0]) | (xq > x[-1]) | (yq < y[0]) | (yq > y[-1])
    fq[outside] = 0.0
    return fq


# ----------------------------------------------------------------------------------
# Doppler shift and resampling
# ----------------------------------------------------------------------------------
def cosmological_doppler_shift(z, wavelength):
    """spectra/ifu.py:66-80 applied at core/ifu.py:261, float32 like the reference."""
    return (np.float32(1.0 + z) * np.asarray(wavelength, dtype=np.float32)).astype(np.float32)


def doppler_factor32(v_los):
    """``exp(v/c)`` of spectra/ifu.py:190 rounded once to float32."""
    v = np.asarray(v_los, dtype=np.float32).astype(np.float64)
    return np.exp(v / SPEED_OF_LIGHT).astype(np.float32)


def velocity_doppler_shift32(wave_z, v_los):
    """spectra/ifu.py:168-220: ``lambda_z * exp(v/c)`` per particle, float32 grid."""
    a = doppler_factor32(v_los)
    return (np.asarray(wave_z, dtype=np.float32)[None, :] * a[:, None]).astype(np.float32)


def calculate_diff(vec, pad_with_zero=True):
    """spectra/ifu.py:84-102: ``diff(vec, prepend=vec[0])`` (first entry 0)."""
    vec = np.asarray(vec)
    if pad_with_zero:
        return np.diff(vec, prepend=vec[..., :1], axis=-1)
    return np.diff(vec, axis=-1)


def _nan_to_num32(s):
    """``jnp.nan_to_num(s, nan=0)`` on a float32 result: inf -> +-FLT_MAX."""
    s = np.asarray(s, dtype=np.float64)
    s = np.where(np.isnan(s), 0.0, s)
    s = np.where(np.isposinf(s), FLT_MAX, s)
    s = np.where(np.isneginf(s), -FLT_MAX, s)
    return s


def resample_spectrum(initial_spectrum, initial_wavelength, target_wavelength):
    """spectra/ifu.py:224-266 for one spectrum (float64 arithmetic)."""
    F = np.asarray(initial_spectrum, dtype=np.float64)
    lp = np.asarray(initial_wavelength, dtype=np.float64)
    lt = np.asarray(target_wavelength, dtype=np.float64)
    in_range = (lp >= lt.min()) & (lp <= lt.max())
    total = np.sum(F * calculate_diff(lp) * in_range)
    lum = np.interp(lt, lp, F)
    new_total = np.sum(lum * calculate_diff(lt))
    with np.errstate(divide="ignore", invalid="ignore"):
        s = total / new_total
    return lum * _nan_to_num32(s)


def _interp_rows(lt, lp, F):
    """Row-wise ``jnp.interp(lt, lp[r], F[r])`` (end clamping), brackets exact on ``lp``.

    ``lp`` holds float32 grid values (one increasing row per particle).  The bracket
    is ``i = clip(#{lp <= lt}, 1, n-1)`` (searchsorted side='right'), taken with exact
    comparisons on ``lp`` itself.
    """
    n, nl = lp.shape
    i = np.empty((n, lt.shape[0]), dtype=np.int64)
    for r in range(n):
        i[r] = np.searchsorted(lp[r], lt, side="right")
    ic = np.clip(i, 1, nl - 1)
    x0 = np.take_along_axis(lp, ic - 1, axis=1)
    x1 = np.take_along_axis(lp, ic, axis=1)
    f0 = np.take_along_axis(F, ic - 1, axis=1)
    f1 = np.take_along_axis(F, ic, axis=1)
    dx = x1 - x0
    with np.errstate(divide="ignore", invalid="ignore"):
        val = np.where(dx == 0, f0, f0 + (lt[None, :] - x0) / np.where(dx == 0, 1.0, dx) * (f1 - f0))
    val = np.where(lt[None, :] < lp[:, :1], F[:, :1], val)
    val = np.where(lt[None, :] > lp[:, -1:], F[:, -1:], val)
    return val


def resample_spectra(F, lam_prime32, wave_t):
    """Vectorised spectra/ifu.py:224-266 over rows; returns (resampled, scale)."""
    F = np.asarray(F, dtype=np.float64)
    lp = np.asarray(lam_prime32, dtype=np.float32).astype(np.float64)
    lt = np.asarray(wave_t, dtype=np.float32).astype(np.float64)
    in_range = (lp >= lt.min()) & (lp <= lt.max())
    total = np.sum(F * calculate_diff(lp) * in_range, axis=1)
    lum = _interp_rows(lt, lp, F)
    new_total = np.sum(lum * calculate_diff(lt)[None, :], axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        s = _nan_to_num32(total / new_total)
    return lum * s[:, None], s


def calculate_cube(spectra, spaxel_index, num_spaxels):
    """spectra/ifu.py:270-288: segment sum (ids outside [0, S^2) dropped) -> [y, x, lambda]."""
    spectra = np.asarray(spectra, dtype=np.float64)
    idx = np.asarray(spaxel_index).astype(np.int64)
    nseg = int(num_spaxels) ** 2
    cube = np.zeros((nseg, spectra.shape[-1]), dtype=np.float64)
    keep = (idx >= 0) & (idx < nseg)
    np.add.at(cube, idx[keep], spectra[keep])
    return cube.reshape(num_spaxels, num_spaxels, spectra.shape[-1])


# ----------------------------------------------------------------------------------
# PSF and LSF
# ----------------------------------------------------------------------------------
def gaussian_kernel_2d(m, n, sigma):
    """telescope/psf/kernels.py:5-31 (float64)."""
    x = np.arange(-((m - 1) / 2), ((m - 1) / 2) + 1)
    y = np.arange(-((n - 1) / 2), ((n - 1) / 2) + 1)
    X, Y = np.meshgrid(x, y, indexing="ij")
    v = np.exp(-(X**2 + Y**2) / (2 * sigma**2))
    return v / np.sum(v)


def _fft_conv_same_2d(cube, K):
    """``convolve2d(plane, K, mode='same')`` for every plane ``cube[:, :, l]``."""
    S0, S1 = cube.shape[:2]
    m, n = K.shape
    P0, P1 = S0 + m - 1, S1 + n - 1
    F0 = np.fft.rfft2(cube, s=(P0, P1), axes=(0, 1))
    Fk = np.fft.rfft2(K, s=(P0, P1))
    full = np.fft.irfft2(F0 * Fk[:, :, None], s=(P0, P1), axes=(0, 1))
    o0 = (m - 1) // 2
    o1 = (n - 1) // 2
    return full[o0 : o0 + S0, o1 : o1 + S1, :]


def apply_psf(datacube, psf_kernel, method="auto"):
    """telescope/psf/psf.py:33-58: per-plane ``convolve2d(..., mode='same')``.

    'same' keeps rows ``(m-1)//2 .. (m-1)//2 + S - 1`` of the full convolution
    (scipy's centring; identical for the odd kernel sizes of every configuration).
    """
    cube = np.asarray(datacube, dtype=np.float64)
    K = np.asarray(psf_kernel, dtype=np.float64)
    if method == "direct" or (method == "auto" and cube.size * K.size < 5e7):
        S0, S1, L = cube.shape
        m, n = K.shape
        o0, o1 = (m - 1) // 2, (n - 1) // 2
        out = np.zeros_like(cube)
        for i in range(m):
            for j in range(n):
                # out[y, x] += K[i, j] * in[y + o0 - i, x + o1 - j]
                dy, dx = o0 - i, o1 - j
                y0, y1 = max(0, -dy), min(S0, S0 - dy)
                x0, x1 = max(0, -dx), min(S1, S1 - dx)
                if y1 > y0 and x1 > x0:
                    out[y0:y1, x0:x1, :] += K[i, j] * cube[y0 + dy:y1 + dy, x0 + dx:x1 + dx, :]
        return out
    return _fft_conv_same_2d(cube, K)


def lsf_kernel(sigma, wave_res, factor=12):
    """telescope/lsf/lsf.py:12-26: taps at float32 ``arange(-f*d, f*d+d, d)``, normalised."""
    x = np.arange(-factor * wave_res, factor * wave_res + wave_res, wave_res, dtype=np.float32)
    x = x.astype(np.float64)
    g = np.exp(-0.5 * x**2 / sigma**2)
    return g / np.sum(g)


def apply_lsf(datacube, lsf_sigma, wave_resolution, extend_factor=12):
    """telescope/lsf/lsf.py:29-105: full 1-D convolution along lambda, crop ``[f : L+K-1-f]``."""
    cube = np.asarray(datacube, dtype=np.float64)
    g = lsf_kernel(lsf_sigma, wave_resolution, extend_factor)
    K = g.shape[0]
    L = cube.shape[-1]
    end = L + K - 1 - extend_factor
    if end - extend_factor != L:
        raise ValueError(
            f"LSF kernel of {K} taps with extend_factor {extend_factor} does not preserve "
            f"the spectral length {L}"
        )
    flat = cube.reshape(-1, L)
    out = np.zeros_like(flat)
    # out[t] = full[t + f] = sum_j g[j] * in[t + f - j]
    for j in range(K):
        d = extend_factor - j
        lo, hi = max(0, -d), min(L, L - d)
        if hi > lo:
            out[:, lo:hi] += g[j] * flat[:, lo + d : hi + d]
    return out.reshape(cube.shape)


# ----------------------------------------------------------------------------------
# Whole path
# ----------------------------------------------------------------------------------
def particle_spectra(mass, metallicity, age, v_los, ssp_metallicity, ssp_age, ssp_flux,
                     wave_z, wave_t):
    """Steps calculate_spectra -> scale_spectrum_by_mass -> doppler_shift_and_resampling
    (core/ifu.py:63-121, :149-157, :269-293) for a block of particles.

    Returns the (n, L) float64 resampled, mass-scaled spectra.
    """
    G = interp2d_linear(metallicity, age, ssp_metallicity, ssp_age, ssp_flux)
    F = G * np.asarray(mass, dtype=np.float32).astype(np.float64)[:, None]
    lp = velocity_doppler_shift32(wave_z, v_los)
    out, _ = resample_spectra(F, lp, wave_t)
    return out


def render_cube(coords, velocity, mass, metallicity, age, edges, sbin,
                ssp_metallicity, ssp_age, ssp_flux, ssp_wave, dist_z, wave_t,
                psf_size=None, psf_sigma=None, lsf_sigma=None, wave_res=None,
                apply_filter=True, velocity_direction="z", chunk=512, rotation=None,
                transmission=None):
    """The calc_ifu chain (rubix/config/pipeline_config.yml:1-60) from rotate_galaxy
    (when ``rotation`` = (halfmass_radius, alpha, beta, gamma) is given) or
    filter_particles through convolve_lsf, noise excluded.  Returns a dict of stages.

    ``transmission`` ((n, L) array or a function of the (rotated, unfiltered)
    coordinates returning one) multiplies the resampled spectra before the per-spaxel
    sum: calculate_extinction of calc_dusty_ifu (pipeline_config.yml:62-136)."""
    coords = np.asarray(coords, dtype=np.float32)
    velocity = np.asarray(velocity, dtype=np.float32)
    mass = np.asarray(mass, dtype=np.float32)
    if rotation is not None:
        coords, velocity = rotate_galaxy(coords, velocity, mass, *rotation)
    metallicity = np.asarray(metallicity, dtype=np.float32)
    age = np.asarray(age, dtype=np.float32)
    edges = np.asarray(edges, dtype=np.float32)
    wave_t = np.asarray(wave_t, dtype=np.float32)
    out = {}
    if apply_filter:
        mask, arrs = filter_particles(coords, edges, mass=mass, metallicity=metallicity, age=age)
        mass, metallicity, age = arrs["mass"], arrs["metallicity"], arrs["age"]
        out["mask"] = mask
    idx = square_spaxel_assignment(coords, edges)
    out["pixel_assignment"] = idx
    if callable(transmission):
        transmission = transmission(coords)
    wave_z = cosmological_doppler_shift(dist_z, ssp_wave)
    v_los = velocity[:, VELOCITY_AXIS[velocity_direction]]
    nseg = int(sbin) ** 2
    cube = np.zeros((nseg, wave_t.shape[0]), dtype=np.float64)
    n = coords.shape[0]
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        sp = particle_spectra(mass[s:e], metallicity[s:e], age[s:e], v_los[s:e],
                              ssp_metallicity, ssp_age, ssp_flux, wave_z, wave_t)
        if transmission is not None:
            sp = sp * np.asarray(transmission[s:e], dtype=np.float64)
        ii = idx[s:e].astype(np.int64)
        keep = (ii >= 0) & (ii < nseg)
        np.add.at(cube, ii[keep], sp[keep])
    cube = cube.reshape(int(sbin), int(sbin), wave_t.shape[0])
    out["cube"] = cube
    if psf_size is not None:
        K = gaussian_kernel_2d(psf_size, psf_size, psf_sigma)
        cube = apply_psf(cube, K)
        out["cube_psf"] = cube
    if lsf_sigma is not None:
        cube = apply_lsf(cube, lsf_sigma, wave_res)
        out["cube_lsf"] = cube
    out["final"] = cube
    return out


def cube_rel_error(test, ref, rel_floor=1e-3):
    """Normwise and elementwise relative errors of a cube against the oracle.

    Returns ``(max|test-ref|/max|ref|, max elementwise rel over |ref| > rel_floor*max|ref|)``.
    """
    test = np.asarray(test, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = float(np.max(np.abs(ref))) if ref.size else 0.0
    if scale == 0.0:
        e = float(np.max(np.abs(test))) if test.size else 0.0
        return e, e
    err = np.abs(test - ref)
    norm = float(np.max(err)) / scale
    sig = np.abs(ref) > rel_floor * scale
    elem = float(np.max(err[sig] / np.abs(ref[sig]))) if np.any(sig) else 0.0
    return norm, elem


__all__ += ["cube_rel_error"]


# ----------------------------------------------------------------------------------
# Gradients (rubix differentiates the same chain with jax.grad,
# RubixPipeline.gradient, core/pipeline.py:204-208)
# ----------------------------------------------------------------------------------
def interp2d_linear_grad(xq, yq, x, y, f, query_dtype=np.float32):
    """``interp2d_linear`` and its derivatives with respect to ``xq`` (metallicity) and
    ``yq`` (age) inside the containing cell; all three are 0 outside the box."""
    xq = np.asarray(xq, dtype=query_dtype).astype(np.float64)
    yq = np.asarray(yq, dtype=query_dtype).astype(np.float64)
    x = np.asarray(x, dtype=np.float32).astype(np.float64)
    y = np.asarray(y, dtype=np.float32).astype(np.float64)
    f = np.asarray(f, dtype=np.float32).astype(np.float64)
    i = np.clip(np.searchsorted(x, xq, side="right"), 1, len(x) - 1)
    j = np.clip(np.searchsorted(y, yq, side="right"), 1, len(y) - 1)
    dx = x[i] - x[i - 1]
    dy = y[j] - y[j - 1]
    tx = np.where(dx == 0, 0.0, (xq - x[i - 1]) / np.where(dx == 0, 1.0, dx))[:, None]
    ty = np.where(dy == 0, 0.0, (yq - y[j - 1]) / np.where(dy == 0, 1.0, dy))[:, None]
    ix = np.where(dx == 0, 0.0, 1.0 / np.where(dx == 0, 1.0, dx))[:, None]
    iy = np.where(dy == 0, 0.0, 1.0 / np.where(dy == 0, 1.0, dy))[:, None]
    f00, f10, f01, f11 = f[i - 1, j - 1], f[i, j - 1], f[i - 1, j], f[i, j]
    fq = (1 - tx) * (1 - ty) * f00 + tx * (1 - ty) * f10 + (1 - tx) * ty * f01 + tx * ty * f11
    fx = ix * ((1 - ty) * (f10 - f00) + ty * (f11 - f01))
    fy = iy * ((1 - tx) * (f01 - f00) + tx * (f11 - f10))
    outside = (xq < x[0]) | (xq > x[-1]) | (yq < y[0]) | (yq > y[-1])
    for a in (fq, fx, fy):
        a[outside] = 0.0
    return fq, fx, fy


def _interp_rows_slope(lt, lp, F):
    """``_interp_rows`` plus the slope dI/dlambda' of the bracket used (0 where the
    value is clamped to an end of the row)."""
    n, nl = lp.shape
    i = np.empty((n, lt.shape[0]), dtype=np.int64)
    for r in range(n):
        i[r] = np.searchsorted(lp[r], lt, side="right")
    ic = np.clip(i, 1, nl - 1)
    x0 = np.take_along_axis(lp, ic - 1, axis=1)
    x1 = np.take_along_axis(lp, ic, axis=1)
    f0 = np.take_along_axis(F, ic - 1, axis=1)
    f1 = np.take_along_axis(F, ic, axis=1)
    dx = x1 - x0
    slope = np.where(dx == 0, 0.0, (f1 - f0) / np.where(dx == 0, 1.0, dx))
    val = f0 + (lt[None, :] - x0) * slope
    lo = lt[None, :] < lp[:, :1]
    hi = lt[None, :] > lp[:, -1:]
    val = np.where(lo, F[:, :1], np.where(hi, F[:, -1:], val))
    slope = np.where(lo | hi, 0.0, slope)
    return val, slope


def doppler_grid(wave_z, v_los, smooth=False):
    """The shifted SSP grid: float32 like the reference, or (``smooth``) float64
    ``lambda_z * exp(v/c)`` for finite differences in v."""
    if not smooth:
        return velocity_doppler_shift32(wave_z, v_los).astype(np.float64)
    v = np.asarray(v_los, dtype=np.float64)
    return np.asarray(wave_z, dtype=np.float32).astype(np.float64)[None, :] * np.exp(
        v / SPEED_OF_LIGHT)[:, None]


def particle_objective(mass, metallicity, age, v_los, ssp_metallicity, ssp_age, ssp_flux,
                       wave_z, wave_t, adj_rows, smooth=True):
    """``sum_t adj_rows[p, t] * c_p[t]`` per particle, with ``c_p`` the resampled,
    mass-scaled spectrum of ``particle_spectra``.  With ``smooth`` the shifted grid and
    the (metallicity, age) queries stay float64, for finite differences."""
    qd = np.float64 if smooth else np.float32
    G = interp2d_linear(metallicity, age, ssp_metallicity, ssp_age, ssp_flux, query_dtype=qd)
    m = np.asarray(mass, dtype=np.float64)
    lp = doppler_grid(wave_z, v_los, smooth)
    lt = np.asarray(wave_t, dtype=np.float32).astype(np.float64)
    in_range = (lp >= lt.min()) & (lp <= lt.max())
    T = np.sum(G * calculate_diff(lp) * in_range, axis=1)
    I = _interp_rows(lt, lp, G)
    Tp = np.sum(I * calculate_diff(lt)[None, :], axis=1)
    with np.errstate(divide="ignore", invalid="ignore"):
        s = _nan_to_num32(T / Tp)
    return m * s * np.sum(np.asarray(adj_rows, dtype=np.float64) * I, axis=1)


def particle_grads(mass, metallicity, age, v_los, ssp_metallicity, ssp_age, ssp_flux,
                   wave_z, wave_t, adj_rows, smooth=False):
    """Analytic d/d(mass, metallicity, age, v_los) of ``particle_objective``: the
    derivative of the forward formulas (core/ifu.py:63-295, spectra/ifu.py:168-266)
    with the interpolation brackets and the in-range mask held fixed.  With
    beta = m T / T' and gamma = sum_t a_t I_t:
        d/dm = (T/T') gamma,
        d/dtheta = beta H_theta + gamma (m/T') (dT/dtheta - (T/T') dT'/dtheta),
    H_theta = sum_t a_t dI_t/dtheta; dI_t/dv = -lambda_t * slope_t / c, dT/dv = T/c.
    Particles with T' = 0 or a non-finite T/T' get zeros.  Returns four (n,) arrays."""
    m = np.asarray(mass, dtype=np.float64)
    qd = np.float64 if smooth else np.float32
    G, GZ, GA = interp2d_linear_grad(metallicity, age, ssp_metallicity, ssp_age, ssp_flux,
                                     query_dtype=qd)
    lp = doppler_grid(wave_z, v_los, smooth)
    lt = np.asarray(wave_t, dtype=np.float32).astype(np.float64)
    a = np.asarray(adj_rows, dtype=np.float64)
    in_range = (lp >= lt.min()) & (lp <= lt.max())
    dlp = calculate_diff(lp) * in_range
    dlt = calculate_diff(lt)[None, :]
    T, TZ, TA = (np.sum(X * dlp, axis=1) for X in (G, GZ, GA))
    I, slope = _interp_rows_slope(lt, lp, G)
    IZ = _interp_rows(lt, lp, GZ)
    IA = _interp_rows(lt, lp, GA)
    Iv = -lt[None, :] * slope / SPEED_OF_LIGHT
    Tp = np.sum(I * dlt, axis=1)
    gamma = np.sum(a * I, axis=1)
    H = {k: np.sum(a * X, axis=1) for k, X in (("Z", IZ), ("A", IA), ("v", Iv))}
    D = {k: np.sum(dlt * X, axis=1) for k, X in (("Z", IZ), ("A", IA), ("v", Iv))}
    dT = {"Z": TZ, "A": TA, "v": T / SPEED_OF_LIGHT}
    with np.errstate(divide="ignore", invalid="ignore"):
        sc = T / Tp
        ok = (Tp != 0) & np.isfinite(sc)
        sc = np.where(ok, sc, 0.0)
        k = np.where(ok, m / np.where(Tp == 0, 1.0, Tp), 0.0)
    beta = m * sc
    out = [np.where(ok, sc * gamma, 0.0)]
    for key in ("Z", "A", "v"):
        out.append(np.where(ok, beta * H[key] + gamma * k * (dT[key] - sc * D[key]), 0.0))
    return tuple(out)


def psf_taps_derivative(m, sigma):
    """1-D PSF taps t (normalised Gaussian of ``gaussian_kernel_2d``) and dt/dsigma."""
    x = np.arange(-((m - 1) / 2), ((m - 1) / 2) + 1)
    e = np.exp(-(x**2) / (2 * sigma**2))
    de = e * x**2 / sigma**3
    S = e.sum()
    t = e / S
    return t, (de - t * de.sum()) / S


def lsf_taps_derivative(sigma, wave_res, factor=12):
    """``lsf_kernel`` taps and their derivative with respect to sigma."""
    x = np.arange(-factor * wave_res, factor * wave_res + wave_res, wave_res,
                  dtype=np.float32).astype(np.float64)
    e = np.exp(-0.5 * x**2 / sigma**2)
    de = e * x**2 / sigma**3
    S = e.sum()
    t = e / S
    return t, (de - t * de.sum()) / S


# ----------------------------------------------------------------------------------
# Orientation (core/rotation.py:11-117, galaxy/alignment.py:66-265)
# ----------------------------------------------------------------------------------
def moment_of_inertia_tensor(positions, masses, halfmass_radius):
    """alignment.py:66-120 in float64.  The reference selects with
    ``jnp.where(distances <= r, size=N)``, whose index list is padded with 0: particle 0
    enters once more for every particle outside the radius."""
    pos = np.asarray(positions, dtype=np.float32)
    m = np.asarray(masses, dtype=np.float32).astype(np.float64)
    d = np.sqrt(np.sum(pos * pos, axis=1, dtype=np.float32))
    inside = np.nonzero(d <= np.float32(halfmass_radius))[0]
    idx = np.concatenate([inside, np.zeros(pos.shape[0] - inside.size, dtype=np.int64)])
    p = pos[idx].astype(np.float64)
    mm = m[idx]
    r2 = np.sum(p * p, axis=1)
    I = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            if i == j:
                I[i, j] = np.sum(mm * r2 - mm * p[:, i] ** 2)
            else:
                I[i, j] = -np.sum(mm * p[:, i] * p[:, j])
    return I


def rotation_matrix_from_inertia_tensor(I):
    """alignment.py:123-138: eigenvectors as columns, ascending eigenvalues."""
    w, v = np.linalg.eigh(np.asarray(I, dtype=np.float64))
    return v[:, np.argsort(w)]


def euler_rotation_matrix(alpha, beta, gamma):
    """alignment.py:162-205: R_z(gamma) R_y(beta) R_x(alpha), degrees."""
    a, b, g = np.deg2rad([alpha, beta, gamma])
    Rx = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
    Ry = np.array([[np.cos(b), 0, np.sin(b)], [0, 1, 0], [-np.sin(b), 0, np.cos(b)]])
    Rz = np.array([[np.cos(g), -np.sin(g), 0], [np.sin(g), np.cos(g), 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def rotate_galaxy(positions, velocities, masses, halfmass_radius, alpha, beta, gamma):
    """alignment.py:228-265: principal-frame rotation then Euler rotation, row vectors;
    float64 products rounded once to float32."""
    R = rotation_matrix_from_inertia_tensor(
        moment_of_inertia_tensor(positions, masses, halfmass_radius))
    M = R @ euler_rotation_matrix(alpha, beta, gamma)
    pos = (np.asarray(positions, dtype=np.float32).astype(np.float64) @ M).astype(np.float32)
    vel = (np.asarray(velocities, dtype=np.float32).astype(np.float64) @ M).astype(np.float32)
    return pos, vel


__all__ += ["moment_of_inertia_tensor", "rotation_matrix_from_inertia_tensor",
            "euler_rotation_matrix", "rotate_galaxy"]


# ----------------------------------------------------------------------------------
# Observation noise (core/noise.py:17-80, telescope/noise/noise.py:35-115)
# ----------------------------------------------------------------------------------
def noise_sigma(datacube, signal_to_noise):
    """calculate_S2N (noise.py:35-76): per-spaxel relative noise
    sqrt(median flux) / s2n / sqrt(flux), 0 where flux <= 0; the median is over
    where(flux > 0, flux, nan), so any flux <= 0 makes it NaN -> 0."""
    cube = np.asarray(datacube, dtype=np.float64)
    flux = cube.sum(axis=-1)
    nonzero = flux > 0
    with np.errstate(invalid="ignore"):
        med = np.median(np.where(nonzero, flux, np.nan))
    med = 0.0 if np.isnan(med) else med
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.sqrt(med) / signal_to_noise / np.sqrt(flux)
    return np.where(nonzero, s, 0.0), med


def philox4x32_10(counter, key):
    """Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), pure Python: 10 rounds of
    two 32x32->64 multiplies with M0 = 0xD2511F53, M1 = 0xCD9E8D57 and a Weyl key
    schedule W0 = 0x9E3779B9, W1 = 0xBB67AE85."""
    m = 0xFFFFFFFF
    c = [int(x) & m for x in counter]
    k0, k1 = int(key[0]) & m, int(key[1]) & m
    for _ in range(10):
        p0 = 0xD2511F53 * c[0]
        p1 = 0xCD9E8D57 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & m, p1 & m, ((p0 >> 32) ^ c[3] ^ k1) & m, p0 & m]
        k0 = (k0 + 0x9E3779B9) & m
        k1 = (k1 + 0xBB67AE85) & m
    return c


def philox4x32_10_arrays(c0, c1, c2, c3, k0, k1):
    """philox4x32_10 over arrays of counters (NumPy uint64 arithmetic, same rounds)."""
    m = np.uint64(0xFFFFFFFF)
    c = [np.asarray(x, dtype=np.uint64) & m for x in (c0, c1, c2, c3)]
    k0, k1 = np.uint64(int(k0) & 0xFFFFFFFF), np.uint64(int(k1) & 0xFFFFFFFF)
    for _ in range(10):
        p0 = np.uint64(0xD2511F53) * c[0]
        p1 = np.uint64(0xCD9E8D57) * c[2]
        c = [((p1 >> np.uint64(32)) ^ c[1] ^ k0) & m, p1 & m,
             ((p0 >> np.uint64(32)) ^ c[3] ^ k1) & m, p0 & m]
        k0 = (k0 + np.uint64(0x9E3779B9)) & m
        k1 = (k1 + np.uint64(0xBB67AE85)) & m
    return c


def noise_draws(n_spaxels, n_wave, seed, distribution="normal"):
    """The draws z[s, t] of rubix_apply_noise (float64): element (s, t) has the index
    e = s * n_wave + t and takes output e % 4 of the Philox4x32-10 call with counter
    (e // 4 low word, high word, 0, 0) and key (seed low word, high word).  Uniform
    draws are (bits >> 8) / 2^24; normal draws pair outputs (0, 1) and (2, 3) by
    Box-Muller, r = sqrt(-2 ln u) with u = ((bits >> 8) + 1) / 2^24 from the first of the
    pair and the angle 2 pi (u' - 1/2) from the second (cos for the first, sin for the
    second).  Test infrastructure: the noise of rubix itself (jax.random with a fixed
    key, telescope/noise/noise.py:103) is matched in distribution only."""
    e = np.arange(int(n_spaxels) * int(n_wave), dtype=np.uint64)
    q = e >> np.uint64(2)
    r = philox4x32_10_arrays(q & np.uint64(0xFFFFFFFF), q >> np.uint64(32), 0, 0,
                             int(seed) & 0xFFFFFFFF, (int(seed) >> 32) & 0xFFFFFFFF)
    u = [(x >> np.uint64(8)).astype(np.float64) / 16777216.0 for x in r]
    if distribution == "uniform":
        outs = u
    else:
        u0 = [((x >> np.uint64(8)).astype(np.float64) + 1.0) / 16777216.0 for x in r]
        r1 = np.sqrt(-2.0 * np.log(u0[0]))
        r2 = np.sqrt(-2.0 * np.log(u0[2]))
        a1 = 2.0 * np.pi * (u[1] - 0.5)
        a2 = 2.0 * np.pi * (u[3] - 0.5)
        outs = [r1 * np.cos(a1), r1 * np.sin(a1), r2 * np.cos(a2), r2 * np.sin(a2)]
    j = (e & np.uint64(3)).astype(np.int64)
    z = np.choose(j, outs)
    return z.reshape(int(n_spaxels), int(n_wave))


__all__ += ["noise_sigma", "philox4x32_10", "philox4x32_10_arrays", "noise_draws"]

__all__ += ["interp2d_linear_grad", "doppler_grid", "particle_objective", "particle_grads",
            "psf_taps_derivative", "lsf_taps_derivative"]


def _selftest():  # pragma: no cover - manual helper
    e, b = calculate_spatial_bin_edges(1.0, np.int64(10), 2.0)
    assert len(e) == 12 and math.isclose(float(b), 0.2, rel_tol=1e-6)
