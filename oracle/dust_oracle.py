"""NumPy restatement of rubix's dust-extinction step (``calculate_extinction``).

TEST INFRASTRUCTURE ONLY.  The product package never imports this module; tests use it
as the checker of the dust kernels and of the host-side extinction curves.

Restated, with the rubix source each part follows (``path:line`` relative to the rubix
project root):

* the extinction-curve building blocks of spectra/dust/generic_models.py (PowerLaw1d,
  Polynomial1d, Drude1d, _modified_drude, FM90) and spectra/dust/helpers.py
  (_smoothstep, poly_map_domain);
* the two R(V) models of spectra/dust/extinction_models.py (Cardelli89, Gordon23) and
  ``extinguish`` of spectra/dust/dust_baseclasses.py:120-164;
* the dust-to-gas ratio and the per-cell extinction of
  spectra/dust/dust_extinction.py:13-160;
* ``apply_spaxel_extinction`` (spectra/dust/dust_extinction.py:169-358) step by step:
  lexsort of gas and stars by (spaxel, z), segment boundaries by searchsorted, and
  for every spaxel the masked cumulative sum, the 1e30 trick for cells of other
  spaxels, the stable key-value sort and ``jnp.interp`` with left extrapolation.

Arithmetic is float32 where the reference computes in float32 (positions, masses, the
cumulative sums, the interpolation); the extinction curves are evaluated in float64
and rounded, as the float32 curve of the reference differs from them by a few ulp.

Parity status.  The reference cannot be imported here (no JAX).  The curve building
blocks are pinned by the reference's known answers (tests/test_dust_classes.py:14-81);
the rest follows the source line by line and is unpinned by reference outputs
("parity unpinned" for the column density and the Cardelli89 / Gordon23 curves beyond
the range checks of tests/test_dust_classes.py:112-166).
"""

from __future__ import annotations

from math import comb

import numpy as np

# rubix/config/rubix_config.yml:6-18 (constants) and :145-150 (dust defaults)
KPC_TO_CM = 3.08568e21
MSUN_TO_GRAMS = 1.989e33
DUST_DEFAULTS = {"extinction_model": "Cardelli89", "Rv": 3.1,
                 "dust_to_gas_model": "broken power law fit", "Xco": "Z",
                 "dust_grain_density": 3.5}
RV_MODELS = ["Cardelli89", "Gordon23"]  # spectra/dust/extinction_models.py:10-13

F32 = np.float32


# ----------------------------------------------------------------------------------
# Generic model functions: spectra/dust/generic_models.py, spectra/dust/helpers.py
# ----------------------------------------------------------------------------------

def power_law_1d(x, amplitude, x_0, alpha):
    """generic_models.py PowerLaw1d: A * (x / x_0) ** -alpha."""
    x = np.asarray(x, np.float64)
    return amplitude * (x / x_0) ** (-alpha)


def poly_map_domain(oldx, domain, window):
    """helpers.py poly_map_domain: shift and scale ``domain`` onto ``window``."""
    d0, d1 = domain
    w0, w1 = window
    scl = (w1 - w0) / (d1 - d0)
    off = (w0 * d1 - w1 * d0) / (d1 - d0)
    return off + scl * np.asarray(oldx, np.float64)


def polynomial_1d(x, coeffs, domain=(-1.0, 1.0), window=(-1.0, 1.0)):
    """generic_models.py Polynomial1d: Horner's rule after the domain map."""
    x = np.asarray(x, np.float64)
    coeffs = list(np.asarray(coeffs, np.float64))
    if domain is not None:
        x = poly_map_domain(x, domain, window)
    if len(coeffs) == 1:
        return coeffs[-1] * np.ones_like(x)
    c0 = coeffs[-1]
    for i in range(2, len(coeffs) + 1):
        c0 = coeffs[-i] + c0 * x
    return c0


def drude_1d(x, amplitude=1.0, x_0=1.0, fwhm=1.0):
    """generic_models.py Drude1d."""
    if x_0 == 0:
        raise ValueError("0 is not an allowed value for x_0")
    x = np.asarray(x, np.float64)
    return amplitude * ((fwhm / x_0) ** 2) / ((x / x_0 - x_0 / x) ** 2 + (fwhm / x_0) ** 2)


def modified_drude(x, scale, x_o, gamma_o, asym):
    """generic_models.py _modified_drude: Drude profile with a variable asymmetry."""
    x = np.asarray(x, np.float64)
    gamma = 2.0 * gamma_o / (1.0 + np.exp(asym * (x - x_o)))
    return scale * ((gamma / x_o) ** 2) / ((x / x_o - x_o / x) ** 2 + (gamma / x_o) ** 2)


_FM90_BOUNDS = {"C1": (-10.0, 5.0), "C2": (-0.1, 5.0), "C3": (-1.0, 6.0), "C4": (-0.5, 1.5),
                "xo": (4.5, 4.9), "gamma": (0.6, 1.7)}


def fm90(x, C1=0.10, C2=0.70, C3=3.23, C4=0.41, xo=4.59, gamma=0.95):
    """generic_models.py FM90 (Fitzpatrick & Massa 1990): E(x-V)/E(B-V) with the
    parameter bounds checked as the reference does."""
    for name, v in (("C1", C1), ("C2", C2), ("C3", C3), ("C4", C4), ("xo", xo),
                    ("gamma", gamma)):
        lo, hi = _FM90_BOUNDS[name]
        if not (lo <= v <= hi):
            raise ValueError(f"{name} is out of bounds: {v}")
    x = np.asarray(x, np.float64)
    e = C1 + C2 * x
    x2 = x ** 2
    e = e + C3 * (x2 / ((x2 - xo ** 2) ** 2 + x2 * gamma ** 2))
    fnuv = x >= 5.9
    y = np.where(fnuv, x - 5.9, 0.0)
    return np.where(fnuv, e + C4 * (0.5392 * y ** 2 + 0.05644 * y ** 3), e)


def smoothstep(x, x_min=0.0, x_max=1.0, N=1):
    """helpers.py _smoothstep: the order-N smoothstep polynomial of the clipped ramp."""
    x = np.clip((np.asarray(x, np.float64) - x_min) / (x_max - x_min), 0, 1)
    result = 0.0
    for n in range(0, N + 1):
        result = result + comb(N + n, n) * comb(2 * N + 1, N - n) * (-x) ** n
    return result * x ** (N + 1)


# ----------------------------------------------------------------------------------
# R(V) models: spectra/dust/extinction_models.py
# ----------------------------------------------------------------------------------

def cardelli89(wave, Rv):
    """Cardelli89.evaluate (extinction_models.py:104-180): A(x)/A(V) with the CCM89
    coefficients applied to ``wave`` as given (rubix passes wavelengths in microns
    where the published formula uses 1/micron; kept as the reference does)."""
    w = np.asarray(wave, np.float64)
    a = np.zeros_like(w)
    b = np.zeros_like(w)
    ir = (0.3 <= w) & (w < 1.1)
    opt = (1.1 <= w) & (w < 3.3)
    nuv = (3.3 <= w) & (w <= 8.0)
    fnuv = (5.9 <= w) & (w <= 8)
    fuv = (8 < w) & (w <= 10)
    a = np.where(ir, 0.574 * w ** 1.61, a)
    b = np.where(ir, -0.527 * w ** 1.61, b)
    y = w - 1.82
    a = np.where(opt, 1 + 0.17699 * y - 0.50447 * y ** 2 - 0.02427 * y ** 3 + 0.72085 * y ** 4
                 + 0.01979 * y ** 5 - 0.77530 * y ** 6 + 0.32999 * y ** 7, a)
    b = np.where(opt, 1.41338 * y + 2.28305 * y ** 2 + 1.07233 * y ** 3 - 5.38434 * y ** 4
                 - 0.62251 * y ** 5 + 5.30260 * y ** 6 - 2.09002 * y ** 7, b)
    with np.errstate(divide="ignore"):
        a = np.where(nuv, 1.752 - 0.316 * w - 0.104 / ((w - 4.67) ** 2 + 0.341), a)
        b = np.where(nuv, -3.09 + 1.825 * w + 1.206 / ((w - 4.62) ** 2 + 0.263), b)
    y = w - 5.9
    a = np.where(fnuv, a + (-0.04473 * y ** 2 - 0.009779 * y ** 3), a)
    b = np.where(fnuv, b + (0.2130 * y ** 2 + 0.1207 * y ** 3), b)
    y = w - 8.0
    a = np.where(fuv, -1.073 - 0.628 * y + 0.137 * y ** 2 - 0.070 * y ** 3, a)
    b = np.where(fuv, 13.670 + 4.257 * y - 0.420 * y ** 2 + 0.374 * y ** 3, b)
    return a + b / Rv


_G23_IR_A = [0.38526, 1.68467, 0.78791, 4.30578, 4.78338, 0.06652, 9.8434, 2.21205, -0.24703,
             0.0267, 19.58294, 17.0, -0.27]
_G23_OPT_A = [-0.35848, 0.7122, 0.08746, -0.05403, 0.00674, 0.03893, 2.288, 0.243,
              0.02965, 2.054, 0.179, 0.01747, 1.587, 0.243]
_G23_OPT_B = [0.12354, -2.68335, 2.01901, -0.39299, 0.03355, 0.18453, 2.288, 0.243,
              0.19728, 2.054, 0.179, 0.1713, 1.587, 0.243]
_G23_UV_A = (0.81297, 0.2775, 1.06295, 0.11303, 4.60, 0.99)
_G23_UV_B = (-2.97868, 1.89808, 3.10334, 0.65484, 4.60, 0.99)


def _g23_nirmir(wave, p):
    """Gordon23.nirmir_intercept (extinction_models.py:400-445)."""
    (scale, alpha, alpha2, swave, swidth, s1a, s1c, s1f, s1s, s2a, s2c, s2f, s2s) = p
    w = np.asarray(wave, np.float64)
    pow1 = scale * w ** (-alpha)
    ratio = swave ** (-alpha) / swave ** (-alpha2)
    pow2 = scale * ratio * w ** (-alpha2)
    wt = smoothstep(w, swave - swidth / 2, swave + swidth / 2, 1)
    ax = pow1 * (1.0 - wt) + pow2 * wt
    ax = ax + modified_drude(w, s1a, s1c, s1f, s1s)
    return ax + modified_drude(w, s2a, s2c, s2f, s2s)


def _g23_cpd(x, p):
    """compound_polynomial_drude_model of Gordon23.evaluate: polynomial plus three
    Drude profiles, in wavenumber."""
    return (polynomial_1d(x, p[:5]) + drude_1d(x, p[5], p[6], p[7]) + drude_1d(x, p[8], p[9], p[10])
            + drude_1d(x, p[11], p[12], p[13]))


def gordon23(wave, Rv):
    """Gordon23.evaluate (extinction_models.py:255-398), ``wave`` in microns."""
    w = np.asarray(wave, np.float64)
    a = np.zeros_like(w)
    b = np.zeros_like(w)
    ir = (1.0 <= w) & (w < 35.0)
    opt = (0.3 <= w) & (w < 1.1)
    uv = (0.09 <= w) & (w <= 0.3)
    optir = (w >= 0.9) & (w <= 1.1)
    uvopt = (w >= 0.3) & (w <= 0.33)
    with np.errstate(all="ignore"):
        ir_a = _g23_nirmir(w, _G23_IR_A)
        ir_b = power_law_1d(w, -1.01251, 1.0, -1.06099)
        opt_a = _g23_cpd(1 / w, _G23_OPT_A)
        opt_b = _g23_cpd(1 / w, _G23_OPT_B)
        uv_a = fm90(1 / w, *_G23_UV_A)
        uv_b = fm90(1 / w, *_G23_UV_B)
    a = np.where(ir, ir_a, a)
    b = np.where(ir, ir_b, b)
    a = np.where(opt, opt_a, a)
    b = np.where(opt, opt_b, b)
    wt = smoothstep(w, 0.9, 1.1, 1)
    a = np.where(optir, (1.0 - wt) * opt_a + wt * ir_a, a)
    b = np.where(optir, (1.0 - wt) * opt_b + wt * ir_b, b)
    a = np.where(uv, uv_a, a)
    b = np.where(uv, uv_b, b)
    wt = smoothstep(w, 0.3, 0.33, 1)
    a = np.where(uvopt, (1.0 - wt) * uv_a + wt * opt_a, a)
    b = np.where(uvopt, (1.0 - wt) * uv_b + wt * opt_b, b)
    return a + b * (1 / Rv - 1 / 3.1)


def axav(model, wave, Rv):
    """A(wave)/A(V) of a model named as in rubix's Rv_model_dict."""
    if model not in RV_MODELS:
        raise ValueError(f"Extinction model '{model}' is not available. Choose from {RV_MODELS}.")
    return cardelli89(wave, Rv) if model == "Cardelli89" else gordon23(wave, Rv)


def extinguish(ax, Av):
    """dust_baseclasses.py:120-164 ``extinguish``: 10 ** (-0.4 * A(x)/A(V) * Av),
    float32 as in the reference (-0.4 * axav rounded first, then times Av)."""
    e = (F32(-0.4) * np.asarray(ax, np.float32)).astype(np.float32)
    y = (e[None, :] * np.asarray(Av, np.float32).reshape(-1, 1)).astype(np.float32)
    return np.power(10.0, y.astype(np.float64)).astype(np.float32)


# ----------------------------------------------------------------------------------
# Dust mass and per-cell extinction: spectra/dust/dust_extinction.py:13-160
# ----------------------------------------------------------------------------------

def dust_to_gas_ratio(log_oh, model, Xco, dtype=np.float32):
    """calculate_dust_to_gas_ratio (dust_extinction.py:13-90), Remy-Ruyer et al. 2014
    Table 1, float32 (``dtype=np.float64`` for differences)."""
    F32 = dtype  # noqa: N806 -- the arithmetic type of this evaluation
    g = np.asarray(log_oh, dtype)
    x_sol = F32(8.69)
    if model == "power law slope fixed":
        raise NotImplementedError("power law slope fixed not implemented yet.")
    if Xco == "MW":
        if model == "power law slope free":
            return (F32(1) / F32(10) ** (F32(2.21) + F32(1.62) * (x_sol - g))).astype(dtype)
        a, ah, b, al, xt = 2.21, 1.00, 0.68, 3.08, 7.96
    elif Xco == "Z":
        if model == "power law slope free":
            return (F32(1) / F32(10) ** (F32(2.21) + F32(2.02) * (x_sol - g))).astype(dtype)
        a, ah, b, al, xt = 2.21, 1.00, 0.96, 3.10, 8.10
    else:
        raise ValueError(f"unknown Xco {Xco!r}")
    if model != "broken power law fit":
        raise ValueError(f"unknown dust_to_gas_model {model!r}")
    hi = F32(10) ** (F32(a) + F32(ah) * (x_sol - g))
    lo = F32(10) ** (F32(b) + F32(al) * (x_sol - g))
    return (F32(1) / np.where(g > F32(xt), hi, lo)).astype(dtype)


def log_oh(metals, h_col=0, o_col=4, dtype=np.float32):
    """12 + log10(O / (16 H)) of every gas cell (dust_extinction.py:291-293)."""
    m = np.asarray(metals, dtype)
    with np.errstate(all="ignore"):
        return (dtype(12) + np.log10(m[:, o_col] / (dtype(16) * m[:, h_col]))).astype(dtype)


def extinction_scale(dust_grain_density, effective_wavelength=5448.0):
    """Constant factor of calculate_extinction (dust_extinction.py:93-160):
    3 pi (Msun/kpc^2 -> g/cm^2) / (0.4 ln10 lambda_V[cm] rho_D)."""
    convert = float(MSUN_TO_GRAMS) / float(KPC_TO_CM) ** 2
    return 3 * np.pi * convert / (0.4 * np.log(10) * effective_wavelength * 1e-8
                                  * dust_grain_density)


def gas_extinction(mass, metals, spaxel_area, dust=None, h_col=0, o_col=4,
                   dtype=np.float32):
    """Per-cell extinction of the gas: dust mass (gas mass times the dust-to-gas ratio
    of 12 + log(O/H)) through calculate_extinction, divided by the spaxel area
    (dust_extinction.py:291-306), float32 (``dtype=np.float64`` for differences)."""
    d = dict(DUST_DEFAULTS)
    d.update(dust or {})
    dgr = dust_to_gas_ratio(log_oh(metals, h_col, o_col, dtype), d["dust_to_gas_model"],
                            d["Xco"], dtype)
    dm = (np.asarray(mass, dtype) * dgr).astype(dtype)
    with np.errstate(all="ignore"):
        e = (dm * dtype(extinction_scale(d["dust_grain_density"]))).astype(dtype)
        return (e / dtype(spaxel_area)).astype(dtype)


# ----------------------------------------------------------------------------------
# Column density at the stars: apply_spaxel_extinction, dust_extinction.py:262-358
# ----------------------------------------------------------------------------------

_INTERP_EPS = np.spacing(np.finfo(np.float32).eps)


def jax_interp(x, xp, fp, left_extrapolate=True, dtype=np.float32):
    """``jnp.interp(x, xp, fp, left="extrapolate")`` in float32 (or ``dtype``): bracket
    i = clip(searchsorted(xp, x, 'right'), 1, n-1), fp[i-1] + (x - xp[i-1]) / dx * df
    (fp[i-1] where |dx| <= spacing(eps)), fp[-1] to the right of xp[-1]."""
    x = np.asarray(x, dtype)
    xp = np.asarray(xp, dtype)
    fp = np.asarray(fp, dtype)
    i = np.clip(np.searchsorted(xp, x, side="right"), 1, len(xp) - 1)
    df = (fp[i] - fp[i - 1]).astype(dtype)
    dx = (xp[i] - xp[i - 1]).astype(dtype)
    delta = (x - xp[i - 1]).astype(dtype)
    dx0 = np.abs(dx) <= _INTERP_EPS
    with np.errstate(all="ignore"):
        q = (delta / np.where(dx0, dtype(1), dx)).astype(dtype)
        f = np.where(dx0, fp[i - 1], (fp[i - 1] + (q * df).astype(dtype)).astype(dtype))
    if not left_extrapolate:
        f = np.where(x < xp[0], fp[0], f)
    f = np.where(x > xp[-1], fp[-1], f)
    return f.astype(dtype)


def spaxel_av(gas_z, gas_pa, gas_ext, star_z, star_pa, n_spaxels, spaxels=None,
              dtype=np.float32):
    """Av of every star (dust_extinction.py:262-343), step by step.

    Gas and stars are lexsorted by (pixel assignment, z); for each spaxel the gas
    extinction is summed cumulatively over the spaxel's cells (others masked to 0),
    the cells of other spaxels are moved to z * 1e30 with value 0, the (z, value)
    pairs are sorted stably and the spaxel's stars take ``jnp.interp`` of their z with
    left extrapolation.  ``spaxels`` restricts the loop to those spaxel ids (the Av of
    stars of other spaxels is then left at 0) so large inputs can be spot-checked.
    Returns float32 Av in the input order of the stars (``dtype=np.float64``: the same
    steps in float64, for differences; the gas heights are then taken as given).
    """
    gz = np.asarray(gas_z, dtype)
    gpa = np.asarray(gas_pa, np.int64)
    gext = np.asarray(gas_ext, dtype)
    sz = np.asarray(star_z, dtype)
    spa = np.asarray(star_pa, np.int64)
    ng, ns = gz.size, sz.size
    gsi = np.lexsort((gz, gpa))
    ssi = np.lexsort((sz, spa))
    ids = np.arange(n_spaxels)
    gb = np.concatenate([np.searchsorted(gpa[gsi], ids, side="left"), [ng]])
    sb = np.concatenate([np.searchsorted(spa[ssi], ids, side="left"), [ns]])
    ext_sorted = gext[gsi]
    z_sorted = gz[gsi]
    sz_sorted = sz[ssi]
    big = dtype(1e30) if dtype is np.float64 else F32(1e30)
    pos_g = np.arange(ng)
    av = np.zeros(ns, dtype)
    loop = ids if spaxels is None else np.asarray(spaxels, np.int64)
    for idx in loop:
        s0, s1 = sb[idx], sb[idx + 1]
        if s1 <= s0 or ng == 0:
            continue
        gmask = (pos_g >= gb[idx]) & (pos_g < gb[idx + 1])
        gmask2 = np.where(gmask, dtype(1), big).astype(dtype)
        with np.errstate(invalid="ignore"):
            cum = (np.cumsum((ext_sorted * gmask).astype(dtype), dtype=dtype)
                   * gmask).astype(dtype)
            xp = (z_sorted * gmask2).astype(dtype)
        order = np.argsort(xp, kind="stable")
        xp, fp = xp[order], cum[order]
        # only the spaxel's own stars keep their value (star_mask)
        av[s0:s1] += jax_interp(sz_sorted[s0:s1], xp, fp, left_extrapolate=True, dtype=dtype)
    out = np.empty_like(av)
    out[ssi] = av
    return out


def apply_spaxel_extinction(spectra, wave_t, gas, stars, n_spaxels, spaxel_area, dust=None):
    """apply_spaxel_extinction (dust_extinction.py:169-358): per-star Av, the model's
    transmission at ``wave_t / 1e4`` and the extincted spectra (float32).

    ``gas``: dict with coords (N_g, 3), pixel_assignment, mass, metals;
    ``stars``: dict with coords (N, 3), pixel_assignment.  Returns (spectra * T, Av, T).
    """
    d = dict(DUST_DEFAULTS)
    d.update(dust or {})
    model = d["extinction_model"]
    if model not in RV_MODELS:
        raise ValueError(f"Extinction model '{model}' is not available. Choose from {RV_MODELS}.")
    gext = gas_extinction(gas["mass"], gas["metals"], spaxel_area, d)
    av = spaxel_av(np.asarray(gas["coords"], np.float32)[:, 2], gas["pixel_assignment"], gext,
                   np.asarray(stars["coords"], np.float32)[:, 2], stars["pixel_assignment"],
                   n_spaxels)
    wave_um = (np.asarray(wave_t, np.float32) / F32(1e4)).astype(np.float32)
    T = extinguish(axav(model, wave_um, d["Rv"]), av)
    return (np.asarray(spectra, np.float32) * T).astype(np.float32), av, T
