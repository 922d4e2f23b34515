"""Host side of the dust extinction: extinction curves, dust-to-gas ratio parameters
and the per-wavelength exponent the dusty accumulate kernel takes.

rubix evaluates the curve of an R(V) model (rubix/spectra/dust/extinction_models.py)
at the telescope wavelengths divided by 1e4 and turns each star's A_V into the
transmission 10^(-0.4 A(x)/A(V) A_V) (spectra/dust/dust_baseclasses.py:120-164).  The
curve depends only on the configuration, so it is a host-side constant like the PSF and
LSF taps; the kernel takes e_t = -0.4 log2(10) A(x_t)/A(V) and computes 2^(e_t A_V).

The curve formulas are the published ones of Cardelli, Clayton & Mathis (1989) and
Gordon et al. (2023), with rubix's coefficient tables, evaluated in float64.  rubix's
Cardelli89 applies the CCM89 polynomials to the wavelength in microns (the published
variable is the wavenumber in 1/micron); this module does the same so that the cube
matches rubix's.
"""

from __future__ import annotations

import math

import numpy as np

__all__ = ["RV_MODELS", "axav", "cardelli89", "gordon23", "extinction_exponent",
           "dust_to_gas_params", "extinction_scale", "DUST_DEFAULTS"]

RV_MODELS = ["Cardelli89", "Gordon23"]  # rubix/spectra/dust/extinction_models.py:10-13

# rubix/config/rubix_config.yml:145-150 (read from rubix's own config, not the user's,
# for the dust-to-gas model and X_CO: spectra/dust/dust_extinction.py:294-298)
DUST_DEFAULTS = {"extinction_model": "Cardelli89", "Rv": 3.1,
                 "dust_to_gas_model": "broken power law fit", "Xco": "Z",
                 "dust_grain_density": 3.5}

_MSUN_G = 1.989e33     # rubix_config.yml:7
_KPC_CM = 3.08568e21   # rubix_config.yml:6
_LAMBDA_V_A = 5448.0   # Johnson V effective wavelength, dust_extinction.py:96


def _horner(x, coeffs):
    out = np.full_like(x, coeffs[-1])
    for c in coeffs[-2::-1]:
        out = out * x + c
    return out


def _drude(x, amp, x0, width):
    r = width / x0
    return amp * r * r / ((x / x0 - x0 / x) ** 2 + r * r)


def _drude_asym(x, amp, x0, width, asym):
    g = 2.0 * width / (1.0 + np.exp(asym * (x - x0)))
    return _drude(x, amp, x0, g)


def _fm90(x, c1, c2, c3, c4, x0, gamma):
    x2 = x * x
    e = c1 + c2 * x + c3 * x2 / ((x2 - x0 * x0) ** 2 + x2 * gamma * gamma)
    y = np.maximum(x - 5.9, 0.0)
    return np.where(x >= 5.9, e + c4 * (0.5392 * y * y + 0.05644 * y ** 3), e)


def _smooth(x, lo, hi):
    t = np.clip((x - lo) / (hi - lo), 0.0, 1.0)
    return t * t * (3.0 - 2.0 * t)


def cardelli89(wave, Rv: float) -> np.ndarray:
    """A(x)/A(V), CCM89 with rubix's use of ``wave`` (extinction_models.py:104-180)."""
    x = np.asarray(wave, dtype=np.float64)
    a = np.zeros_like(x)
    b = np.zeros_like(x)
    m = (x >= 0.3) & (x < 1.1)
    p = np.power(np.where(m, x, 1.0), 1.61)
    a[m], b[m] = 0.574 * p[m], -0.527 * p[m]
    m = (x >= 1.1) & (x < 3.3)
    y = x - 1.82
    a = np.where(m, _horner(y, [1.0, 0.17699, -0.50447, -0.02427, 0.72085, 0.01979, -0.77530,
                                0.32999]), a)
    b = np.where(m, _horner(y, [0.0, 1.41338, 2.28305, 1.07233, -5.38434, -0.62251, 5.30260,
                                -2.09002]), b)
    m = (x >= 3.3) & (x <= 8.0)
    a = np.where(m, 1.752 - 0.316 * x - 0.104 / ((x - 4.67) ** 2 + 0.341), a)
    b = np.where(m, -3.09 + 1.825 * x + 1.206 / ((x - 4.62) ** 2 + 0.263), b)
    m = (x >= 5.9) & (x <= 8.0)
    y = x - 5.9
    a = np.where(m, a - 0.04473 * y * y - 0.009779 * y ** 3, a)
    b = np.where(m, b + 0.2130 * y * y + 0.1207 * y ** 3, b)
    m = (x > 8.0) & (x <= 10.0)
    y = x - 8.0
    a = np.where(m, -1.073 - 0.628 * y + 0.137 * y * y - 0.070 * y ** 3, a)
    b = np.where(m, 13.670 + 4.257 * y - 0.420 * y * y + 0.374 * y ** 3, b)
    return a + b / Rv


# Gordon et al. (2023) coefficients as tabulated by rubix (extinction_models.py:288-330)
_G23_IR = (0.38526, 1.68467, 0.78791, 4.30578, 4.78338,
           (0.06652, 9.8434, 2.21205, -0.24703), (0.0267, 19.58294, 17.0, -0.27))
_G23_OPT_A = ((-0.35848, 0.7122, 0.08746, -0.05403, 0.00674),
              ((0.03893, 2.288, 0.243), (0.02965, 2.054, 0.179), (0.01747, 1.587, 0.243)))
_G23_OPT_B = ((0.12354, -2.68335, 2.01901, -0.39299, 0.03355),
              ((0.18453, 2.288, 0.243), (0.19728, 2.054, 0.179), (0.1713, 1.587, 0.243)))
_G23_UV_A = (0.81297, 0.2775, 1.06295, 0.11303, 4.60, 0.99)
_G23_UV_B = (-2.97868, 1.89808, 3.10334, 0.65484, 4.60, 0.99)


def _g23_ir_a(w):
    scale, a1, a2, sw, width, sil1, sil2 = _G23_IR
    pw1 = scale * w ** (-a1)
    pw2 = scale * (sw ** (-a1) / sw ** (-a2)) * w ** (-a2)
    t = _smooth(w, sw - width / 2, sw + width / 2)
    return pw1 * (1 - t) + pw2 * t + _drude_asym(w, *sil1) + _drude_asym(w, *sil2)


def _g23_opt(x, table):
    poly, drudes = table
    return _horner(x, list(poly)) + sum(_drude(x, *d) for d in drudes)


def gordon23(wave, Rv: float) -> np.ndarray:
    """A(x)/A(V) of Gordon et al. 2023 (extinction_models.py:255-398), ``wave`` in
    microns: NIR/MIR broken power law with silicate features, optical polynomial plus
    Drude profiles, FM90 in the UV, smoothstep blends across 0.9-1.1 and 0.3-0.33."""
    w = np.asarray(wave, dtype=np.float64)
    with np.errstate(all="ignore"):
        x = 1.0 / w
        ir_a, ir_b = _g23_ir_a(w), -1.01251 * w ** 1.06099
        op_a, op_b = _g23_opt(x, _G23_OPT_A), _g23_opt(x, _G23_OPT_B)
        uv_a, uv_b = _fm90(x, *_G23_UV_A), _fm90(x, *_G23_UV_B)
    a = np.zeros_like(w)
    b = np.zeros_like(w)
    ir = (w >= 1.0) & (w < 35.0)
    a, b = np.where(ir, ir_a, a), np.where(ir, ir_b, b)
    opt = (w >= 0.3) & (w < 1.1)
    a, b = np.where(opt, op_a, a), np.where(opt, op_b, b)
    t = _smooth(w, 0.9, 1.1)
    band = (w >= 0.9) & (w <= 1.1)
    a = np.where(band, (1 - t) * op_a + t * ir_a, a)
    b = np.where(band, (1 - t) * op_b + t * ir_b, b)
    uv = (w >= 0.09) & (w <= 0.3)
    a, b = np.where(uv, uv_a, a), np.where(uv, uv_b, b)
    t = _smooth(w, 0.3, 0.33)
    band = (w >= 0.3) & (w <= 0.33)
    a = np.where(band, (1 - t) * uv_a + t * op_a, a)
    b = np.where(band, (1 - t) * uv_b + t * op_b, b)
    return a + b * (1.0 / Rv - 1.0 / 3.1)


def axav(model: str, wave, Rv: float) -> np.ndarray:
    """A(x)/A(V) of rubix's model ``model`` at ``wave`` (microns)."""
    if model not in RV_MODELS:
        raise ValueError(f"Extinction model '{model}' is not available. Choose from {RV_MODELS}.")
    return cardelli89(wave, Rv) if model == "Cardelli89" else gordon23(wave, Rv)


def extinction_exponent(wave_t, model: str, Rv: float) -> np.ndarray:
    """float32 [L]: -0.4 log2(10) A(x)/A(V) at x = wave_t / 1e4 (rubix passes the
    telescope wavelengths in Angstrom divided by 1e4, dust_extinction.py:347-349)."""
    x = np.asarray(wave_t, dtype=np.float32) / np.float32(1e4)
    return (-0.4 * math.log2(10.0) * axav(model, x.astype(np.float64), Rv)).astype(np.float32)


def dust_to_gas_params(model: str, Xco: str):
    """(params [x_sol, a_hi, alpha_hi, a_lo, alpha_lo, x_transition], broken) of the
    dust-to-gas ratio 1 / 10^(a + alpha (x_sol - 12 - log(O/H))), Remy-Ruyer et al.
    2014 Table 1 as rubix tabulates it (dust_extinction.py:13-90)."""
    if model == "power law slope fixed":
        raise NotImplementedError("power law slope fixed not implemented yet.")
    x_sol = 8.69  # Asplund et al. 2009
    table = {
        ("power law slope free", "MW"): ((2.21, 1.62), None),
        ("power law slope free", "Z"): ((2.21, 2.02), None),
        ("broken power law fit", "MW"): ((2.21, 1.00), (0.68, 3.08, 7.96)),
        ("broken power law fit", "Z"): ((2.21, 1.00), (0.96, 3.10, 8.10)),
    }
    if (model, Xco) not in table:
        raise ValueError(f"unknown dust-to-gas model {model!r} / Xco {Xco!r}")
    (a, al), low = table[(model, Xco)]
    if low is None:
        return [x_sol, a, al, a, al, 0.0], False
    return [x_sol, a, al, low[0], low[1], low[2]], True


def extinction_scale(dust_grain_density: float) -> float:
    """3 pi (Msun/kpc^2 -> g/cm^2) / (0.4 ln10 lambda_V[cm] rho_D): A_V per unit dust
    surface density (dust_extinction.py:93-160)."""
    convert = _MSUN_G / _KPC_CM ** 2
    return 3.0 * math.pi * convert / (0.4 * math.log(10.0) * _LAMBDA_V_A * 1e-8
                                      * float(dust_grain_density))
