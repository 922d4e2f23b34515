"""Telescope description, spatial/spectral grids and the PSF/LSF taps (host side).

Mirrors rubix's telescope factory (rubix/telescope/factory.py:38-100, base.py:10-39)
with the telescope table of rubix/telescope/telescopes.yaml held as a Python dict
(PyYAML is not a dependency).  All grids are built once on the host in float32 with
the reference's arithmetic and then uploaded; the kernels receive them as arrays.
"""

from __future__ import annotations

import functools
import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

# rubix/telescope/telescopes.yaml (the same entries and values)
TELESCOPES = {
    "MUSE": dict(fov=5.0, spatial_res=0.2, wave_range=[4700.15, 9351.4], wave_res=1.25,
                 lsf_fwhm=2.51, signal_to_noise=None, aperture_type="square",
                 pixel_type="square"),
    "NIRSpec_PRISM_CLEAR": dict(fov=3.0, spatial_res=0.1, wave_range=[6000, 53000],
                                wave_res=114.36, lsf_fwhm=471.00, signal_to_noise=None,
                                aperture_type="square", pixel_type="square"),
    "NIRSpec_G140M_F070LP": dict(fov=3.0, spatial_res=0.1, wave_range=[7000, 12600],
                                 wave_res=6.38, lsf_fwhm=15.02, signal_to_noise=None,
                                 aperture_type="square", pixel_type="square"),
    "NIRSpec_G140M_F100LP": dict(fov=3.0, spatial_res=0.1, wave_range=[9800, 18800],
                                 wave_res=6.38, lsf_fwhm=15.02, signal_to_noise=None,
                                 aperture_type="square", pixel_type="square"),
}


@dataclass
class Telescope:
    """BaseTelescope fields (rubix/telescope/base.py:10-39)."""

    name: str
    fov: float
    spatial_res: float
    wave_range: list
    wave_res: float
    lsf_fwhm: float
    signal_to_noise: Optional[float]
    sbin: int
    pixel_type: str
    aperture_type: str
    wave_seq: np.ndarray = field(repr=False)
    wave_edges: np.ndarray = field(repr=False)


def calculate_wave_seq(wave_range, wave_res) -> np.ndarray:
    """float32 ``arange(wave_range[0], wave_range[1], wave_res)`` (telescope/utils.py:42-53)."""
    return np.arange(wave_range[0], wave_range[1], wave_res, dtype=np.float32)


def calculate_wave_edges(wave_seq, wave_res) -> np.ndarray:
    """telescope/utils.py:56-74."""
    start = wave_seq[0] - wave_res / 2
    end = wave_seq[-1] + wave_res / 2
    return np.arange(start, end, wave_res, dtype=np.float32)


def create_telescope(name: str, telescopes_config: Optional[dict] = None) -> Telescope:
    """TelescopeFactory.create_telescope (rubix/telescope/factory.py:38-100)."""
    table = TELESCOPES if telescopes_config is None else telescopes_config
    if name not in table:
        raise ValueError(f"Telescope {name} not found in config")
    c = table[name]
    sbin = int(np.floor(c["fov"] / c["spatial_res"]))
    if c["aperture_type"] not in ("square", "circular", "hexagonal"):
        raise ValueError(f"Unknown aperture type: {c['aperture_type']}")
    ws, we = _wave_grids(tuple(float(x) for x in c["wave_range"]), float(c["wave_res"]))
    return Telescope(
        name=name, fov=c["fov"], spatial_res=c["spatial_res"], wave_range=list(c["wave_range"]),
        wave_res=c["wave_res"], lsf_fwhm=c["lsf_fwhm"], signal_to_noise=c["signal_to_noise"],
        sbin=sbin, pixel_type=c["pixel_type"], aperture_type=c["aperture_type"],
        wave_seq=ws, wave_edges=we,
    )


@functools.lru_cache(maxsize=64)
def _wave_grids(wave_range: tuple, wave_res: float):
    """wave_seq and wave_edges of a telescope, computed once per (range, resolution)
    and shared read-only (every pipeline step builds the telescope)."""
    ws = calculate_wave_seq(wave_range, wave_res)
    we = calculate_wave_edges(ws, wave_res)
    ws.flags.writeable = False
    we.flags.writeable = False
    return ws, we


# ------------------------------------------------------------------ cosmology
PLANCK15 = dict(Om0=0.3075, w0=-1.0, wa=0.0, h=0.6774)  # rubix/cosmology/__init__.py:3
COSMOLOGIES = {"PLANCK15": PLANCK15}


@functools.lru_cache(maxsize=64)
def angular_scale(z: float, Om0=0.3075, w0=-1.0, wa=0.0, h=0.6774) -> np.float32:
    """kpc per arcsec at redshift z for flat wCDM (rubix/cosmology/base.py:121-139, 290-314):
    comoving distance by the trapezoid rule on 256 nodes of [0, z]."""
    ztab = np.linspace(0.0, float(z), 256)
    a = 1.0 / (1.0 + ztab)
    rho_de = a ** (-3.0 * (1.0 + w0 + wa)) * np.exp(-3.0 * wa * (1.0 - a))
    inv_e = 1.0 / np.sqrt(Om0 * (1.0 + ztab) ** 3 + (1.0 - Om0) * rho_de)
    dc = float(np.sum(np.diff(ztab) * (inv_e[1:] + inv_e[:-1]) * 0.5)) * 2.99792458e8 * 1e-5 / h
    da = dc / (1.0 + z)
    return np.float32(da * (math.pi / (180 * 60 * 60)) * 1e3)


def spatial_bin_edges(fov, sbin, dist_z, cosmology="PLANCK15"):
    """calculate_spatial_bin_edges (rubix/telescope/utils.py:12-37) with float32 scalars.

    Returns (edges float32 [nb+1], bin size).  The float arange may give sbin+1 or
    sbin+2 edges, exactly as in the reference.
    """
    cos = COSMOLOGIES[cosmology] if isinstance(cosmology, str) else cosmology
    ang = angular_scale(dist_z, **cos)
    aperture = np.float32(ang * np.float32(fov))
    bin_size = np.float32(aperture / np.float32(sbin))
    start = np.float32(-aperture / np.float32(2))
    stop = np.float32(aperture / np.float32(2) + bin_size)
    return np.arange(start, stop, bin_size, dtype=np.float32), bin_size


# ------------------------------------------------------------------ PSF / LSF taps
def gaussian_kernel_2d(m: int, n: int, sigma: float) -> np.ndarray:
    """rubix/telescope/psf/kernels.py:5-31 (float64)."""
    x = np.arange(-((m - 1) / 2), ((m - 1) / 2) + 1)
    y = np.arange(-((n - 1) / 2), ((n - 1) / 2) + 1)
    X, Y = np.meshgrid(x, y, indexing="ij")
    v = np.exp(-(X**2 + Y**2) / (2 * sigma**2))
    return v / np.sum(v)


def gaussian_taps_1d(m: int, sigma: float) -> np.ndarray:
    """Normalised 1-D Gaussian whose outer product with itself is gaussian_kernel_2d(m, m)."""
    x = np.arange(-((m - 1) / 2), ((m - 1) / 2) + 1)
    g = np.exp(-(x**2) / (2 * sigma**2))
    return g / np.sum(g)


def lsf_taps(sigma: float, wave_res: float, factor: int = 12) -> np.ndarray:
    """rubix/telescope/lsf/lsf.py:12-26: taps at the float32 grid arange(-f*d, f*d+d, d)."""
    x = np.arange(-factor * wave_res, factor * wave_res + wave_res, wave_res, dtype=np.float32)
    x = x.astype(np.float64)
    g = np.exp(-0.5 * x**2 / sigma**2)
    return g / np.sum(g)


def cosmological_doppler_shift(z: float, wavelength) -> np.ndarray:
    """float32 ``(1+z) * wavelength`` (rubix/spectra/ifu.py:66-80, core/ifu.py:261)."""
    return (np.float32(1.0 + z) * np.asarray(wavelength, dtype=np.float32)).astype(np.float32)
