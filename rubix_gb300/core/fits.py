"""Cube output: store_fits / load_fits (rubix/core/fits.py:13-115).

``store_fits`` writes the same two HDUs as rubix (a header-only primary HDU with the
run's configuration, then the cube as an IMAGE extension "DATA" holding datacube.T with
a celestial + wavelength WCS) to the same file name.  A cube on the GPU is put into the
FITS layout there (``rubix_fits_cube_layout``: transpose to [lambda][x][y] and
big-endian byte order in one pass at HBM speed) and downloaded once; the host only
writes bytes.  rubix reads configuration keys that come from its simulation loaders
(simulation name, galaxy id, snapshot, subset); missing ones are written as "unknown"
here, since particle data reaches this package without those loaders.
"""

from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from .. import fits as fitsio
from .. import ops
from ..logging import get_logger
from .telescope import get_telescope

__all__ = ["store_fits", "load_fits", "FitsCube", "cube_fits_bytes"]


def _get(config: dict, *path, default="unknown"):
    cur = config
    for p in path:
        if not isinstance(cur, dict) or p not in cur:
            return default
        cur = cur[p]
    return cur


def cube_fits_bytes(datacube) -> bytes:
    """The big-endian float32 bytes of ``datacube.T`` (FITS array order): on the GPU for
    CUDA tensors, with NumPy otherwise."""
    if isinstance(datacube, torch.Tensor) and datacube.is_cuda:
        return ops.fits_cube_layout(datacube).cpu().numpy().tobytes()
    a = np.asarray(datacube.cpu() if isinstance(datacube, torch.Tensor) else datacube,
                   dtype=np.float32)
    return np.ascontiguousarray(a.T).astype(">f4").tobytes()


def store_fits(config: dict, data, filepath: str) -> str:
    """rubix/core/fits.py:13-102.  Returns the file name written."""
    logger = get_logger(config.get("logger", None))
    cube_type = _get(config, "data", "args", "cube_type", default="stars")
    parttype = "gas" if cube_type == "gas" else "stars"
    datacube = getattr(data, parttype).datacube
    telescope = get_telescope(config)

    hdr = fitsio.Header()
    hdr["PIPELINE"] = _get(config, "pipeline", "name")
    hdr["DIST_z"] = _get(config, "galaxy", "dist_z")
    hdr["ROTATION"] = _get(config, "galaxy", "rotation", "type")
    sim = _get(config, "simulation", "name")
    hdr["SIM"] = sim
    galaxy_id = _get(config, "data", "load_galaxy_args", "id")
    snapshot = _get(config, "data", "args", "snapshot")
    hdr["GALAXYID"] = galaxy_id
    hdr["SNAPSHOT"] = snapshot
    subset = _get(config, "data", "subset", "use_subset")
    hdr["SUBSET"] = subset
    hdr["SSP"] = _get(config, "ssp", "template", "name")
    hdr["INSTR"] = _get(config, "telescope", "name")
    hdr["PSF"] = _get(config, "telescope", "psf", "name")
    hdr["PSF_SIZE"] = _get(config, "telescope", "psf", "size")
    hdr["PSFSIGMA"] = _get(config, "telescope", "psf", "sigma")
    hdr["LSF"] = _get(config, "telescope", "lsf", "sigma")
    s2n = _get(config, "telescope", "noise", "signal_to_noise")
    hdr["S_TO_N"] = s2n if s2n is not None else "None"
    hdr["N_DISTR"] = _get(config, "telescope", "noise", "noise_distribution")
    hdr["COSMO"] = _get(config, "cosmology", "name")

    shape = tuple(int(x) for x in datacube.shape)
    hdr1 = fitsio.Header()
    hdr1["EXTNAME"] = "DATA"
    hdr1["OBJECT"] = f"{sim} {galaxy_id}"
    hdr1["BUNIT"] = "erg/(s*cm^2*A)"
    hdr1["CRPIX1"] = (shape[0] - 1) / 2
    hdr1["CRPIX2"] = (shape[1] - 1) / 2
    hdr1["CD1_1"] = telescope.spatial_res / 3600
    hdr1["CD1_2"] = 0
    hdr1["CD2_1"] = 0
    hdr1["CD2_2"] = telescope.spatial_res / 3600
    hdr1["CUNIT1"] = "deg"
    hdr1["CUNIT2"] = "deg"
    hdr1["CTYPE1"] = "RA---TAN"
    hdr1["CTYPE2"] = "DEC--TAN"
    hdr1["CTYPE3"] = "AWAV"
    hdr1["CUNIT3"] = "Angstrom"
    hdr1["CD3_3"] = telescope.wave_res
    hdr1["CRPIX3"] = 1
    hdr1["CRVAL3"] = telescope.wave_range[0]
    hdr1["CD1_3"] = 0
    hdr1["CD2_3"] = 0
    hdr1["CD3_1"] = 0
    hdr1["CD3_2"] = 0
    hdr1["BITPIX"] = -32
    hdr1["NAXIS"] = len(shape)
    for i, n in enumerate(shape):  # datacube.T: NAXIS1 is the cube's first axis
        hdr1[f"NAXIS{i + 1}"] = n

    out = (f"{filepath}{sim}_id{galaxy_id}_snap{snapshot}_{parttype}_subset{subset}.fits")
    d = os.path.dirname(out)
    if d:
        os.makedirs(d, exist_ok=True)
    fitsio.write_fits(out, [fitsio.HDU(hdr), fitsio.HDU(hdr1, raw=cube_fits_bytes(datacube))])
    logger.info(f"Datacube saved to {out}")
    return out


@dataclass
class FitsCube:
    """A cube read back from ``store_fits``'s layout: ``data`` [lambda, y, x] as in the
    file (the transpose of rubix's datacube), the wavelength axis from the WCS."""

    data: np.ndarray
    header: fitsio.Header
    primary_header: fitsio.Header
    wave: Optional[np.ndarray] = None

    @property
    def datacube(self) -> np.ndarray:
        """The cube in rubix's layout [x, y, lambda] (datacube = data.T)."""
        return self.data.T


def load_fits(filepath: str) -> FitsCube:
    """rubix/core/fits.py:105-115 (which returns an mpdaf Cube; mpdaf is not a
    dependency): the DATA extension, its header and the primary header."""
    hdus = fitsio.read_fits(filepath)
    ext = next((h for h in hdus[1:] if h.header.get("EXTNAME") == "DATA"),
               hdus[1] if len(hdus) > 1 else hdus[0])
    h = ext.header
    wave = None
    if "CRVAL3" in h and ext.data is not None:
        n = ext.data.shape[0]
        wave = h["CRVAL3"] + h.get("CD3_3", h.get("CDELT3", 1.0)) * (
            np.arange(n) + 1 - h.get("CRPIX3", 1))
    return FitsCube(data=ext.data, header=h, primary_header=hdus[0].header, wave=wave)
