"""Dust extinction step: get_extinction / calculate_extinction (rubix/core/dust.py:16-65)
and apply_spaxel_extinction (rubix/spectra/dust/dust_extinction.py:169-358).

The step computes every star's A_V from the gas in front of it on the GPU
(``rubix_dust_gas_extinction`` + ``rubix_dust_av``) and the model's curve on the host.
With lazy spectra (the fused path) it records A_V and the curve in the
``ParticleSpectra`` so that ``calculate_datacube`` applies the transmission inside the
accumulate kernel; materialised spectra are multiplied in place by a kernel.
"""

from __future__ import annotations

import dataclasses
from typing import Callable

import numpy as np
import torch

from .. import dust as dust_host
from .. import ops
from .. import telescope as tel
from ..logging import get_logger
from .config import rubix_config
from .data import RubixData, device_constant, device_of, flat_particles, to_device
from .ifu import ParticleSpectra, _spectra_tensor
from .telescope import get_spatial_bin_edges, get_telescope

__all__ = ["get_extinction", "apply_spaxel_extinction", "star_av"]


def _spaxel_area(config: dict) -> float:
    telescope = get_telescope(config)
    cosmo = config.get("cosmology", {}).get("name", "PLANCK15")
    _, size = tel.spatial_bin_edges(telescope.fov, telescope.sbin, config["galaxy"]["dist_z"],
                                    cosmo)
    return float(np.float32(size) ** 2)


def star_av(config: dict, rubixdata: RubixData, n_spaxels: int, spaxel_area: float,
            pa_limit: int = None) -> torch.Tensor:
    """A_V [N] of every star (dust_extinction.py:262-343): per-cell extinction of the gas
    (dust mass from 12 + log(O/H) through the dust-to-gas ratio, over the spaxel area),
    cumulated along z within each spaxel and interpolated at the stars' z."""
    dev = device_of(config)
    gas, st = rubixdata.gas, rubixdata.stars
    if gas is None or gas.coords is None or gas.pixel_assignment is None or gas.mass is None \
            or gas.metals is None:
        raise ValueError("dust extinction needs gas coords, pixel_assignment, mass and metals "
                         "(run spaxel_assignment on the gas first)")
    d = rubix_config["ssp"]["dust"]
    params, broken = dust_host.dust_to_gas_params(d["dust_to_gas_model"], d["Xco"])
    grain = config["ssp"]["dust"].get("dust_grain_density", d["dust_grain_density"])
    gmass = flat_particles(gas.mass, dev)
    metals = to_device(gas.metals, dev).reshape(gmass.numel(), -1)
    gext = ops.dust_gas_extinction(gmass, metals, params, broken,
                                   dust_host.extinction_scale(grain), spaxel_area)
    gcoords = flat_particles(gas.coords, dev, width=3)
    gpa = flat_particles(gas.pixel_assignment, dev, dtype=torch.int32)
    scoords = flat_particles(st.coords, dev, width=3)
    spa = flat_particles(st.pixel_assignment, dev, dtype=torch.int32)
    if pa_limit is None:
        nb = len(get_spatial_bin_edges(config)) - 1
        pa_limit = max(nb * nb, n_spaxels)
    return ops.dust_av(gcoords, gpa, gext, scoords, spa, n_spaxels, pa_limit)


def apply_spaxel_extinction(config: dict, rubixdata: RubixData, wavelength, n_spaxels: int,
                            spaxel_area):
    """dust_extinction.py:169-358: the stars' spectra times their dust transmission.

    Returns the new ``stars.spectra``: a lazy ``ParticleSpectra`` carrying A_V and the
    curve (applied by the fused cube kernel), or the materialised spectra multiplied
    in place."""
    logger = get_logger(config.get("logger", None))
    logger.info("Applying dust extinction to the spaxel data using vmap...")
    ext_model = config["ssp"]["dust"]["extinction_model"]
    Rv = config["ssp"]["dust"]["Rv"]
    if ext_model not in dust_host.RV_MODELS:
        raise ValueError(
            f"Extinction model '{ext_model}' is not available. Choose from "
            f"{dust_host.RV_MODELS}.")
    dev = device_of(config)
    av = star_av(config, rubixdata, n_spaxels, float(np.asarray(spaxel_area)))
    exponent = device_constant(
        dust_host.extinction_exponent(np.asarray(wavelength), ext_model, Rv), dev)
    spec = rubixdata.stars.spectra
    if isinstance(spec, ParticleSpectra) and spec.stage == "resampled":
        return dataclasses.replace(spec, dust_av=av, dust_exponent=exponent)
    rows = _spectra_tensor(spec, dev)
    if isinstance(spec, torch.Tensor) and rows.data_ptr() == spec.data_ptr():
        rows = rows.clone()
    ops.dust_apply_rows_(rows, av, exponent)
    return rows.reshape(tuple(np.shape(spec)))


def get_extinction(config: dict) -> Callable:
    """rubix/core/dust.py:16-65: the ``calculate_extinction`` step."""
    logger = get_logger(config.get("logger", None))
    if "dust" not in config["ssp"]:
        raise ValueError("Dust configuration not found in config file.")
    if "extinction_model" not in config["ssp"]["dust"]:
        raise ValueError("Extinction model not found in dust configuration.")
    telescope = get_telescope(config)
    n_spaxels = int(telescope.sbin ** 2)
    wavelength = telescope.wave_seq
    spaxel_area = _spaxel_area(config)

    def calculate_extinction(rubixdata: RubixData) -> RubixData:
        logger.info("Applying dust extinction to the spaxel data...")
        rubixdata.stars.spectra = apply_spaxel_extinction(config, rubixdata, wavelength,
                                                          n_spaxels, spaxel_area)
        return rubixdata

    return calculate_extinction
