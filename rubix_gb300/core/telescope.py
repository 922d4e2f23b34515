"""Telescope steps: spatial bin edges, spaxel assignment, aperture filter
(rubix/core/telescope.py:20-201)."""

from __future__ import annotations

from typing import Callable

import numpy as np
import torch

from .. import ops
from .. import telescope as tel
from ..logging import get_logger
from .data import RubixData, device_of, flat_particles, has_device_axis, to_device

_CUSTOM = {}


def register_telescope(name: str, params: dict) -> None:
    """Add a telescope entry (the keys of rubix/telescope/telescopes.yaml)."""
    _CUSTOM[name] = dict(params)


def get_telescope(config) -> tel.Telescope:
    """rubix/core/telescope.py:20-47."""
    name = config["telescope"]["name"]
    table = dict(tel.TELESCOPES)
    table.update(_CUSTOM)
    return tel.create_telescope(name, table)


def get_spatial_bin_edges(config: dict) -> np.ndarray:
    """rubix/core/telescope.py:50-77: float32 edges from the angular scale at dist_z."""
    logger = get_logger(config.get("logger", None))
    logger.info("Calculating spatial bin edges...")
    telescope = get_telescope(config)
    cosmo = config.get("cosmology", {}).get("name", "PLANCK15")
    edges, _ = tel.spatial_bin_edges(telescope.fov, telescope.sbin, config["galaxy"]["dist_z"],
                                     cosmo)
    return edges


def _component(rubixdata: RubixData, name: str):
    return getattr(rubixdata, name)


def get_spaxel_assignment(config: dict) -> Callable:
    """rubix/core/telescope.py:80-126 (square pixels only)."""
    logger = get_logger(config.get("logger", None))
    telescope = get_telescope(config)
    if telescope.pixel_type not in ["square"]:
        raise ValueError(f"Pixel type {telescope.pixel_type} not supported")
    edges_np = get_spatial_bin_edges(config)
    dev = device_of(config)

    def spaxel_assignment(rubixdata: RubixData) -> RubixData:
        logger.info("Assigning particles to spaxels...")
        edges = to_device(edges_np, dev)
        for comp in (rubixdata.stars, rubixdata.gas):
            if comp is None or comp.coords is None:
                continue
            coords = flat_particles(comp.coords, dev, width=3)
            idx = ops.spaxel_assign(coords, edges)
            comp.pixel_assignment = idx.unsqueeze(0) if has_device_axis(comp.coords, True) else idx
            comp.spatial_bin_edges = edges
        return rubixdata

    return spaxel_assignment


def get_filter_particles(config: dict) -> Callable:
    """rubix/core/telescope.py:129-201: particles outside the aperture get every
    non-coordinate, non-velocity field set to 0 and ``mask`` records who is inside."""
    logger = get_logger(config.get("logger", None))
    edges_np = get_spatial_bin_edges(config)
    dev = device_of(config)
    types = config.get("data", {}).get("args", {}).get("particle_type", ["stars"])

    def filter_particles(rubixdata: RubixData) -> RubixData:
        logger.info("Filtering particles outside the aperture...")
        edges = to_device(edges_np, dev)
        for name in ("stars", "gas"):
            comp = getattr(rubixdata, name)
            if name not in types or comp is None or comp.coords is None:
                continue
            coords = flat_particles(comp.coords, dev, width=3)
            mask = ops.aperture_mask(coords, edges)
            skip = ("coords", "velocity") + (("metals",) if name == "gas" else ())
            for attr, val in list(vars(comp).items()):
                if attr in skip or attr in ("mask", "spatial_bin_edges") or val is None:
                    continue
                if not isinstance(val, (np.ndarray, torch.Tensor)) or np.ndim(val) == 0:
                    continue
                t = to_device(val, dev, torch.float32 if _is_float(val) else None).clone()
                if t.dtype == torch.float32:
                    ops.mask_zero_(t, mask)
                else:
                    t = torch.where(_expand(mask, t), t, torch.zeros((), dtype=t.dtype, device=dev))
                setattr(comp, attr, t)
            comp.mask = mask.bool().unsqueeze(0) if has_device_axis(comp.coords, True) else mask.bool()
        return rubixdata

    return filter_particles


def _is_float(v) -> bool:
    dt = v.dtype
    return (dt.is_floating_point if isinstance(v, torch.Tensor) else np.issubdtype(dt, np.floating))


def _expand(mask: torch.Tensor, t: torch.Tensor) -> torch.Tensor:
    m = mask.bool().reshape(-1)
    if t.dim() >= 2 and t.shape[0] == 1 and t.shape[1] == m.numel():
        return m.view((1, -1) + (1,) * (t.dim() - 2))
    return m.view((-1,) + (1,) * (t.dim() - 1))
