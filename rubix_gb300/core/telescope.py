"""Telescope steps: spatial bin edges, spaxel assignment, aperture filter
(rubix/core/telescope.py:20-201)."""

from __future__ import annotations

from typing import Callable, Optional

import numpy as np
import torch

from .. import ops
from .. import telescope as tel
from ..logging import get_logger
from .data import RubixData, device_constant, device_of, flat_particles, has_device_axis, to_device

_CUSTOM = {}


def register_telescope(name: str, params: dict) -> None:
    """Add a telescope entry (the keys of rubix/telescope/telescopes.yaml)."""
    _CUSTOM[name] = dict(params)


def register_telescopes_file(path: str) -> list:
    """Register every telescope of a file in the layout of rubix's telescopes.yaml
    (TelescopeFactory(telescopes_config=path), telescope/factory.py:28-36); returns the
    names."""
    from .. import yaml_subset

    table = yaml_subset.load_file(path)
    if not isinstance(table, dict):
        raise ValueError(f"{path}: expected a mapping of telescope names to parameters")
    for name, params in table.items():
        register_telescope(name, params)
    return list(table)


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


class FrameHandoff:
    """Links rotate_galaxy, filter_particles and spaxel_assignment of one pipeline run
    when they run back to back (calc_ifu's order).  rotate_galaxy derives each
    component's rotation matrix (``matrix``: name -> (M, device coords, device
    velocity)), filter_particles records which components it filters (``filter``), and
    spaxel_assignment turns, filters and assigns the particles in one pass
    (``rubix_orient_filter_assign``) instead of a launch per array."""

    def __init__(self, rotation: bool = True):
        self.rotation = rotation  # rotate_galaxy defers to spaxel_assignment
        self.matrix: dict = {}
        self.filter = None


def frame_fusion(step_names):
    """A FrameHandoff for a run whose filter_particles is directly followed by
    spaxel_assignment (with rotate_galaxy directly before them, the rotation joins the
    pass as well); None otherwise."""
    names = list(step_names)
    for i in range(len(names) - 1):
        if names[i] == "filter_particles" and names[i + 1] == "spaxel_assignment":
            return FrameHandoff(rotation=i > 0 and names[i - 1] == "rotate_galaxy")
    return None


def _filter_targets(comp, name: str):
    """The arrays filter_particles zeroes outside the aperture: every per-particle array
    but coords, velocity (and the gas metals), as (attr, value) pairs."""
    skip = ("coords", "velocity") + (("metals",) if name == "gas" else ())
    out = []
    for attr, val in list(vars(comp).items()):
        if attr in skip or attr in ("mask", "spatial_bin_edges") or val is None:
            continue
        if not isinstance(val, (np.ndarray, torch.Tensor)) or np.ndim(val) == 0:
            continue
        out.append((attr, val))
    return out


def _masked_copy(val, mask, dev):
    t = to_device(val, dev, torch.float32 if _is_float(val) else None).clone()
    if t.dtype == torch.float32:
        return ops.mask_zero_(t, mask)
    return torch.where(_expand(mask, t), t, torch.zeros((), dtype=t.dtype, device=dev))


def _fused_frame(rubixdata: RubixData, handoff: FrameHandoff, edges, dev) -> None:
    """The deferred rotation and filter of each component with the assignment, in one
    rubix_orient_filter_assign launch per component."""
    for name in ("stars", "gas"):
        comp = getattr(rubixdata, name)
        if comp is None or comp.coords is None:
            continue
        pend = handoff.matrix.pop(name, None)
        if pend is not None:
            M, coords, vel = pend
        else:
            M, coords, vel = None, to_device(comp.coords, dev), None
        filt = handoff.filter is not None and name in handoff.filter
        fields, attrs, others = [], [], []
        if filt:
            for attr, val in _filter_targets(comp, name):
                if _is_float(val) and len(fields) < 8:
                    fields.append(to_device(val, dev, torch.float32))
                    attrs.append(attr)
                else:
                    others.append((attr, val))
        co, vo, outs, mask, idx = ops.orient_filter_assign(
            coords.reshape(-1, 3), None if vel is None else vel.reshape(-1, 3), M, edges,
            fields, mask=filt)
        axis = has_device_axis(comp.coords, True)
        if M is not None:
            comp.coords = co.reshape(coords.shape)
            comp.velocity = vo.reshape(vel.shape)
        if filt:
            for attr, o in zip(attrs, outs):
                setattr(comp, attr, o)
            for attr, val in others:
                setattr(comp, attr, _masked_copy(val, mask, dev))
            comp.mask = mask.bool().unsqueeze(0) if axis else mask.bool()
        comp.pixel_assignment = idx.unsqueeze(0) if axis else idx
        comp.spatial_bin_edges = edges
    handoff.filter = None


def get_spaxel_assignment(config: dict, handoff: Optional[FrameHandoff] = None) -> Callable:
    """rubix/core/telescope.py:80-126 (square pixels only).  With ``handoff`` the
    rotation and filter deferred by the two steps before run in the same launch."""
    logger = get_logger(config.get("logger", None))
    telescope = get_telescope(config)
    if telescope.pixel_type not in ["square"]:
        raise ValueError(f"Pixel type {telescope.pixel_type} not supported")
    edges_np = get_spatial_bin_edges(config)
    dev = device_of(config)

    def spaxel_assignment(rubixdata: RubixData) -> RubixData:
        logger.info("Assigning particles to spaxels...")
        edges = device_constant(edges_np, dev)
        if handoff is not None and (handoff.filter is not None or handoff.matrix):
            _fused_frame(rubixdata, handoff, edges, dev)
            return rubixdata
        for comp in (rubixdata.stars, rubixdata.gas):
            if comp is None or comp.coords is None:
                continue
            coords = flat_particles(comp.coords, dev, width=3)
            idx = ops.spaxel_assign(coords, edges)
            comp.pixel_assignment = idx.unsqueeze(0) if has_device_axis(comp.coords, True) else idx
            comp.spatial_bin_edges = edges
        return rubixdata

    return spaxel_assignment


def get_filter_particles(config: dict, handoff: Optional[FrameHandoff] = None) -> Callable:
    """rubix/core/telescope.py:129-201: particles outside the aperture get every
    non-coordinate, non-velocity field set to 0 and ``mask`` records who is inside.
    With ``handoff`` the filter is left to the spaxel_assignment that follows."""
    logger = get_logger(config.get("logger", None))
    edges_np = get_spatial_bin_edges(config)
    dev = device_of(config)
    types = config.get("data", {}).get("args", {}).get("particle_type", ["stars"])

    def filter_particles(rubixdata: RubixData) -> RubixData:
        logger.info("Filtering particles outside the aperture...")
        if handoff is not None:
            handoff.filter = tuple(types)
            return rubixdata
        edges = device_constant(edges_np, dev)
        for name in ("stars", "gas"):
            comp = getattr(rubixdata, name)
            if name not in types or comp is None or comp.coords is None:
                continue
            coords = flat_particles(comp.coords, dev, width=3)
            mask = ops.aperture_mask(coords, edges)
            for attr, val in _filter_targets(comp, name):
                setattr(comp, attr, _masked_copy(val, mask, dev))
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
