"""Data containers passed between pipeline steps (rubix/core/data.py:68-355).

The fields match rubix's ``Galaxy``, ``StarsData``, ``GasData`` and ``RubixData``.  Arrays
may be NumPy arrays or torch tensors; steps move what they need to the GPU once and
store CUDA tensors back.  ``stars.spectra`` can hold a ``ParticleSpectra`` — the lazy
stand-in for rubix's N x lambda arrays (see ``rubix_gb300.core.ifu``).
"""

from __future__ import annotations

from dataclasses import dataclass, fields
from typing import Any, Optional

import numpy as np
import torch

from ..logging import get_logger


@dataclass
class Galaxy:
    redshift: Optional[Any] = None
    center: Optional[Any] = None
    halfmassrad_stars: Optional[Any] = None


@dataclass
class StarsData:
    coords: Optional[Any] = None
    velocity: Optional[Any] = None
    mass: Optional[Any] = None
    metallicity: Optional[Any] = None
    age: Optional[Any] = None
    pixel_assignment: Optional[Any] = None
    spatial_bin_edges: Optional[Any] = None
    mask: Optional[Any] = None
    spectra: Optional[Any] = None
    datacube: Optional[Any] = None


@dataclass
class GasData:
    coords: Optional[Any] = None
    velocity: Optional[Any] = None
    mass: Optional[Any] = None
    density: Optional[Any] = None
    internal_energy: Optional[Any] = None
    metallicity: Optional[Any] = None
    metals: Optional[Any] = None
    sfr: Optional[Any] = None
    electron_abundance: Optional[Any] = None
    pixel_assignment: Optional[Any] = None
    spatial_bin_edges: Optional[Any] = None
    mask: Optional[Any] = None
    spectra: Optional[Any] = None
    datacube: Optional[Any] = None


@dataclass
class RubixData:
    galaxy: Optional[Galaxy] = None
    stars: Optional[StarsData] = None
    gas: Optional[GasData] = None

    def __post_init__(self):
        if self.galaxy is None:
            self.galaxy = Galaxy()
        if self.stars is None:
            self.stars = StarsData()
        if self.gas is None:
            self.gas = GasData()


def device_of(config: Optional[dict] = None) -> torch.device:
    """The CUDA device the steps run on (config["device"], default cuda:current)."""
    dev = (config or {}).get("device", "cuda")
    d = torch.device(dev)
    if d.type != "cuda":
        raise ValueError("rubix_gb300 steps run on a CUDA device only")
    return d


def to_device(x, device, dtype=torch.float32) -> torch.Tensor:
    """NumPy array / tensor -> contiguous CUDA tensor of ``dtype``."""
    if isinstance(x, torch.Tensor):
        t = x
    else:
        a = np.ascontiguousarray(np.asarray(x))
        if not a.flags.writeable:  # shared read-only constants: torch wants its own copy
            a = a.copy()
        t = torch.from_numpy(a)
    if dtype is not None and t.dtype != dtype:
        # a bool mask is read as uint8 without a copy (same one-byte storage)
        t = t.view(dtype) if (t.dtype == torch.bool and dtype == torch.uint8) else t.to(dtype)
    if t.device != device:
        t = t.to(device)
    return t.contiguous()


_CONSTANTS: dict = {}


def device_constant(x, device, dtype=torch.float32) -> torch.Tensor:
    """A host constant of the configuration (bin edges, wavelength grids, extinction
    exponents) on the device, uploaded once per (contents, device, dtype).  A copy from
    pageable host memory waits for the stream's queued work, so steps that uploaded their
    constants on every call kept the host from running ahead of the GPU.  The tensors
    are shared: callers must not write to them."""
    a = np.ascontiguousarray(np.asarray(x))
    key = (a.dtype.str, a.shape, a.tobytes(), str(torch.device(device)), str(dtype))
    t = _CONSTANTS.get(key)
    if t is None:
        if len(_CONSTANTS) >= 256:
            _CONSTANTS.clear()
        t = to_device(a, device, dtype)
        _CONSTANTS[key] = t
    return t


_VECTOR_FIELDS = ("coords", "velocity")


def has_device_axis(x, vector: bool = False) -> bool:
    """True if a per-particle array carries rubix's leading device axis:
    scalar fields (N,) -> (1, N), vector fields (N, 3) -> (1, N, 3)."""
    return getattr(x, "ndim", 0) == (3 if vector else 2)


def flat_particles(x, device, dtype=torch.float32, width=None) -> torch.Tensor:
    """Per-particle array (N,), (1, N), (N, w) or (1, N, w) -> CUDA tensor (N,) / (N, w)."""
    t = to_device(x, device, dtype)
    if width is None:
        return t.reshape(-1)
    return t.reshape(-1, width)


def like_input(t: torch.Tensor, ref_scalar_field) -> torch.Tensor:
    """Give ``t`` (N, ...) a leading device axis if the scalar field ``ref`` has one."""
    return t.unsqueeze(0) if has_device_axis(ref_scalar_field) else t


def reshape_array(arr):
    """rubix/core/data.py:447-487 with one device per process: (N, ...) -> (1, N, ...).

    rubix pads to a multiple of ``jax.device_count()``; a rubix_gb300 process drives one
    GPU, so the device axis has length 1 and no padding is needed.
    """
    if isinstance(arr, torch.Tensor):
        return arr.unsqueeze(0)
    return np.asarray(arr)[None, ...]


_PER_PARTICLE = ("coords", "velocity", "mass", "metallicity", "age", "pixel_assignment",
                 "mask")


def get_reshape_data(config) -> Any:
    """rubix/core/data.py:639-671: returns the ``reshape_data`` step."""
    logger = get_logger(config.get("logger", None) if isinstance(config, dict) else None)

    def reshape_data(rubixdata: RubixData) -> RubixData:
        for comp in (rubixdata.stars, rubixdata.gas):
            if comp is None or comp.coords is None:
                continue
            for f in fields(comp):
                v = getattr(comp, f.name)
                if f.name not in _PER_PARTICLE:
                    continue
                if v is None:
                    logger.debug("Attribute value of %s is None", f.name)
                elif not has_device_axis(v, vector=f.name in _VECTOR_FIELDS):
                    setattr(comp, f.name, reshape_array(v))
        return rubixdata

    return reshape_data
