"""SSP templates and their lookup (rubix/core/ssp.py:12-98, spectra/ssp/grid.py:22-124).

rubix loads named templates from HDF5/FITS files (spectra/ssp/factory.py:13-76) that
are not shipped with this package; templates are registered here instead, either as
arrays (``register_ssp_template``) or from the seeded synthetic generator with the
name ``"synthetic"`` (parameters under ``config["ssp"]["template"]``).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Dict

import numpy as np
import torch

from .. import ops, synth
from ..logging import get_logger
from .data import device_of, flat_particles, like_input


@dataclass
class SSPGrid:
    """SSPGrid fields (spectra/ssp/grid.py:28-31): flux layout [metallicity, age, lambda]."""

    age: np.ndarray
    metallicity: np.ndarray
    wavelength: np.ndarray
    flux: np.ndarray

    def __post_init__(self):
        self.age = np.asarray(self.age, dtype=np.float32)
        self.metallicity = np.asarray(self.metallicity, dtype=np.float32)
        self.wavelength = np.asarray(self.wavelength, dtype=np.float32)
        self.flux = np.asarray(self.flux, dtype=np.float32)
        nz, na, nw = self.flux.shape
        if (nz, na, nw) != (self.metallicity.size, self.age.size, self.wavelength.size):
            raise ValueError("SSP flux must be [metallicity, age, wavelength]")

    def device_arrays(self, device):
        key = str(device)
        cache = self.__dict__.setdefault("_dev", {})
        if key not in cache:
            cache[key] = tuple(torch.from_numpy(a).to(device) for a in
                               (self.flux, self.metallicity, self.age, self.wavelength))
        return cache[key]

    def get_lookup_interpolation(self, method: str = "cubic", extrap: int = 0,
                                 device="cuda") -> Callable:
        """Lookup function f(metallicity, age) -> spectra (grid.py:61-124), bilinear only."""
        if method != "linear":
            raise ValueError(
                f"SSP interpolation method {method!r} is not available: rubix_gb300 "
                "implements method='linear' (bilinear in metallicity and age)")
        if extrap != 0:
            raise ValueError("only extrap=0 (zero outside the grid) is implemented")
        dev = torch.device(device)

        def lookup(metallicity, age):
            flux, zg, ag, _ = self.device_arrays(dev)
            z = flat_particles(metallicity, dev)
            a = flat_particles(age, dev)
            out = ops.ssp_lookup(flux, zg, ag, z, a)
            return out.reshape(tuple(np.shape(metallicity)) + (self.wavelength.size,))

        lookup.__doc__ = "Interpolation function for SSP grid, args: f(metallicity, age)"
        return lookup


_TEMPLATES: Dict[str, SSPGrid] = {}


def register_ssp_template(name: str, grid: SSPGrid) -> None:
    """Make ``grid`` available as ``config["ssp"]["template"]["name"] == name``."""
    if not isinstance(grid, SSPGrid):
        grid = SSPGrid(**grid) if isinstance(grid, dict) else grid
    _TEMPLATES[name] = grid


def get_ssp_template(name: str, params: dict | None = None) -> SSPGrid:
    if name in _TEMPLATES:
        return _TEMPLATES[name]
    if name == "synthetic":
        p = dict(n_age=20, n_met=6, n_wave=1000, seed=0)
        p.update({k: v for k, v in (params or {}).items() if k in p})
        s = synth.make_ssp(p["n_age"], p["n_met"], p["n_wave"], seed=p["seed"])
        return SSPGrid(age=s.age, metallicity=s.metallicity, wavelength=s.wavelength, flux=s.flux)
    raise ValueError(
        f"SSP template {name} is not available: register its grid with "
        "rubix_gb300.core.ssp.register_ssp_template (template files are not shipped)")


def get_ssp(config: dict) -> SSPGrid:
    """rubix/core/ssp.py:12-34 (same checks and messages)."""
    if "ssp" not in config:
        raise ValueError("Configuration does not contain 'ssp' field")
    if "template" not in config["ssp"]:
        raise ValueError("Configuration does not contain 'template' field")
    if "name" not in config["ssp"]["template"]:
        raise ValueError("Configuration does not contain 'name' field")
    return get_ssp_template(config["ssp"]["template"]["name"], config["ssp"]["template"])


def lookup_method(config: dict) -> str:
    """rubix/core/ssp.py:57-62: ``config["ssp"]["method"]``, rubix's default is "cubic"."""
    return config["ssp"].get("method", "cubic")


def get_lookup_interpolation(config: dict) -> Callable:
    """rubix/core/ssp.py:38-65."""
    logger = get_logger(config.get("logger", None))
    ssp = get_ssp(config)
    method = lookup_method(config)
    logger.debug("Using SSP interpolation method %s", method)
    return ssp.get_lookup_interpolation(method=method, device=device_of(config))


__all__ = ["SSPGrid", "register_ssp_template", "get_ssp", "get_ssp_template",
           "get_lookup_interpolation", "like_input"]
