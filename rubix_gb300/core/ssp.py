"""SSP templates and their lookup (rubix/core/ssp.py:12-98, spectra/ssp/grid.py:22-124).

rubix loads named templates from HDF5/FITS files (spectra/ssp/factory.py:13-76).  Here a
template is, in order: a grid registered as arrays (``register_ssp_template``); the
seeded synthetic generator (name ``"synthetic"``, parameters under
``config["ssp"]["template"]``); or one of rubix's named templates read from its file in
the template directory (``RUBIX_GB300_TEMPLATE_PATH``, default ``templates/`` next to
this package).  Files in rubix's pyPipe3D FITS format (MaStar, .fits or .fits.gz) are
read with the package's own FITS reader, HDF5 templates (BC03, FSPS) with its own HDF5
reader (``rubix_gb300.hdf5``).  Nothing is downloaded.
"""

from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Callable, Dict

import numpy as np
import torch

from .. import fits as fitsio
from .. import hdf5
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

# rubix/config/rubix_config.yml:136-240: the units the SSP grid is held in, and the
# named templates with their file formats and field units
SSP_UNITS = {"age": "Gyr", "metallicity": "", "wavelength": "Angstrom",
             "flux": "Lsun/Angstrom"}
_FIELDS = {k: {"name": k, "units": u, "in_log": False} for k, u in SSP_UNITS.items()}
SSP_TEMPLATES = {
    "BruzualCharlot2003": {"name": "Bruzual & Charlot (2003)", "format": "HDF5",
                           "file_name": "BC03lr.h5", "fields": _FIELDS},
    "Mastar_CB19_SLOG_1_5": {"name": "Mastar Charlot & Bruzual (2019)", "format": "PyPipe3D",
                             "file_name": "MaStar_CB19.slog_1_5.fits.gz", "fields": _FIELDS},
    "FSPS": {"name": "FSPS (Conroy et al. 2009)", "format": "fsps", "file_name": "fsps.h5",
             "fields": dict(_FIELDS, age={"name": "age", "units": "Gyr", "in_log": True},
                            metallicity={"name": "metallicity", "units": "",
                                         "in_log": True})},
}

# unit factors to the internal units (the conversions rubix does with astropy units)
_UNIT_FACTORS = {
    "age": {"Gyr": 1.0, "Myr": 1e-3, "kyr": 1e-6, "yr": 1e-9},
    "metallicity": {"": 1.0},
    "wavelength": {"Angstrom": 1.0, "nm": 10.0, "um": 1e4, "micron": 1e4, "cm": 1e8, "m": 1e10},
    "flux": {"Lsun/Angstrom": 1.0, "erg/s/Angstrom": 1.0 / 3.828e33,
             "Lsun/nm": 0.1, "Lsun/um": 1e-4},
}


def template_path() -> str:
    return os.environ.get("RUBIX_GB300_TEMPLATE_PATH",
                          os.path.join(os.path.dirname(os.path.dirname(__file__)), "templates"))


def convert_units(data, field: str, from_units: str) -> np.ndarray:
    """grid.py:128-149 for the units of ``_UNIT_FACTORS`` (float32 result)."""
    table = _UNIT_FACTORS[field]
    if from_units not in table:
        raise ValueError(f"cannot convert {field} from units {from_units!r} "
                         f"(known: {sorted(table)})")
    return (np.asarray(data, dtype=np.float64) * table[from_units]).astype(np.float32)


def _pypipe3d_models(header, n_models: int):
    """grid.py:466-515: ages (Gyr), metallicities and mass-to-light of each model from
    the NAME<i> ("..._<age>[Gyr|Myr]_z<digits>...") and NORM<i> cards."""
    ages = np.zeros(n_models, np.float32)
    Zs = np.zeros(n_models, np.float32)
    mtol = np.ones(n_models, np.float32)
    for i in range(n_models):
        parts = str(header[f"NAME{i}"]).split("_")[2:]
        tok = parts[0]
        mult = 1.0
        if "yr" in tok:
            mult = {"Gyr": 1.0, "Myr": 1.0 / 1000}[tok[-3:]]
            tok = tok[:-3]
        ages[i] = np.float32(mult * np.float32(tok))
        Zs[i] = np.float32(parts[1].split(".")[0].replace("z", "0."))
        norm = np.float32(header[f"NORM{i}"])
        mtol[i] = np.float32(1) / norm if norm != 0 else np.float32(1)
    return np.unique(ages), np.unique(Zs), mtol


def load_pypipe3d(path: str, fields: dict = None) -> SSPGrid:
    """pyPipe3DSSPGrid.from_file (grid.py:518-581): models along NAXIS2 (metallicity
    major, then age), wavelengths CRVAL1 + CDELT1 (i + 1 - CRPIX1), flux divided by
    each model's mass-to-light ratio, fields converted to the internal units."""
    hdu = fitsio.read_fits(path)[0]
    h = hdu.header
    n_models = int(h["NAXIS2"])
    ages, mets, m2l = _pypipe3d_models(h, n_models)
    cdelt = h.get("CDELT1", 1) or 1
    wave = (h["CRVAL1"] + cdelt * (np.arange(int(h["NAXIS1"])) + 1 - h["CRPIX1"]))
    flux = (np.asarray(hdu.data, np.float32) / m2l[:, None]).astype(np.float32)
    flux = flux.reshape(len(mets), len(ages), len(wave))
    raw = {"flux": flux, "wavelength": wave, "age": ages, "metallicity": mets}
    out = {}
    for name, info in (fields or _FIELDS).items():
        if name not in raw:
            raise ValueError(f"Field {name} not recognized")
        d = raw[name]
        if info.get("in_log"):
            d = np.power(10.0, np.asarray(d, np.float64))
        out[name] = convert_units(d, name, info.get("units", SSP_UNITS[name]))
    return SSPGrid(**out)


def load_hdf5_template(path: str, fields: dict = None) -> SSPGrid:
    """HDF5SSPGrid.from_file (grid.py:304-335): dataset ``fields[f]["name"]`` of each
    field, 10**data when ``in_log``, float32, converted to the internal units."""
    out = {}
    with hdf5.File(path, "r") as f:
        for name, info in (fields or _FIELDS).items():
            d = np.asarray(f[info["name"]][()], dtype=np.float64)
            if info.get("in_log"):
                d = np.power(10.0, d)
            d = d.astype(np.float32)
            out[name] = convert_units(d, name, info.get("units", SSP_UNITS[name]))
    return SSPGrid(**out)


def load_ssp_file(name: str) -> SSPGrid:
    """spectra/ssp/factory.py:13-76 for the templates rubix names, from the template
    directory."""
    cfg = SSP_TEMPLATES[name]
    path = os.path.join(template_path(), cfg["file_name"])
    fmt = cfg["format"].lower()
    if not os.path.exists(path):
        raise FileNotFoundError(f"SSP template file {path} not found (templates are not "
                                "downloaded; place the file there or set "
                                "RUBIX_GB300_TEMPLATE_PATH)")
    if fmt in ("hdf5", "fsps"):
        return load_hdf5_template(path, cfg["fields"])
    return load_pypipe3d(path, cfg["fields"])


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
    if name in SSP_TEMPLATES:
        grid = load_ssp_file(name)
        _TEMPLATES[name] = grid
        return grid
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
           "get_lookup_interpolation", "like_input", "load_pypipe3d", "load_ssp_file",
           "SSP_TEMPLATES", "SSP_UNITS", "convert_units", "template_path",
           "load_hdf5_template"]
