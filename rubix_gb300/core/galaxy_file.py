"""rubix's galaxy file: writing it, reading it back and preparing the pipeline input.

* ``create_rubix_file`` writes the layout of rubix/galaxy/input_handler/base.py:17-73:
  groups ``meta``, ``galaxy`` and ``particles/<type>``, one dataset per field with its
  unit as the ``unit`` attribute.  rubix converts every field to the configured unit
  with astropy first; astropy is not a dependency here, so the values are written as
  given and ``units`` names the units they are in.
* ``load_galaxy_data`` is rubix/utils.py:160-200 (same keys, same unit dictionary).
* ``center_particles`` is rubix/galaxy/alignment.py:10-62.
* ``prepare_input`` / ``get_rubix_data`` are rubix/core/data.py:490-619: the file
  ``<output_path>/rubix_galaxy.h5`` becomes a ``RubixData`` (galaxy fields and
  ``<field>_unit`` attributes, the configured particle types, centred, with rubix's
  seeded random subset).  Producing that file from simulation snapshots (rubix's
  IllustrisTNG / NIHAO input handlers and API download) is not part of this package.

The files are HDF5, read and written by ``rubix_gb300.hdf5``.
"""

from __future__ import annotations

import os
from typing import Dict, Tuple, Union

import numpy as np

from .. import hdf5
from ..logging import get_logger
from .config import get_config
from .data import Galaxy, GasData, RubixData, StarsData

__all__ = ["create_rubix_file", "load_galaxy_data", "center_particles", "prepare_input",
           "get_rubix_data", "RUBIX_FILE_NAME"]

RUBIX_FILE_NAME = "rubix_galaxy.h5"


def create_rubix_file(file_path: str, particle_data: Dict[str, dict], galaxy_data: dict,
                      simulation_metadata: dict, units: Dict[str, dict]) -> str:
    """rubix/galaxy/input_handler/base.py:17-73 (values already in ``units``).

    units["galaxy"][key] and units[<type>][field] are the unit strings stored as each
    dataset's ``unit`` attribute.  Returns ``file_path``."""
    tree = {"meta": {k: np.asarray(v) if not isinstance(v, str) else v
                     for k, v in simulation_metadata.items()},
            "galaxy": {k: (np.asarray(v), {"unit": str(units["galaxy"][k])})
                       for k, v in galaxy_data.items()},
            "particles": {}}
    for ptype, fields in particle_data.items():
        tree["particles"][ptype] = {f: (np.asarray(v), {"unit": str(units[ptype][f])})
                                    for f, v in fields.items()}
    d = os.path.dirname(file_path)
    if d:
        os.makedirs(d, exist_ok=True)
    hdf5.write_file(file_path, tree)
    return file_path


def load_galaxy_data(path_to_file: str) -> Tuple[dict, dict]:
    """rubix/utils.py:160-200: (galaxy_data, units) of a rubix galaxy file."""
    if not os.path.exists(path_to_file):
        raise FileNotFoundError(f"File {str(path_to_file)} does not exist")
    galaxy_data: dict = {}
    units: dict = {}
    with hdf5.File(path_to_file, "r") as f:
        galaxy_data["subhalo_center"] = f["galaxy/center"][()]
        galaxy_data["subhalo_halfmassrad_stars"] = f["galaxy/halfmassrad_stars"][()]
        galaxy_data["redshift"] = f["galaxy/redshift"][()]
        units["galaxy"] = {}
        for key in f["galaxy"].keys():
            units["galaxy"][key] = f["galaxy"][key].attrs["unit"]
        galaxy_data["particle_data"] = {}
        for key in f["particles"].keys():
            galaxy_data["particle_data"][key] = {}
            units[key] = {}
            for field in f["particles"][key].keys():
                ds = f[f"particles/{key}/{field}"]
                galaxy_data["particle_data"][key][field] = ds[()]
                units[key][field] = ds.attrs["unit"]
    return galaxy_data, units


def _jax_default(a: np.ndarray) -> np.ndarray:
    """The dtype jnp.array gives with 64-bit types disabled (rubix's setting): float64
    -> float32, int64 -> int32."""
    a = np.asarray(a)
    if a.dtype == np.float64:
        return a.astype(np.float32)
    if a.dtype == np.int64:
        return a.astype(np.int32)
    if a.dtype == np.uint64:
        return a.astype(np.uint32)
    return a


def center_particles(rubixdata: RubixData, key: str) -> RubixData:
    """rubix/galaxy/alignment.py:10-62: coordinates relative to the galaxy centre,
    velocities relative to the median velocity of the particles within 10 (kpc) of it;
    a centre outside the particles' bounding box is an error.  In the particles' own
    precision (float32 in rubix), the centre cast to it."""
    comp = rubixdata.stars if key == "stars" else rubixdata.gas
    coords = np.asarray(comp.coords)
    vel = np.asarray(comp.velocity)
    center = np.asarray(rubixdata.galaxy.center, dtype=coords.dtype)
    inside = all(coords[:, i].min() <= center[i] <= coords[:, i].max() for i in range(3))
    if not inside:
        raise ValueError("Center is not within the bounds of the galaxy")
    mask = np.linalg.norm(coords - center, axis=1) < 10
    with np.errstate(invalid="ignore"):
        central_velocity = (np.median(vel[mask], axis=0) if mask.any()
                            else np.full(3, np.nan, dtype=vel.dtype))
    comp.coords = coords - center
    comp.velocity = vel - central_velocity
    return rubixdata


def prepare_input(config: Union[dict, str]) -> RubixData:
    """rubix/core/data.py:490-604."""
    config = get_config(config) if isinstance(config, str) else config
    logger = get_logger(config.get("logger", None))
    file_path = os.path.join(config["output_path"], RUBIX_FILE_NAME)
    data, units = load_galaxy_data(file_path)
    rubixdata = RubixData(Galaxy(), StarsData(), GasData())
    rubixdata.galaxy.redshift = data["redshift"]
    rubixdata.galaxy.redshift_unit = units["galaxy"]["redshift"]
    rubixdata.galaxy.center = data["subhalo_center"]
    rubixdata.galaxy.center_unit = units["galaxy"]["center"]
    rubixdata.galaxy.halfmassrad_stars = data["subhalo_halfmassrad_stars"]
    rubixdata.galaxy.halfmassrad_stars_unit = units["galaxy"]["halfmassrad_stars"]
    for part_type in config["data"]["args"]["particle_type"]:
        if part_type not in data["particle_data"]:
            continue
        comp = getattr(rubixdata, part_type)
        for attribute, value in data["particle_data"][part_type].items():
            setattr(comp, attribute, _jax_default(value))  # rubix: jnp.array(value)
            setattr(comp, attribute + "_unit", units[part_type][attribute])
        logger.info(f"Centering {part_type} particles")
        rubixdata = center_particles(rubixdata, part_type)
        subset = config.get("data", {}).get("subset", {})
        if subset.get("use_subset"):
            size = subset["subset_size"]
            np.random.seed(42)
            if rubixdata.stars.coords is not None:
                n = len(rubixdata.stars.coords)
            elif rubixdata.gas.coords is not None:
                n = len(rubixdata.gas.coords)
            else:
                raise ValueError("Neither stars nor gas coordinates are available.")
            indices = np.random.choice(np.arange(n), size=size, replace=False)
            for attribute in data["particle_data"][part_type].keys():
                v = getattr(comp, attribute)
                setattr(comp, attribute, v[indices, :] if v.ndim == 2 else v[indices])
            logger.warning(f"The Subset value is set in config. Using only subset of size "
                           f"{size} for {part_type}")
    return rubixdata


def get_rubix_data(config: Union[dict, str]) -> RubixData:
    """rubix/core/data.py:607-619 for a galaxy already in rubix's file format."""
    config = get_config(config) if isinstance(config, str) else config
    if "output_path" not in config:
        raise ValueError("no particle data: pass data= (a RubixData) or set "
                         f"config['output_path'] to the directory of a {RUBIX_FILE_NAME}")
    path = os.path.join(config["output_path"], RUBIX_FILE_NAME)
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} not found: rubix_gb300 reads galaxies in rubix's file format "
            "(rubix_gb300.core.create_rubix_file writes it); converting simulation "
            "snapshots is not part of this package")
    return prepare_input(config)
