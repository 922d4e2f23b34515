"""Configuration: the constants and pipeline definitions rubix keeps in YAML.

``rubix_config`` holds the entries of rubix/config/rubix_config.yml this path uses
(``SPEED_OF_LIGHT`` :8, ``ifu.doppler.velocity_direction`` :241-245); ``PIPELINES`` holds
the ``calc_ifu`` chain of rubix/config/pipeline_config.yml:1-60 as a dict (PyYAML is
not a dependency).
"""

from __future__ import annotations

import copy
import json
import os

rubix_config = {
    "constants": {"SPEED_OF_LIGHT": 299792.458},
    "ifu": {"doppler": {"velocity_direction": "z"}},
}

_CALC_IFU_ORDER = [
    "rotate_galaxy", "filter_particles", "spaxel_assignment", "reshape_data",
    "calculate_spectra", "scale_spectrum_by_mass", "doppler_shift_and_resampling",
    "calculate_datacube", "convolve_psf", "convolve_lsf", "apply_noise",
]


def _chain(names):
    out = {}
    prev = None
    for n in names:
        out[n] = {"name": n, "depends_on": prev, "args": [], "kwargs": {}}
        prev = n
    return {"Transformers": out}


PIPELINES = {"calc_ifu": _chain(_CALC_IFU_ORDER)}


def get_config(config):
    """A user config dict (copied) or the path of a JSON file (rubix/utils.py:10-27)."""
    if isinstance(config, dict):
        return copy.deepcopy(config)
    if isinstance(config, str) and os.path.exists(config):
        with open(config) as f:
            return json.load(f)
    raise ValueError(f"Cannot read configuration {config!r} (a dict or a JSON file path)")


def get_pipeline_config(name: str):
    """rubix/utils.py:30-44."""
    if name not in PIPELINES:
        raise ValueError(f"Pipeline {name} not found in the configuration")
    return copy.deepcopy(PIPELINES[name])
