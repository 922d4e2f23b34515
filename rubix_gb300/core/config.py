"""Configuration: the constants and pipeline definitions rubix keeps in YAML.

``rubix_config`` holds the entries of rubix/config/rubix_config.yml this path uses
(constants :6-18, ``ssp.dust`` :145-150, ``ifu.doppler.velocity_direction`` :241-245);
``PIPELINES`` holds the ``calc_ifu`` and ``calc_dusty_ifu`` chains of
rubix/config/pipeline_config.yml:1-136 as dicts (PyYAML is not a dependency).
"""

from __future__ import annotations

import copy
import json
import os

from .. import yaml_subset

rubix_config = {
    "constants": {"SPEED_OF_LIGHT": 299792.458, "KPC_TO_CM": 3.08568e21,
                  "MSUN_TO_GRAMS": 1.989e33, "MASS_OF_PROTON": 1.67262e-24},
    "ifu": {"doppler": {"velocity_direction": "z"}},
    # rubix_config.yml:145-150; the dust step reads dust_to_gas_model and Xco from here
    "ssp": {"dust": {"extinction_model": "Cardelli89", "Rv": 3.1,
                     "dust_to_gas_model": "broken power law fit", "Xco": "Z",
                     "dust_grain_density": 3.5}},
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


# rubix/config/pipeline_config.yml:62-136: calc_ifu with calculate_extinction between
# the resampling and the datacube
_CALC_DUSTY_IFU_ORDER = (_CALC_IFU_ORDER[:7] + ["calculate_extinction"]
                         + _CALC_IFU_ORDER[7:])

PIPELINES = {"calc_ifu": _chain(_CALC_IFU_ORDER),
             "calc_dusty_ifu": _chain(_CALC_DUSTY_IFU_ORDER)}


def get_config(config):
    """rubix/utils.py:10-27: a user config dict (copied) or the path of a YAML file (read
    with ``rubix_gb300.yaml_subset``, which covers what rubix's configurations use) or of
    a JSON file (``.json``)."""
    if isinstance(config, dict):
        return copy.deepcopy(config)
    if isinstance(config, str) and os.path.exists(config):
        if config.lower().endswith(".json"):
            with open(config) as f:
                return json.load(f)
        return yaml_subset.load_file(config)
    raise ValueError(f"Cannot read configuration {config!r} (a dict or a YAML / JSON file "
                     "path)")


def get_pipeline_config(name: str):
    """rubix/utils.py:30-44 (a fresh copy of the named pipeline's node table)."""
    if name not in PIPELINES:
        raise ValueError(f"Pipeline {name} not found in the configuration")
    src = PIPELINES[name]
    # nodes hold name, depends_on, args (list) and kwargs (dict): copied one level deep,
    # which is all a deep copy would copy, at a fraction of its cost
    return {k: ({n: {f: (list(v) if isinstance(v, list) else dict(v) if isinstance(v, dict)
                        else v) for f, v in node.items()} for n, node in val.items()}
                if k == "Transformers" else copy.deepcopy(val))
            for k, val in src.items()}
