"""Step apply_noise (rubix/core/noise.py:17-80) on the CUDA noise kernels.

Same config keys, validation messages and closure name as rubix.  rubix draws the noise
from jax.random with the fixed key 0 (rubix/telescope/noise/noise.py:103); here the
draws come from a Philox4x32-10 generator keyed by ``config["telescope"]["noise"]
["seed"]`` (default 0): reproducible per seed and distributed like rubix's noise, but
not the same numbers.
"""

from __future__ import annotations

from typing import Callable

from .. import ops
from ..logging import get_logger
from .data import RubixData

SUPPORTED_NOISE_DISTRIBUTIONS = ["normal", "uniform"]


def get_apply_noise(config: dict) -> Callable:
    if "noise" not in config["telescope"]:
        raise ValueError("Noise information not provided in telescope config")
    if "signal_to_noise" not in config["telescope"]["noise"]:
        raise ValueError("Signal to noise information not provided in noise config")
    if "noise_distribution" not in config["telescope"]["noise"]:
        raise ValueError(
            "Noise distribution not provided in noise config. Currently supported "
            f"distributions are: {SUPPORTED_NOISE_DISTRIBUTIONS}")
    signal_to_noise = config["telescope"]["noise"]["signal_to_noise"]
    noise_distribution = config["telescope"]["noise"]["noise_distribution"]
    seed = int(config["telescope"]["noise"].get("seed", 0))
    logger = get_logger(config.get("logger", None))

    def apply_noise(rubixdata: RubixData) -> RubixData:
        logger.info(
            f"Applying noise to datacube with signal to noise ratio: {signal_to_noise} and "
            f"noise distribution: {noise_distribution}")
        cube = rubixdata.stars.datacube.contiguous()
        ops.apply_noise_(cube, float(signal_to_noise), noise_distribution, seed)
        rubixdata.stars.datacube = cube
        return rubixdata

    return apply_noise
