"""PSF step (rubix/core/psf.py:15-75, telescope/psf/psf.py:14-58)."""

from __future__ import annotations

from typing import Callable

import numpy as np

import torch

from .. import ops
from .. import telescope as tel
from ..logging import get_logger
from .data import RubixData, device_of, to_device


def get_psf_kernel(name: str, m: int, n: int, **kwargs) -> np.ndarray:
    """telescope/psf/psf.py:14-30 (float64 2-D kernel)."""
    if name == "gaussian":
        return tel.gaussian_kernel_2d(m=m, n=n, **kwargs)
    raise ValueError(f"Unknown PSF kernel name: {name}")


def get_convolve_psf(config: dict) -> Callable:
    """rubix/core/psf.py:15-75: same config checks and messages; the Gaussian kernel is
    applied as its two exact 1-D factors."""
    logger = get_logger(config.get("logger", None))
    if "psf" not in config["telescope"]:
        raise ValueError("PSF configuration not found in telescope configuration")
    if "name" not in config["telescope"]["psf"]:
        raise ValueError("PSF name not found in telescope configuration")
    if config["telescope"]["psf"]["name"] == "gaussian":
        if "size" not in config["telescope"]["psf"]:
            raise ValueError("PSF size not found in telescope configuration")
        if "sigma" not in config["telescope"]["psf"]:
            raise ValueError("PSF sigma not found in telescope configuration")
        m = n = config["telescope"]["psf"]["size"]
        sigma = config["telescope"]["psf"]["sigma"]
        taps_y = tel.gaussian_taps_1d(m, sigma)
        taps_x = tel.gaussian_taps_1d(n, sigma)
    else:
        raise ValueError(f"Unknown PSF kernel name: {config['telescope']['psf']['name']}")
    dev = device_of(config)

    def convolve_psf(rubixdata: RubixData) -> RubixData:
        """Convolve the input datacube with the PSF kernel."""
        logger.info("Convolving with PSF...")
        cube = rubixdata.stars.datacube
        # a device cube with unit wavelength stride goes in as it is: the PSF takes any
        # spaxel stride (calculate_datacube's 16-byte rows included) and writes a dense cube
        on_dev = (isinstance(cube, torch.Tensor) and cube.is_cuda
                  and (dev.index is None or cube.device.index == dev.index))
        if not (on_dev and cube.dim() == 3 and cube.dtype == torch.float32
                and cube.stride(2) == 1):
            cube = to_device(cube, dev)
        rubixdata.stars.datacube = ops.psf_forward(cube, taps_y, taps_x)
        return rubixdata

    return convolve_psf
