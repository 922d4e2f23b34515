"""LSF step (rubix/core/lsf.py:14-67, telescope/lsf/lsf.py:12-105)."""

from __future__ import annotations

from typing import Callable, Optional

from .. import ops
from .. import telescope as tel
from ..logging import get_logger
from .data import RubixData, device_of, to_device
from .telescope import get_telescope

EXTEND_FACTOR = 12  # telescope/lsf/lsf.py:68-74


def lsf_taps_checked(sigma: float, wave_res: float, extend_factor: int = EXTEND_FACTOR):
    """The rubix LSF taps; the crop [f, L+K-1-f) must keep the spectral length
    (lsf.py:59-65), which fails in rubix as well when the float arange gives K != 2f+1."""
    taps = tel.lsf_taps(sigma, wave_res, extend_factor)
    if taps.size != 2 * extend_factor + 1:
        raise ValueError(
            f"LSF kernel of {taps.size} taps (wave_res {wave_res}) does not preserve the "
            "spectral length with the fixed crop of 12 bins on each side")
    return taps


class LsfHandoff:
    """Links the ``calculate_datacube`` and ``convolve_lsf`` steps of one pipeline run
    in which only ``convolve_psf`` lies between them.  The LSF (along wavelength) and the
    PSF (across spaxels) commute, so ``calculate_datacube`` can apply the LSF in the
    epilogue of the fused accumulate kernel, which saves a read and a write of the
    cube; it then sets ``pending`` and ``convolve_lsf`` passes the cube through."""

    def __init__(self):
        self.taps = None      # set by get_convolve_lsf
        self.pending = False  # the current datacube already holds the LSF


def lsf_fusable(step_names) -> bool:
    """True when convolve_lsf follows calculate_datacube with nothing but convolve_psf
    in between."""
    names = list(step_names)
    if "calculate_datacube" not in names or "convolve_lsf" not in names:
        return False
    i, j = names.index("calculate_datacube"), names.index("convolve_lsf")
    return i < j and set(names[i + 1:j]) <= {"convolve_psf"}


def get_convolve_lsf(config: dict, handoff: Optional[LsfHandoff] = None) -> Callable:
    """rubix/core/lsf.py:14-67 (same config checks and messages).  With ``handoff``
    the step passes through a cube whose LSF ``calculate_datacube`` already applied."""
    logger = get_logger(config.get("logger", None))
    if "lsf" not in config["telescope"]:
        raise ValueError("LSF configuration not found in telescope configuration")
    if "sigma" not in config["telescope"]["lsf"]:
        raise ValueError("LSF sigma size not found in telescope configuration")
    sigma = config["telescope"]["lsf"]["sigma"]
    telescope = get_telescope(config)
    taps = lsf_taps_checked(sigma, telescope.wave_res)
    dev = device_of(config)
    if handoff is not None:
        handoff.taps = taps

    def convolve_lsf(rubixdata: RubixData) -> RubixData:
        """Convolve the input datacube with the LSF."""
        logger.info("Convolving with LSF...")
        if handoff is not None and handoff.pending:
            handoff.pending = False  # applied in the accumulate epilogue
            return rubixdata
        cube = to_device(rubixdata.stars.datacube, dev)
        rubixdata.stars.datacube = ops.lsf_forward(cube, taps, EXTEND_FACTOR)
        return rubixdata

    return convolve_lsf
