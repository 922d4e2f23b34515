"""RubixPipeline (rubix/core/pipeline.py:30-208), eager, on the rubix_gb300 kernels.

Differences from rubix, all outside the particle -> cube path: the particle data is
passed in (``data=``, with ``galaxy.halfmassrad_stars`` for the rotation) or read from a
galaxy already in rubix's file format (``<output_path>/rubix_galaxy.h5``), not converted
from simulation snapshots; the SSP lookup is bilinear (``ssp.method =
"linear"``); the noise of ``apply_noise`` comes from a seeded Philox generator instead
of jax.random.
"""

from __future__ import annotations

import time
from typing import Optional

from ..logging import get_logger
from ..pipeline import LinearTransformerPipeline, step_names
from .config import get_config, get_pipeline_config
from .data import RubixData, get_reshape_data
from .dust import get_extinction
from .galaxy_file import get_rubix_data
from .ifu import (get_calculate_datacube, get_calculate_spectra,
                  get_doppler_shift_and_resampling, get_scale_spectrum_by_mass)
from .lsf import LsfHandoff, get_convolve_lsf, lsf_fusable
from .noise import get_apply_noise
from .psf import get_convolve_psf
from .rotation import get_galaxy_rotation
from .ssp import get_ssp
from .telescope import (FrameHandoff, frame_fusion, get_filter_particles,
                        get_spaxel_assignment, get_telescope)


class RubixPipeline:
    """``fuse_lsf``: when the pipeline runs convolve_lsf after calculate_datacube with
    only convolve_psf between them, apply the LSF in the accumulate kernel's epilogue
    (the two convolutions commute) instead of in a separate pass over the cube.
    ``fuse_frame``: when filter_particles is directly followed by spaxel_assignment
    (and directly preceded by rotate_galaxy), turn, filter and assign the particles in
    one pass.  Neither changes the result of the run."""

    def __init__(self, user_config, data: Optional[RubixData] = None, *,
                 fuse_lsf: bool = True, fuse_frame: bool = True):
        self.user_config = get_config(user_config)
        self.pipeline_config = get_pipeline_config(self.user_config["pipeline"]["name"])
        self.logger = get_logger(self.user_config.get("logger"))
        self.ssp = get_ssp(self.user_config)
        self.telescope = get_telescope(self.user_config)
        # without data the galaxy is read at run time from <output_path>/rubix_galaxy.h5
        # (rubix/core/pipeline.py:145-150 via get_rubix_data)
        self.data = data
        self.func = None
        self.fuse_lsf = fuse_lsf
        self.fuse_frame = fuse_frame

    def _get_pipeline_functions(self, handoff: Optional[LsfHandoff] = None,
                                frame: Optional[FrameHandoff] = None,
                                psf_follows: bool = False) -> list:
        c = self.user_config
        lsf = get_convolve_lsf(c, handoff)
        funcs = [
            get_galaxy_rotation(c, frame), get_filter_particles(c, frame),
            get_spaxel_assignment(c, frame), get_calculate_spectra(c), get_reshape_data(c),
            get_scale_spectrum_by_mass(c), get_doppler_shift_and_resampling(c),
            get_calculate_datacube(c, handoff, psf_follows), get_convolve_psf(c), lsf,
            get_apply_noise(c),
        ]
        # rubix builds calculate_extinction for every pipeline (core/pipeline.py:114);
        # here it is built when the configuration has a dust section
        if "dust" in c.get("ssp", {}):
            funcs.insert(7, get_extinction(c))
        return funcs

    def run(self) -> RubixData:
        t0 = time.time()
        if self.data is None:
            self.data = get_rubix_data(self.user_config)
        names = step_names(self.pipeline_config)
        lsf = LsfHandoff() if self.fuse_lsf and lsf_fusable(names) else None
        frame = frame_fusion(names) if self.fuse_frame else None
        # calculate_datacube writes TMA-ready (16-byte) spaxel rows when convolve_psf,
        # which replaces the cube with a dense one, runs directly after it
        i = names.index("calculate_datacube") if "calculate_datacube" in names else -1
        psf_follows = 0 <= i < len(names) - 1 and names[i + 1] == "convolve_psf"
        self._pipeline = LinearTransformerPipeline(
            self.pipeline_config, self._get_pipeline_functions(lsf, frame, psf_follows))
        self.func = self._pipeline.expression
        out = self.func(self.data)
        import torch

        torch.cuda.synchronize()
        self.logger.info("Pipeline run completed in %.2f seconds.", time.time() - t0)
        return out

    def gradient(self):
        """rubix/core/pipeline.py:204-208 raises here as well; gradients of the cube are
        available through rubix_gb300.autograd."""
        raise NotImplementedError("Gradient calculation is not implemented yet")
