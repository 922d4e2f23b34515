"""rubix-compatible pipeline steps backed by the rubix_gb300 CUDA kernels.

Every factory keeps the name, config keys, error messages and closure ``__name__`` of
its rubix counterpart (rubix/core/*.py), so the closures can be registered in a
pipeline exactly as rubix registers its own.
"""

from .config import get_config, get_pipeline_config, rubix_config  # noqa: F401
from .data import (Galaxy, GasData, RubixData, StarsData, get_reshape_data,  # noqa: F401
                   reshape_array)
from .dust import apply_spaxel_extinction, get_extinction  # noqa: F401
from .galaxy_file import (center_particles, create_rubix_file, get_rubix_data,  # noqa: F401
                          load_galaxy_data, prepare_input)
from .ifu import (get_calculate_datacube, get_calculate_spectra,  # noqa: F401
                  get_doppler_shift_and_resampling, get_scale_spectrum_by_mass)
from .lsf import get_convolve_lsf  # noqa: F401
from .noise import get_apply_noise  # noqa: F401
from .pipeline import RubixPipeline  # noqa: F401
from .psf import get_convolve_psf  # noqa: F401
from .rotation import get_galaxy_rotation  # noqa: F401
from .ssp import get_lookup_interpolation, get_ssp, register_ssp_template  # noqa: F401
from .telescope import (get_filter_particles, get_spatial_bin_edges,  # noqa: F401
                        get_spaxel_assignment, get_telescope, register_telescope)
