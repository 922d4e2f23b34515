"""rubix_gb300: the rubix particle -> IFU datacube path as hand-written sm_103a CUDA kernels.

The CUDA library (``librubix_gb300.so``, C ABI in include/rubix_gb300.h) is the only
compute path.  ``rubix_gb300.core`` mirrors rubix's pipeline-step API
(``get_calculate_spectra``, ``get_scale_spectrum_by_mass``,
``get_doppler_shift_and_resampling``, ``get_calculate_datacube``, ``get_convolve_psf``,
``get_convolve_lsf``, ``RubixPipeline``) on top of it.
"""

__version__ = "0.1.0"


def build(force: bool = False) -> str:
    """Compile the CUDA library in-tree if it is missing or stale; returns its path."""
    from ._build import build as _b

    return _b(force=force)
