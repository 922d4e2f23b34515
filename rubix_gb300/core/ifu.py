"""IFU steps: calculate_spectra, scale_spectrum_by_mass, doppler_shift_and_resampling,
calculate_datacube (rubix/core/ifu.py:28-341).

rubix materialises an (1, N, n_lambda_ssp) array after ``calculate_spectra`` and an
(1, N, n_lambda_telescope) array after ``doppler_shift_and_resampling``
(core/ifu.py:114-118, 280-283).  Here those steps store a ``ParticleSpectra`` that
records what the spectra are; ``calculate_datacube`` then runs the fused kernel
(lookup + mass + Doppler + resample + per-spaxel sum) without ever writing the
per-particle spectra.  Reading ``stars.spectra`` (``.materialize()``, ``np.asarray``,
``torch.as_tensor``) computes the array on the GPU with the materialising kernels, so
every step can still be used on its own.  Steps also accept materialised spectra
supplied by the caller.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np
import torch

from .. import ops
from .. import telescope as tel
from ..logging import get_logger
from .config import rubix_config
from .data import RubixData, device_constant, device_of, flat_particles, has_device_axis, to_device
from .ssp import get_ssp, lookup_method
from .lsf import EXTEND_FACTOR
from .telescope import get_telescope

_AXIS = {"x": 0, "y": 1, "z": 2}


@dataclass
class ParticleSpectra:
    """Per-particle spectra that have not been written to memory.

    stage "lookup":    SSP lookup at (metallicity, age)        -> [1, N, n_lambda_ssp]
    stage "mass":      times mass                              -> [1, N, n_lambda_ssp]
    stage "resampled": Doppler shifted and resampled to wave_t -> [1, N, n_lambda_t]

    ``dust_av`` / ``dust_exponent`` (set by ``calculate_extinction``): every resampled
    spectrum is multiplied by its dust transmission 2^(dust_exponent[t] * dust_av[i]).
    """

    stage: str
    ssp: object
    metallicity: torch.Tensor
    age: torch.Tensor
    device: torch.device
    mass: Optional[torch.Tensor] = None
    velocity: Optional[torch.Tensor] = None
    velocity_axis: int = 2
    wave_z: Optional[torch.Tensor] = None
    wave_t: Optional[torch.Tensor] = None
    device_axis: bool = True
    dust_av: Optional[torch.Tensor] = None
    dust_exponent: Optional[torch.Tensor] = None

    @property
    def n(self) -> int:
        return int(self.metallicity.numel())

    @property
    def shape(self):
        width = self.wave_t.numel() if self.stage == "resampled" else self.ssp.wavelength.size
        return (1, self.n, int(width)) if self.device_axis else (self.n, int(width))

    @property
    def ndim(self):
        return len(self.shape)

    def materialize(self) -> torch.Tensor:
        """The spectra as a CUDA tensor of ``self.shape``."""
        flux, zg, ag, _ = self.ssp.device_arrays(self.device)
        if self.stage in ("lookup", "mass"):
            out = ops.ssp_lookup(flux, zg, ag, self.metallicity, self.age,
                                 self.mass if self.stage == "mass" else None)
        else:
            # every particle its own segment: the fused kernel writes one row each
            n = self.n
            ident = torch.arange(n, dtype=torch.int32, device=self.device)
            offs = torch.arange(n + 1, dtype=torch.int32, device=self.device)
            out = ops.cube_forward(flux, zg, ag, self.wave_z, self.wave_t, self.mass,
                                   self.metallicity, self.age, self.velocity, self.velocity_axis,
                                   ident, offs, n, dust_av=self.dust_av,
                                   dust_exponent=self.dust_exponent)
        return out.reshape(self.shape)

    def __array__(self, dtype=None, copy=None):
        a = self.materialize().cpu().numpy()
        return a if dtype is None else a.astype(dtype)


def _spectra_tensor(spec, device) -> torch.Tensor:
    """Materialised spectra (1, N, w) / (N, w) -> CUDA tensor (N, w)."""
    if isinstance(spec, ParticleSpectra):
        spec = spec.materialize()
    t = to_device(spec, device)
    return t.reshape(-1, t.shape[-1])


def get_calculate_spectra(config: dict) -> Callable:
    """rubix/core/ifu.py:28-123 (SSP lookup; ``config["ssp"]["method"]`` must be
    "linear")."""
    logger = get_logger(config.get("logger", None))
    ssp = get_ssp(config)
    method = lookup_method(config)
    if method != "linear":
        raise ValueError(
            f"SSP interpolation method {method!r} is not available: rubix_gb300 implements "
            "method='linear' (set config['ssp']['method'] = 'linear')")
    dev = device_of(config)

    def calculate_spectra(rubixdata: RubixData) -> RubixData:
        logger.info("Calculating IFU cube...")
        st = rubixdata.stars
        st.spectra = ParticleSpectra(
            stage="lookup", ssp=ssp, metallicity=flat_particles(st.metallicity, dev),
            age=flat_particles(st.age, dev), device=dev,
            device_axis=True)
        return rubixdata

    return calculate_spectra


def get_scale_spectrum_by_mass(config: dict) -> Callable:
    """rubix/core/ifu.py:126-159."""
    logger = get_logger(config.get("logger", None))
    dev = device_of(config)

    def scale_spectrum_by_mass(rubixdata: RubixData) -> RubixData:
        logger.info("Scaling Spectra by Mass...")
        st = rubixdata.stars
        mass = flat_particles(st.mass, dev)
        spec = st.spectra
        if isinstance(spec, ParticleSpectra) and spec.stage == "lookup":
            st.spectra = ParticleSpectra(
                stage="mass", ssp=spec.ssp, metallicity=spec.metallicity, age=spec.age,
                device=dev, mass=mass, device_axis=spec.device_axis)
        else:
            rows = _spectra_tensor(spec, dev)
            out = ops.scale_rows(rows, mass)
            st.spectra = out.reshape(tuple(np.shape(spec)))
        return rubixdata

    return scale_spectrum_by_mass


def get_doppler_shift_and_resampling(config: dict) -> Callable:
    """rubix/core/ifu.py:225-295: SSP wavelengths shifted by (1+z) and exp(v/c) along
    ``rubix_config["ifu"]["doppler"]["velocity_direction"]``, resampled onto the
    telescope grid with flux conservation."""
    logger = get_logger(config.get("logger", None))
    direction = rubix_config["ifu"]["doppler"]["velocity_direction"]
    axis = _AXIS[direction]
    z = config["galaxy"]["dist_z"]
    telescope = get_telescope(config)
    ssp = get_ssp(config)
    dev = device_of(config)
    wave_z_np = tel.cosmological_doppler_shift(z, ssp.wavelength)
    wave_t_np = np.asarray(telescope.wave_seq, dtype=np.float32)

    def doppler_shift_and_resampling(rubixdata: RubixData) -> RubixData:
        wave_z = device_constant(wave_z_np, dev)
        wave_t = device_constant(wave_t_np, dev)
        for name in ("stars", "gas"):
            comp = getattr(rubixdata, name)
            if comp is None or comp.spectra is None:
                continue
            logger.info("Doppler shifting and resampling spectra...")
            vel = flat_particles(comp.velocity, dev, width=3)
            spec = comp.spectra
            if isinstance(spec, ParticleSpectra) and spec.stage == "mass":
                comp.spectra = ParticleSpectra(
                    stage="resampled", ssp=spec.ssp, metallicity=spec.metallicity, age=spec.age,
                    device=dev, mass=spec.mass, velocity=vel, velocity_axis=axis,
                    wave_z=wave_z, wave_t=wave_t, device_axis=spec.device_axis)
            else:
                rows = _spectra_tensor(spec, dev)
                out = ops.resample_rows(rows, wave_z, vel, axis, wave_t)
                comp.spectra = out.unsqueeze(0) if np.ndim(spec) == 3 else out
        return rubixdata

    return doppler_shift_and_resampling


def get_calculate_datacube(config: dict, lsf_handoff=None, psf_follows: bool = False) -> Callable:
    """rubix/core/ifu.py:298-341: per-spaxel sum into a [sbin, sbin, n_lambda] cube.

    With lazy spectra the fused kernel runs (stable spaxel sort + lookup/mass/Doppler/
    resample/accumulate); with materialised spectra the rows are summed per spaxel.
    Particles outside the aperture (zero mass after ``filter_particles``) contribute
    exactly 0 and are left out of the sort.  With ``lsf_handoff`` (a
    ``core.lsf.LsfHandoff`` shared with the run's ``convolve_lsf``) the fused kernel
    also applies the LSF, and the later ``convolve_lsf`` passes the cube through.  With
    ``psf_follows`` (the pipeline runs ``convolve_psf`` next) the cube is written with a
    spaxel stride of n_lambda rounded up to a multiple of 4, which lets the PSF stage its
    rows by TMA; ``convolve_psf`` then replaces it with its dense output.
    """
    logger = get_logger(config.get("logger", None))
    telescope = get_telescope(config)
    num_spaxels = int(telescope.sbin)
    dev = device_of(config)

    def calculate_datacube(rubixdata: RubixData) -> RubixData:
        logger.info("Calculating Data Cube...")
        st = rubixdata.stars
        idx = flat_particles(st.pixel_assignment, dev, dtype=torch.int32)
        nseg = num_spaxels * num_spaxels
        spec = st.spectra
        lazy = isinstance(spec, ParticleSpectra) and spec.stage == "resampled"
        keep = None
        if lazy and st.mask is not None:
            # filtered particles have zero mass in the lazy record: dropping them is exact
            keep = flat_particles(st.mask, dev, dtype=torch.uint8)
        perm, offs = ops.spaxel_sort(idx, nseg, keep)
        fuse = lazy and lsf_handoff is not None and lsf_handoff.taps is not None
        if lsf_handoff is not None:
            lsf_handoff.pending = fuse
        if lazy:
            flux, zg, ag, _ = spec.ssp.device_arrays(dev)
            out = None
            if psf_follows:
                # 16-byte spaxel rows, so convolve_psf stages them by TMA; the PSF step
                # replaces this cube with its dense output
                L = int(spec.wave_t.numel())
                out = torch.empty((nseg, (L + 3) // 4 * 4), dtype=torch.float32,
                                  device=dev)[:, :L]
            cube = ops.cube_forward(flux, zg, ag, spec.wave_z, spec.wave_t, spec.mass,
                                    spec.metallicity, spec.age, spec.velocity,
                                    spec.velocity_axis, perm, offs, nseg, dust_av=spec.dust_av,
                                    dust_exponent=spec.dust_exponent,
                                    lsf_taps=lsf_handoff.taps if fuse else None,
                                    lsf_crop=EXTEND_FACTOR, out=out)
        else:
            rows = _spectra_tensor(spec, dev)
            cube = ops.segment_sum_rows(rows, perm, offs, nseg)
        st.datacube = cube.reshape(num_spaxels, num_spaxels, -1)
        return rubixdata

    return calculate_datacube
