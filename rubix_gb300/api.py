"""Device-resident renderer for the particle -> datacube path.

``IFURenderer`` holds the per-configuration constants on the GPU (SSP template grid,
redshifted SSP wavelengths, telescope wavelength grid, spatial bin edges, PSF and
LSF taps) and runs the kernels of the C ABI for one set of particles:

    aperture mask -> spaxel assignment -> stable sort by spaxel
    [-> A_V of every star from the gas (dust extinction, when configured)]
    -> fused lookup/mass/Doppler/resample/(dust)/accumulate -> PSF -> LSF

It is the engine behind the rubix-compatible step functions in ``rubix_gb300.core``
(where each step stays separately callable) and the one-call path used for
benchmarks.  Inputs may be host (numpy / CPU tensors, copied once) or CUDA tensors.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import dust as dust_host
from . import ops
from . import telescope as tel


def _dev(a, device, dtype=torch.float32):
    if isinstance(a, torch.Tensor):
        t = a
    else:
        t = torch.from_numpy(np.ascontiguousarray(a))
    if t.dtype != dtype:
        t = t.to(dtype)
    if t.device != torch.device(device):
        t = t.to(device, non_blocking=True)
    return t.contiguous()


@dataclass
class CubeStages:
    pixel_assignment: torch.Tensor
    mask: Optional[torch.Tensor]
    perm: torch.Tensor
    seg_offsets: torch.Tensor
    cube: torch.Tensor             # output of the accumulate kernel [sbin, sbin, L]
    cube_psf: Optional[torch.Tensor]
    cube_lsf: Optional[torch.Tensor]
    lsf_fused: bool = False        # cube already holds the LSF (applied before the PSF)
    final: Optional[torch.Tensor] = None


class IFURenderer:
    """Constants of one (SSP, telescope, redshift, PSF, LSF) configuration on a device."""

    def __init__(self, ssp_age, ssp_metallicity, ssp_wavelength, ssp_flux, wave_t, edges,
                 sbin: int, dist_z: float, psf_taps=None, lsf_taps=None, lsf_crop: int = 12,
                 velocity_axis: int = 2, apply_filter: bool = True, device="cuda",
                 noise_s2n: Optional[float] = None, noise_distribution: str = "normal",
                 noise_seed: int = 0, dust: Optional[dict] = None,
                 spaxel_area: Optional[float] = None):
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("IFURenderer needs a CUDA device (rubix_gb300 has no CPU path)")
        self.ssp_age = _dev(ssp_age, self.device)
        self.ssp_metallicity = _dev(ssp_metallicity, self.device)
        flux = np.asarray(ssp_flux, dtype=np.float32) if not isinstance(ssp_flux, torch.Tensor) else ssp_flux
        self.ssp_flux = _dev(flux, self.device)
        wz = tel.cosmological_doppler_shift(dist_z, np.asarray(ssp_wavelength, dtype=np.float32)
                                            if not isinstance(ssp_wavelength, torch.Tensor)
                                            else ssp_wavelength.cpu().numpy())
        self.ssp_wave_z = _dev(wz, self.device)
        self.wave_t = _dev(wave_t, self.device)
        self.edges = _dev(edges, self.device)
        self.sbin = int(sbin)
        self.n_wave_t = int(self.wave_t.numel())
        self.psf_taps = None if psf_taps is None else np.asarray(psf_taps, dtype=np.float64)
        self.lsf_taps = None if lsf_taps is None else np.asarray(lsf_taps, dtype=np.float64)
        self.lsf_crop = int(lsf_crop)
        self.velocity_axis = int(velocity_axis)
        self.apply_filter = bool(apply_filter)
        self.noise_s2n = None if noise_s2n is None else float(noise_s2n)
        self.noise_distribution = noise_distribution
        self.noise_seed = int(noise_seed)
        # dust: keys of rubix's ssp.dust config (extinction_model, Rv, dust_grain_density,
        # dust_to_gas_model, Xco); spaxel_area in kpc^2 (square of the spatial bin size)
        self.dust = None
        if dust is not None:
            d = dict(dust_host.DUST_DEFAULTS)
            d.update(dust)
            if spaxel_area is None:
                raise ValueError("dust extinction needs the spaxel area (kpc^2)")
            self.dust = d
            self.spaxel_area = float(spaxel_area)
            self.dust_exponent = _dev(dust_host.extinction_exponent(
                self.wave_t.cpu().numpy(), d["extinction_model"], d["Rv"]), self.device)
            self.dgr_params, self.dgr_broken = dust_host.dust_to_gas_params(
                d["dust_to_gas_model"], d["Xco"])
            self.ext_scale = dust_host.extinction_scale(d["dust_grain_density"])

    @classmethod
    def from_workload(cls, w, device="cuda", psf=True, lsf=True, dust=None):
        area = None
        if dust is not None:
            from .synth import WORKLOADS

            _, size = tel.spatial_bin_edges(WORKLOADS[w.name]["fov"], w.sbin, w.dist_z)
            area = float(np.float32(size) ** 2)
        return cls(w.ssp.age, w.ssp.metallicity, w.ssp.wavelength, w.ssp.flux, w.wave_t, w.edges,
                   w.sbin, w.dist_z,
                   psf_taps=tel.gaussian_taps_1d(w.psf_size, w.psf_sigma) if psf else None,
                   lsf_taps=tel.lsf_taps(w.lsf_sigma, w.wave_res) if lsf else None,
                   device=device, noise_s2n=getattr(w, "noise_s2n", None), dust=dust,
                   spaxel_area=area)

    # -------------------------------------------------------------- steps
    def assign(self, coords):
        coords = _dev(coords, self.device)
        idx = ops.spaxel_assign(coords, self.edges)
        mask = ops.aperture_mask(coords, self.edges) if self.apply_filter else None
        return idx, mask

    def sort(self, idx, mask=None):
        return ops.spaxel_sort(idx, self.sbin * self.sbin, mask)

    def dust_av(self, star_coords, star_idx, gas_coords, gas_mass, gas_metals):
        """A_V of every star from the gas (rubix's calculate_extinction): gas outside the
        aperture has zero mass (filter_particles), per-cell extinction from
        12 + log(O/H), cumulative column along z per spaxel, interpolated at the stars."""
        if self.dust is None:
            raise ValueError("this renderer has no dust configuration")
        gc = _dev(gas_coords, self.device)
        gm = _dev(gas_mass, self.device)
        gidx = ops.spaxel_assign(gc, self.edges)
        if self.apply_filter:
            gm = ops.mask_zero_(gm.clone(), ops.aperture_mask(gc, self.edges))
        gext = ops.dust_gas_extinction(gm, _dev(gas_metals, self.device), self.dgr_params,
                                       self.dgr_broken, self.ext_scale, self.spaxel_area)
        nb = int(self.edges.numel()) - 1
        nseg = self.sbin * self.sbin
        return ops.dust_av(gc, gidx, gext, _dev(star_coords, self.device), star_idx, nseg,
                           max(nb * nb, nseg))

    def cube_buffer(self) -> torch.Tensor:
        """An uninitialised [sbin*sbin, L] float32 buffer for ``accumulate(out=...)``.  With a
        PSF its spaxel stride is L rounded up to a multiple of 4 floats, so the PSF stages
        the cube's rows with tiled TMA copies (16-byte row strides); the view is [.., L]
        and the padding is never read.  ``.contiguous()`` gives the dense layout."""
        n, L = self.sbin * self.sbin, self.n_wave_t
        if self.psf_taps is None:
            return torch.empty((n, L), dtype=torch.float32, device=self.device)
        buf = torch.empty((n, (L + 3) // 4 * 4), dtype=torch.float32, device=self.device)
        return buf[:, :L]

    def accumulate(self, mass, metallicity, age, velocity, perm, seg_offsets, out=None,
                   with_lsf=False, dust_av=None):
        """Fused lookup/mass/Doppler/resample/sum; ``with_lsf`` adds the LSF epilogue and
        ``dust_av`` (A_V per particle) the dust transmission of each spectrum.  Without
        ``out`` the cube goes to ``cube_buffer()``: with a PSF, a [sbin, sbin, L] view
        whose spaxel stride is L rounded up to a multiple of 4."""
        if out is None:
            out = self.cube_buffer()
        cube = ops.cube_forward(self.ssp_flux, self.ssp_metallicity, self.ssp_age, self.ssp_wave_z,
                                self.wave_t, _dev(mass, self.device), _dev(metallicity, self.device),
                                _dev(age, self.device), _dev(velocity, self.device),
                                self.velocity_axis, perm, seg_offsets, self.sbin * self.sbin, out=out,
                                lsf_taps=self.lsf_taps if with_lsf else None,
                                lsf_crop=self.lsf_crop, dust_av=dust_av,
                                dust_exponent=None if dust_av is None else self.dust_exponent)
        return cube.view(self.sbin, self.sbin, self.n_wave_t)

    def psf(self, cube, out=None):
        return ops.psf_forward(cube, self.psf_taps, out=out)

    def lsf(self, cube, out=None):
        return ops.lsf_forward(cube, self.lsf_taps, self.lsf_crop, out=out)

    def noise_(self, cube):
        """apply_noise in place when the renderer has a signal-to-noise (else no-op)."""
        if self.noise_s2n is not None:
            ops.apply_noise_(cube, self.noise_s2n, self.noise_distribution, self.noise_seed)
        return cube

    # -------------------------------------------------------------- whole path
    def render(self, coords, velocity, mass, metallicity, age, fuse_lsf=True,
               gas=None) -> CubeStages:
        """Whole path.  With ``fuse_lsf`` the LSF runs inside the accumulate kernel and the
        PSF afterwards (the two act on different axes and commute), saving one read and
        one write of the cube; the final cube is the same.  ``gas`` = (coords, mass,
        metals) applies the dust extinction of a renderer built with ``dust``."""
        idx, mask = self.assign(coords)
        perm, offs = self.sort(idx, mask)
        av = None
        if gas is not None:
            av = self.dust_av(coords, idx, *gas)
        fuse = fuse_lsf and self.lsf_taps is not None
        cube = self.accumulate(mass, metallicity, age, velocity, perm, offs, with_lsf=fuse,
                               dust_av=av)
        if fuse:
            c_psf = self.psf(cube) if self.psf_taps is not None else None
            final = c_psf if c_psf is not None else cube
            if self.noise_s2n is not None and final is cube:
                final = cube.clone()  # keep the accumulate stage noise-free
            final = self.noise_(final)
            return CubeStages(idx, mask, perm, offs, cube, c_psf, None, True, final)
        c_psf = self.psf(cube) if self.psf_taps is not None else None
        c_lsf = self.lsf(c_psf if c_psf is not None else cube) if self.lsf_taps is not None else None
        final = c_lsf if c_lsf is not None else (c_psf if c_psf is not None else cube)
        if self.noise_s2n is not None and final is cube:
            final = cube.clone()  # keep the accumulate stage noise-free
        final = self.noise_(final)
        return CubeStages(idx, mask, perm, offs, cube, c_psf, c_lsf, False, final)

    def host_stream(self, n_slots: int = 2) -> "HostStream":
        """A ``HostStream`` rendering pinned host inputs into pinned host outputs with
        the copies of one render overlapped with the compute of the next."""
        return HostStream(self, n_slots)


class HostStream:
    """Back-to-back renders from host to host with overlapped transfers.

    Each ``submit`` copies one galaxy's particle arrays from (pinned) host memory to a
    device slot on an upload stream, renders it on the caller's current stream into
    the slot's cube buffers, and copies the final cube to the given (pinned) host
    tensor on a download stream.  Slots rotate, so the download of render k and the
    upload of render k+1 run while render k+1 / k computes; events order the three
    streams and keep a slot from being overwritten before its download ended.
    ``synchronize`` makes the current stream wait for every download.
    """

    def __init__(self, renderer: IFURenderer, n_slots: int = 2):
        self.r = renderer
        dev = renderer.device
        self.up = torch.cuda.Stream(dev)
        self.down = torch.cuda.Stream(dev)
        self.slots = [dict(inputs=None, cube=None, final=None,
                           computed=torch.cuda.Event(), downloaded=torch.cuda.Event(),
                           uploaded=torch.cuda.Event(), used=False)
                      for _ in range(max(1, int(n_slots)))]
        self.k = 0

    def submit(self, coords, velocity, mass, metallicity, age, out: torch.Tensor) -> None:
        r = self.r
        slot = self.slots[self.k % len(self.slots)]
        self.k += 1
        host = (coords, velocity, mass, metallicity, age)
        compute = torch.cuda.current_stream(r.device)
        fresh = slot["inputs"] is None or any(d.shape != torch.Size(np.shape(h))
                                              for d, h in zip(slot["inputs"], host))
        if fresh:
            slot["inputs"] = [torch.empty(tuple(np.shape(h)), dtype=torch.float32,
                                          device=r.device) for h in host]
        # upload: after the compute that last read this slot's inputs; into fresh
        # buffers only after everything already on the compute stream, which may still
        # use the recycled memory
        if slot["used"] and not fresh:
            self.up.wait_event(slot["computed"])
        else:
            self.up.wait_stream(compute)
        with torch.cuda.stream(self.up):
            for d, h in zip(slot["inputs"], host):
                d.copy_(torch.as_tensor(h), non_blocking=True)
            slot["uploaded"].record(self.up)
        compute.wait_event(slot["uploaded"])
        if slot["used"]:
            compute.wait_event(slot["downloaded"])  # cube buffers free again
        c, v, m, z, a = slot["inputs"]
        idx, mask = r.assign(c)
        perm, offs = r.sort(idx, mask)
        fuse = r.lsf_taps is not None
        if slot["cube"] is None:
            L = r.n_wave_t
            slot["cube"] = r.cube_buffer()
            slot["final"] = torch.empty((r.sbin, r.sbin, L), dtype=torch.float32,
                                        device=r.device)
        cube = r.accumulate(m, z, a, v, perm, offs, out=slot["cube"], with_lsf=fuse)
        if r.psf_taps is not None:
            final = r.psf(cube, out=slot["final"])
        else:
            slot["final"].copy_(cube)
            final = slot["final"]
        if not fuse and r.lsf_taps is not None:
            final = slot["final"].copy_(r.lsf(final))
        r.noise_(final)
        slot["computed"].record(compute)
        self.down.wait_event(slot["computed"])
        with torch.cuda.stream(self.down):
            out.copy_(final, non_blocking=True)
            slot["downloaded"].record(self.down)
        slot["used"] = True

    def synchronize(self) -> None:
        """The current stream waits for every upload and download issued so far."""
        compute = torch.cuda.current_stream(self.r.device)
        compute.wait_stream(self.up)
        compute.wait_stream(self.down)
