"""Gradients of the datacube with respect to the particles and the PSF/LSF widths.

rubix differentiates its pipeline with ``jax.grad`` (``RubixPipeline.gradient``,
rubix/core/pipeline.py:204-208): the cube is a differentiable function of the particle
masses, metallicities, ages and velocities and of the telescope's PSF and LSF widths.
``DatacubeFunction`` is the same function as a ``torch.autograd.Function`` over the
CUDA kernels:

    forward   A    = rubix_cube_fwd(particles)            (no LSF epilogue; kept)
              Q    = rubix_lsf_fwd(A, lsf taps(sigma_lsf)) (kept)
              cube = rubix_psf_fwd(Q, psf taps(sigma_psf))
    backward  gP   = PSF^T g,  h = LSF^T gP                (convolutions with reversed taps)
              particle gradients = rubix_cube_bwd(h)
              dL/dsigma_psf = <g, PSF_{dt x t}(Q)> + <g, PSF_{t x dt}(Q)>
              dL/dsigma_lsf = <gP, LSF_{dt}(A)>

The PSF and LSF act on different axes and commute, so the forward cube equals
rubix's convolve_psf followed by convolve_lsf.  With ``dust_av`` / ``dust_exponent``
(calc_dusty_ifu's calculate_extinction) every particle's spectrum carries its dust
transmission in both passes; A_V itself is held fixed (no gradient to the coordinates
or the gas).  Gradients flow to the particle
inputs (velocity: the line-of-sight component only) and to ``sigma_psf`` /
``sigma_lsf`` given as tensors; the spaxel assignment (coordinates) is piecewise
constant and gets none, as in rubix.  For sigmas given as CUDA tensors the taps and
their derivatives are computed on the device (``rubix_gauss_taps``) and read there by
the PSF/LSF kernels, so a step never reads a value back to the host.
"""

from __future__ import annotations

import numpy as np
import torch

from . import ops
from . import telescope as tel

__all__ = ["DatacubeFunction", "render_cube", "psf_taps_grad", "lsf_taps_grad"]


def psf_taps_grad(m: int, sigma: float):
    """1-D PSF taps (gaussian_kernel_2d(m, m, sigma) is their outer product) and their
    derivative with respect to sigma, float64."""
    x = np.arange(-((m - 1) / 2), ((m - 1) / 2) + 1)
    e = np.exp(-(x**2) / (2 * sigma**2))
    de = e * x**2 / sigma**3
    S = e.sum()
    t = e / S
    return t, (de - t * de.sum()) / S


def lsf_taps_grad(sigma: float, wave_res: float, factor: int = 12):
    """LSF taps of rubix/telescope/lsf/lsf.py:12-26 and their derivative, float64."""
    x = np.arange(-factor * wave_res, factor * wave_res + wave_res, wave_res,
                  dtype=np.float32).astype(np.float64)
    e = np.exp(-0.5 * x**2 / sigma**2)
    de = e * x**2 / sigma**3
    S = e.sum()
    t = e / S
    return t, (de - t * de.sum()) / S


def _psf_adjoint_taps(t: np.ndarray) -> np.ndarray:
    """Taps whose 'same' convolution (centre (m-1)//2) is the adjoint of the 'same'
    convolution with ``t``: reversed, plus a trailing zero for even m."""
    r = np.asarray(t, dtype=np.float64)[::-1]
    return r if r.size % 2 == 1 else np.concatenate([r, [0.0]])


def _psf_positions(m: int) -> np.ndarray:
    return np.arange(-((m - 1) / 2), ((m - 1) / 2) + 1)


def _lsf_positions(wave_res: float, factor: int = 12) -> np.ndarray:
    return np.arange(-factor * wave_res, factor * wave_res + wave_res, wave_res,
                     dtype=np.float32).astype(np.float64)


def _psf_taps(sigma, m: int):
    """(taps, dtaps, adjoint taps): on the device from a CUDA sigma tensor (no read-back
    of sigma), else on the host."""
    if isinstance(sigma, torch.Tensor) and sigma.is_cuda:
        return ops.gauss_taps(sigma, _psf_positions(m), reversed_pad=(m % 2 == 0))
    t, dt = psf_taps_grad(m, float(sigma))
    return t, dt, _psf_adjoint_taps(t)


def _lsf_taps(sigma, wave_res: float):
    """(taps, dtaps, reversed taps) of the LSF, on the device for a CUDA sigma tensor."""
    if isinstance(sigma, torch.Tensor) and sigma.is_cuda:
        return ops.gauss_taps(sigma, _lsf_positions(wave_res))
    t, dt = lsf_taps_grad(float(sigma), wave_res)
    return t, dt, t[::-1].copy()


class DatacubeFunction(torch.autograd.Function):
    """cube [sbin, sbin, L] = PSF(LSF(accumulate(mass, metallicity, age, velocity))).

    ``renderer`` is an ``IFURenderer`` (SSP grid, wavelength grids, bins, velocity
    axis); ``perm`` / ``seg_offsets`` its sort of the particles; ``psf_size`` the PSF
    kernel width in spaxels and ``wave_res`` the telescope wavelength step (LSF taps).
    """

    @staticmethod
    def forward(ctx, mass, metallicity, age, velocity, sigma_psf, sigma_lsf, renderer, perm,
                seg_offsets, psf_size, wave_res, dust_av=None):
        r = renderer
        nseg = r.sbin * r.sbin
        dust_e = None if dust_av is None else r.dust_exponent
        A = ops.cube_forward(r.ssp_flux, r.ssp_metallicity, r.ssp_age, r.ssp_wave_z, r.wave_t,
                             mass, metallicity, age, velocity, r.velocity_axis, perm,
                             seg_offsets, nseg, dust_av=dust_av, dust_exponent=dust_e)
        lsf_t = _lsf_taps(sigma_lsf, wave_res)
        psf_t = _psf_taps(sigma_psf, int(psf_size))
        crop = (len(lsf_t[0]) - 1) // 2
        # Q with 16-byte spaxel rows: the PSF and the sigma_PSF gradient stage them by TMA
        L = A.shape[-1]
        Q = torch.empty((nseg, (L + 3) // 4 * 4), dtype=torch.float32, device=A.device)[:, :L]
        Q = ops.lsf_forward(A, lsf_t[0], crop, out=Q)
        cube = ops.psf_forward(Q.view(r.sbin, r.sbin, -1), psf_t[0])
        ctx.save_for_backward(mass, metallicity, age, velocity, A, Q)
        ctx.r = r
        ctx.perm, ctx.seg_offsets = perm, seg_offsets
        ctx.dust = (dust_av, dust_e)
        ctx.lsf_t, ctx.psf_t, ctx.crop = lsf_t, psf_t, crop
        ctx.sigma_dtypes = (
            sigma_psf.dtype if isinstance(sigma_psf, torch.Tensor) else None,
            sigma_lsf.dtype if isinstance(sigma_lsf, torch.Tensor) else None)
        return cube

    @staticmethod
    def backward(ctx, g):
        mass, metallicity, age, velocity, A, Q = ctx.saved_tensors
        r = ctx.r
        nseg = r.sbin * r.sbin
        g = g.contiguous().float()
        tp, dtp, rtp = ctx.psf_t
        tl, dtl, rtl = ctx.lsf_t
        crop = ctx.crop
        gP = ops.psf_forward(g, rtp)
        need = ctx.needs_input_grad
        grads = [None] * 12
        want_av = len(need) > 11 and need[11]
        if any(need[:4]) or want_av:
            h = ops.lsf_forward(gP, rtl, len(tl) - 1 - crop)
            out = ops.cube_backward(
                r.ssp_flux, r.ssp_metallicity, r.ssp_age, r.ssp_wave_z, r.wave_t, mass,
                metallicity, age, velocity, r.velocity_axis, ctx.perm, ctx.seg_offsets, nseg,
                h.view(nseg, -1), dust_av=ctx.dust[0], dust_exponent=ctx.dust[1],
                av_grad=want_av)
            gm, gz, ga, gv = out[:4]
            if want_av:
                grads[11] = out[4].view_as(ctx.dust[0]).to(ctx.dust[0].dtype)
            grads[0] = gm.view_as(mass).to(mass.dtype) if need[0] else None
            grads[1] = gz.view_as(metallicity).to(metallicity.dtype) if need[1] else None
            grads[2] = ga.view_as(age).to(age.dtype) if need[2] else None
            if need[3]:
                gvel = torch.zeros_like(velocity)
                if velocity.dim() == 2:
                    gvel[:, r.velocity_axis] = gv.to(velocity.dtype)
                else:
                    gvel.copy_(gv.view_as(velocity))
                grads[3] = gvel
        if need[4]:
            Qc = Q.view(r.sbin, r.sbin, -1)
            if tp.numel() <= 21 and tp.numel() % 2 == 1:
                # <g, PSF(Q)> fused: the two convolutions are never written
                d = ops.psf_dot(Qc, dtp, tp, g) + ops.psf_dot(Qc, tp, dtp, g)
            else:
                d = (ops.dot(g, ops.psf_forward(Qc, dtp, tp))
                     + ops.dot(g, ops.psf_forward(Qc, tp, dtp)))
            grads[4] = d.to(ctx.sigma_dtypes[0] or torch.float32)
        if need[5]:
            if dtl.numel() <= 28:
                d = ops.lsf_dot(A, dtl, crop, gP.view(nseg, -1))
            else:
                d = ops.dot(gP.view(nseg, -1), ops.lsf_forward(A, dtl, crop))
            grads[5] = d.to(ctx.sigma_dtypes[1] or torch.float32)
        return tuple(grads)


class DustColumnFunction(torch.autograd.Function):
    """A_V [n_stars] of every star from the gas in front of it (rubix's
    calculate_extinction: the dust mass of each gas cell from its mass and 12 +
    log10(O/H), cells outside the aperture emptied, the cumulative column of the star's
    spaxel interpolated at the star's z; rubix/core/dust.py:16-65,
    rubix/spectra/dust/dust_extinction.py:169-343) as a differentiable function of the
    stars' coordinates (z: the x and y pick the spaxel, a piecewise-constant choice, and
    get no gradient, as in rubix) and of the gas masses and metal fractions (hydrogen and
    oxygen columns).  The gas coordinates are held fixed.  ``star_idx`` are the stars'
    spaxel assignments; ``renderer`` an ``IFURenderer`` built with ``dust``."""

    @staticmethod
    def forward(ctx, star_coords, gas_mass, gas_metals, renderer, star_idx, gas_coords):
        r = renderer
        gc = gas_coords.contiguous()
        gidx = ops.spaxel_assign(gc, r.edges)
        gm = gas_mass.contiguous()
        keep = None
        if r.apply_filter:
            keep = ops.aperture_mask(gc, r.edges)
            gm = ops.mask_zero_(gm.clone(), keep)
        gext = ops.dust_gas_extinction(gm, gas_metals, r.dgr_params, r.dgr_broken,
                                       r.ext_scale, r.spaxel_area)
        nb = int(r.edges.numel()) - 1
        nseg = r.sbin * r.sbin
        pa_limit = max(nb * nb, nseg)
        av = ops.dust_av(gc, gidx, gext, star_coords, star_idx, nseg, pa_limit)
        ctx.save_for_backward(star_coords, gm, gas_metals, gc, gidx, gext, star_idx)
        ctx.keep = keep
        ctx.r, ctx.nseg, ctx.pa_limit = r, nseg, pa_limit
        return av

    @staticmethod
    def backward(ctx, g):
        star_coords, gm, gas_metals, gc, gidx, gext, star_idx = ctx.saved_tensors
        r = ctx.r
        gz, gdext = ops.dust_av_backward(gc, gidx, gext, star_coords, star_idx, ctx.nseg,
                                         ctx.pa_limit, g.contiguous().float())
        g_coords = None
        if ctx.needs_input_grad[0]:
            g_coords = torch.zeros_like(star_coords)
            g_coords.view(-1, 3)[:, 2] = gz
        g_mass = g_met = None
        if ctx.needs_input_grad[1] or ctx.needs_input_grad[2]:
            g_mass, g_met = ops.dust_gas_extinction_backward(
                gm, gas_metals, r.dgr_params, r.dgr_broken, r.ext_scale, r.spaxel_area, gdext)
            if ctx.keep is not None:
                g_mass = ops.mask_zero_(g_mass, ctx.keep)  # emptied cells: no dependence
        return (g_coords, g_mass if ctx.needs_input_grad[1] else None,
                g_met if ctx.needs_input_grad[2] else None, None, None, None)


def render_cube(renderer, coords, velocity, mass, metallicity, age, sigma_psf, sigma_lsf,
                psf_size: int, wave_res: float, gas=None, log_age: bool = False):
    """Differentiable datacube of one galaxy: aperture filter, spaxel sort (no
    gradient) and ``DatacubeFunction``.  All particle tensors must be CUDA tensors;
    ``sigma_psf`` / ``sigma_lsf`` are tensors (or floats when no gradient is wanted).
    ``gas`` = (coords, mass, metals) with a renderer built with ``dust`` applies the dust
    extinction; gradients reach A_V and through it the stars' z and the gas masses and
    metal fractions (``DustColumnFunction``) when those require them.  With ``log_age`` the ``age``
    tensor holds log10(age / Gyr): the SSP lookup receives 10^age (float32) and the
    gradient is dL/dlog10(age) = dL/dage * age * ln 10."""
    if log_age:
        age = torch.pow(10.0, age)
    idx, mask = renderer.assign(coords)
    perm, offs = renderer.sort(idx, mask)
    av = None
    if gas is not None:
        if torch.is_grad_enabled() and (coords.requires_grad or gas[1].requires_grad
                                        or gas[2].requires_grad):
            av = DustColumnFunction.apply(coords, gas[1], gas[2], renderer, idx, gas[0])
        else:
            with torch.no_grad():
                av = renderer.dust_av(coords, idx, *gas)
    return DatacubeFunction.apply(mass, metallicity, age, velocity, sigma_psf, sigma_lsf,
                                  renderer, perm, offs, psf_size, wave_res, av)
