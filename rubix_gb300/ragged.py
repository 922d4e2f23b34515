"""Ragged batches: many galaxies with different particle counts, spaxel grids and PSF
widths rendered (and differentiated) in one launch per kernel.

rubix renders one galaxy per pipeline run (rubix/core/pipeline.py:137-170); a batch
here is the concatenation of independent galaxies that share the SSP template, the
redshift and the telescope wavelength grid.  Galaxy g owns particles
[poff[g], poff[g+1]) and the square S_g x S_g spaxel grid stored as global spaxels
[seg_base[g], seg_base[g] + S_g^2) of one concatenated cube [sum_g S_g^2, L].  Spaxel
ids are made global by ``rubix_ragged_assign``, after which the stable sort, the fused
accumulate kernel (a persistent launch over every (galaxy spaxel, particle chunk) work
item of the batch), its adjoint and the LSF run once for the whole batch; the PSF runs
as one ``rubix_ragged_psf_fwd`` launch with per-galaxy taps.  Every launch takes device
tables built once per batch, so a whole forward + backward can be captured in one CUDA
graph (``RaggedBatch.capture``).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib, ops
from . import telescope as tel
from .autograd import lsf_taps_grad, psf_taps_grad

PSF_TILE = 32  # x strip and wavelength strip of the PSF kernels
MAX_PSF_TAPS = 21


def pad_taps(t, m: int) -> np.ndarray:
    """Zero-pad 1-D PSF taps of size k to odd size m >= k so that the 'same'
    convolution (centre (size-1)//2) is unchanged: t[i] moves to i + (m-1)//2 - (k-1)//2."""
    t = np.asarray(t, dtype=np.float64)
    k = t.size
    if m % 2 == 0 or m < k:
        raise ValueError(f"pad size must be odd and >= {k}, got {m}")
    d = (m - 1) // 2 - (k - 1) // 2
    out = np.zeros(m)
    out[d:d + k] = t
    return out


def padded_size(sizes: Sequence[int]) -> int:
    m = max(int(s) for s in sizes)
    m = m if m % 2 == 1 else m + 1
    if m > MAX_PSF_TAPS:
        raise ValueError(f"PSF kernels of up to {MAX_PSF_TAPS} taps are supported, got {m}")
    return m


def adjoint_taps(t) -> np.ndarray:
    """Taps of the adjoint of the 'same' convolution with t (reversed; a trailing zero
    for even sizes keeps the centre)."""
    r = np.asarray(t, dtype=np.float64)[::-1]
    return r if r.size % 2 == 1 else np.concatenate([r, [0.0]])


@dataclass
class BatchTables:
    """Host copies of the batch layout (see module docstring)."""

    poff: np.ndarray        # int64 [n_gal+1] particle offsets
    eoff: np.ndarray        # int32 [n_gal+1] edge offsets
    edges: np.ndarray       # float32 concatenated ascending bin edges
    sbin: np.ndarray        # int32 [n_gal]
    seg_base: np.ndarray    # int64 [n_gal+1] first global spaxel of each galaxy
    block_off: np.ndarray   # int32 [n_gal+1] PSF blocks per galaxy (prefix)
    n_blocks: int

    @property
    def n_gal(self) -> int:
        return int(self.sbin.size)

    @property
    def n_segments(self) -> int:
        return int(self.seg_base[-1])


def build_tables(counts: Sequence[int], sbins: Sequence[int], edges: Sequence[np.ndarray],
                 n_wave_t: int) -> BatchTables:
    counts = np.asarray(counts, dtype=np.int64)
    sb = np.asarray(sbins, dtype=np.int64)
    if counts.size != sb.size or len(edges) != sb.size:
        raise ValueError("counts, sbins and edges must have one entry per galaxy")
    if np.any(counts < 0) or np.any(sb < 1):
        raise ValueError("particle counts must be >= 0 and spaxel grids >= 1")
    e32 = [np.asarray(e, dtype=np.float32) for e in edges]
    for e in e32:
        if e.size < 2 or np.any(np.diff(e) < 0):
            raise ValueError("each galaxy needs >= 2 ascending bin edges")
    poff = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    eoff = np.concatenate([[0], np.cumsum([e.size for e in e32])]).astype(np.int32)
    seg_base = np.concatenate([[0], np.cumsum(sb * sb)]).astype(np.int64)
    if seg_base[-1] >= 2**31:
        raise ValueError("too many spaxels in one batch")
    nl = (int(n_wave_t) + PSF_TILE - 1) // PSF_TILE
    blocks = ((sb + PSF_TILE - 1) // PSF_TILE) * nl
    block_off = np.concatenate([[0], np.cumsum(blocks)]).astype(np.int64)
    if block_off[-1] >= 2**31:
        raise ValueError("too many PSF blocks in one batch")
    return BatchTables(poff=poff, eoff=eoff, edges=np.concatenate(e32), sbin=sb.astype(np.int32),
                       seg_base=seg_base, block_off=block_off.astype(np.int32),
                       n_blocks=int(block_off[-1]))


def psf_table(taps_y: Sequence[np.ndarray], taps_x: Sequence[np.ndarray], m: int) -> np.ndarray:
    """[n_gal, 2, m] float32 table of padded (y, x) taps."""
    return np.stack([np.stack([pad_taps(ty, m), pad_taps(tx, m)])
                     for ty, tx in zip(taps_y, taps_x)]).astype(np.float32)


class RaggedBatch:
    """Device tables of one batch and the launches that render it.

    ``renderer`` supplies the shared constants (an ``IFURenderer``: SSP grid, redshifted
    SSP wavelengths, telescope grid, velocity axis); ``galaxies`` gives per galaxy its
    particle count, spaxels per side, bin edges and PSF width/size.
    """

    def __init__(self, renderer, counts, sbins, edges, psf_sigma, psf_size, lsf_sigma: float,
                 wave_res: float):
        self.r = renderer
        dev = renderer.device
        self.device = dev
        L = renderer.n_wave_t
        self.L = L
        self.t = build_tables(counts, sbins, edges, L)
        self.psf_sigma = np.asarray(psf_sigma, dtype=np.float64).reshape(-1)
        self.psf_size = np.asarray(psf_size, dtype=np.int64).reshape(-1)
        if self.psf_sigma.size != self.t.n_gal or self.psf_size.size != self.t.n_gal:
            raise ValueError("one PSF sigma and size per galaxy")
        self.lsf_sigma = float(lsf_sigma)
        self.wave_res = float(wave_res)
        self.m = padded_size(self.psf_size)
        taps = [psf_taps_grad(int(k), float(s)) for k, s in zip(self.psf_size, self.psf_sigma)]
        self.psf_t = [t for t, _ in taps]
        self.psf_dt = [d for _, d in taps]
        self.lsf_t, self.lsf_dt = lsf_taps_grad(self.lsf_sigma, self.wave_res)
        self.lsf_crop = (self.lsf_t.size - 1) // 2

        def dv(a, dtype):
            return torch.as_tensor(np.ascontiguousarray(a)).to(device=dev, dtype=dtype)

        t = self.t
        self.d_poff = dv(t.poff, torch.int64)
        self.d_eoff = dv(t.eoff, torch.int32)
        self.d_edges = dv(t.edges, torch.float32)
        self.d_sbin = dv(t.sbin, torch.int32)
        self.d_seg_base = dv(t.seg_base, torch.int64)
        self.d_block_off = dv(t.block_off, torch.int32)
        self.d_rows = self.d_seg_base * L  # element offsets of each galaxy's cube
        adj = [adjoint_taps(x) for x in self.psf_t]
        self.tab_fwd = dv(psf_table(self.psf_t, self.psf_t, self.m), torch.float32)
        self.tab_adj = dv(psf_table(adj, adj, self.m), torch.float32)
        self.tab_dy = dv(psf_table(self.psf_dt, self.psf_t, self.m), torch.float32)
        self.tab_dx = dv(psf_table(self.psf_t, self.psf_dt, self.m), torch.float32)

    @property
    def n_gal(self) -> int:
        return self.t.n_gal

    @property
    def n_segments(self) -> int:
        return self.t.n_segments

    # ------------------------------------------------------------------ launches
    def assign(self, coords: torch.Tensor):
        coords = ops._contig("coords", coords, torch.float32)
        n = coords.shape[0]
        if n != int(self.t.poff[-1]):
            raise ValueError(f"batch has {int(self.t.poff[-1])} particles, coords has {n}")
        idx = torch.empty(n, dtype=torch.int32, device=self.device)
        keep = torch.empty(n, dtype=torch.uint8, device=self.device)
        _lib.call("rubix_ragged_assign", ops._ptr(coords), n, coords.stride(0),
                  ops._ptr(self.d_poff), self.n_gal, ops._ptr(self.d_edges),
                  ops._ptr(self.d_eoff), ops._ptr(self.d_sbin), ops._ptr(self.d_seg_base),
                  ops._ptr(idx), ops._ptr(keep), ops._stream(self.device))
        ops._count(1 if n > 0 else 0)
        return idx, keep

    def sort(self, idx, keep):
        return ops.spaxel_sort(idx, self.n_segments, keep)

    def accumulate(self, mass, metallicity, age, velocity, perm, offs, with_lsf=True, out=None):
        r = self.r
        return ops.cube_forward(r.ssp_flux, r.ssp_metallicity, r.ssp_age, r.ssp_wave_z, r.wave_t,
                                mass, metallicity, age, velocity, r.velocity_axis, perm, offs,
                                self.n_segments, out=out,
                                lsf_taps=self.lsf_t if with_lsf else None, lsf_crop=self.lsf_crop)

    def psf(self, cube: torch.Tensor, table: Optional[torch.Tensor] = None, out=None):
        table = self.tab_fwd if table is None else table
        cube = cube.reshape(self.n_segments, self.L)
        if not cube.is_contiguous():
            cube = cube.contiguous()
        if out is None:
            out = torch.empty_like(cube)
        _lib.call("rubix_ragged_psf_fwd", ops._ptr(cube), ops._ptr(out), self.L, cube.stride(0),
                  out.stride(0), self.n_gal, ops._ptr(self.d_sbin), ops._ptr(self.d_seg_base),
                  ops._ptr(self.d_block_off), self.t.n_blocks, ops._ptr(table), self.m,
                  ops._stream(self.device))
        ops._count(1 if self.t.n_blocks > 0 else 0)
        return out

    def lsf(self, cube, taps=None, crop=None, out=None):
        taps = self.lsf_t if taps is None else taps
        crop = self.lsf_crop if crop is None else crop
        return ops.lsf_forward(cube.reshape(self.n_segments, self.L), taps, crop, out=out)

    def galaxy_dot(self, a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
        """[n_gal] float64: per-galaxy sum(a * b) over each galaxy's cube."""
        a = a.reshape(-1).contiguous()
        b = b.reshape(-1).contiguous()
        out = torch.empty(self.n_gal, dtype=torch.float64, device=self.device)
        ws = ops.workspace(_lib.query("rubix_segmented_dot_workspace_size", self.n_gal),
                           self.device)
        _lib.call("rubix_segmented_dot", ops._ptr(a), ops._ptr(b), ops._ptr(self.d_rows),
                  self.n_gal, ops._ptr(out), ops._ptr(ws), ws.numel(), ops._stream(self.device))
        ops._count(2 if self.n_gal > 0 else 0)
        return out

    def galaxy_view(self, cube: torch.Tensor, g: int) -> torch.Tensor:
        s0, s1 = int(self.t.seg_base[g]), int(self.t.seg_base[g + 1])
        S = int(self.t.sbin[g])
        return cube.reshape(self.n_segments, self.L)[s0:s1].view(S, S, self.L)

    # ------------------------------------------------------------------ whole path
    def render(self, coords, velocity, mass, metallicity, age):
        """Forward of the whole batch: [n_segments, L] final cubes (LSF fused into the
        accumulate kernel, then the per-galaxy PSF)."""
        idx, keep = self.assign(coords)
        perm, offs = self.sort(idx, keep)
        cube = self.accumulate(mass, metallicity, age, velocity, perm, offs, with_lsf=True)
        return self.psf(cube)

    def forward_backward(self, coords, velocity, mass, metallicity, age, target, weight,
                         keep_cube: bool = True):
        """Loss sum(weight * (cube - target)^2) over the batch and its gradients with
        respect to every particle's mass, metallicity, age and line-of-sight velocity
        and to each galaxy's PSF sigma and the shared LSF sigma.  Only device work with
        the batch's prebuilt tables: capturable in a CUDA graph.  Returns
        (loss, (d_mass, d_metallicity, d_age, d_vlos), d_sigma_psf [n_gal], d_sigma_lsf,
        cube or None); keep_cube=False reuses the cube's memory for the gradient."""
        r = self.r
        idx, keep = self.assign(coords)
        perm, offs = self.sort(idx, keep)
        A = self.accumulate(mass, metallicity, age, velocity, perm, offs, with_lsf=False)
        Q = self.lsf(A)
        cube = self.psf(Q)
        g = cube - target if keep_cube else cube.sub_(target)
        loss = torch.dot((g * g).view(-1), weight.reshape(-1))
        g.mul_(weight).mul_(2.0)
        gP = self.psf(g, self.tab_adj)
        h = self.lsf(gP, self.lsf_t[::-1].copy(), self.lsf_t.size - 1 - self.lsf_crop)
        grads = ops.cube_backward(r.ssp_flux, r.ssp_metallicity, r.ssp_age, r.ssp_wave_z,
                                  r.wave_t, mass, metallicity, age, velocity, r.velocity_axis,
                                  perm, offs, self.n_segments, h)
        del h
        d_psf = self.galaxy_dot(g, self.psf(Q, self.tab_dy))
        d_psf = d_psf + self.galaxy_dot(g, self.psf(Q, self.tab_dx))
        d_lsf = ops.dot(gP, self.lsf(A, self.lsf_dt, self.lsf_crop))
        return loss, grads, d_psf, d_lsf, (cube if keep_cube else None)

    def capture(self, fn, *args, warmup: int = 2):
        """Record ``fn(*args)`` (e.g. ``self.forward_backward``) in a CUDA graph after
        ``warmup`` eager runs on a side stream; returns (graph, static outputs)."""
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            for _ in range(warmup):
                fn(*args)
        torch.cuda.current_stream(self.device).wait_stream(s)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            out = fn(*args)
        return graph, out


def synthetic_batch_spec(n_gal: int = 256, n_min: float = 1e3, n_max: float = 1e6,
                         s_min: int = 16, s_max: int = 64, sigma_min: float = 0.8,
                         sigma_max: float = 2.0, seed: int = 4):
    """Seeded ragged batch layout: particle counts log-uniform in [n_min, n_max], spaxels
    per side uniform in [s_min, s_max], PSF sigma uniform in [sigma_min, sigma_max]
    (kernel size 2*ceil(3 sigma)+1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    counts = np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_gal)).astype(np.int64)
    sbins = rng.integers(s_min, s_max + 1, n_gal)
    sig = rng.uniform(sigma_min, sigma_max, n_gal)
    sizes = 2 * np.ceil(3 * sig).astype(np.int64) + 1
    return counts, sbins, sig, sizes


def galaxy_edges(sbin: int, dist_z: float, spatial_res: float = 0.2) -> np.ndarray:
    edges, _ = tel.spatial_bin_edges(sbin * spatial_res, sbin, dist_z)
    return edges


def render_per_galaxy(batch: RaggedBatch, coords, velocity, mass, metallicity, age):
    """The same batch rendered galaxy by galaxy with the single-galaxy launches (the
    loop a ragged launch replaces); returns the concatenated [n_segments, L] cubes."""
    r = batch.r
    out = torch.empty((batch.n_segments, batch.L), dtype=torch.float32, device=batch.device)
    edges_d = batch.d_edges
    for g in range(batch.n_gal):
        p0, p1 = int(batch.t.poff[g]), int(batch.t.poff[g + 1])
        e0, e1 = int(batch.t.eoff[g]), int(batch.t.eoff[g + 1])
        S = int(batch.t.sbin[g])
        s0, s1 = int(batch.t.seg_base[g]), int(batch.t.seg_base[g + 1])
        c = coords[p0:p1]
        e = edges_d[e0:e1]
        idx = ops.spaxel_assign(c, e)
        keep = ops.aperture_mask(c, e)
        perm, offs = ops.spaxel_sort(idx, S * S, keep)
        cube = ops.cube_forward(r.ssp_flux, r.ssp_metallicity, r.ssp_age, r.ssp_wave_z, r.wave_t,
                                mass[p0:p1], metallicity[p0:p1], age[p0:p1], velocity[p0:p1],
                                r.velocity_axis, perm, offs, S * S, lsf_taps=batch.lsf_t,
                                lsf_crop=batch.lsf_crop)
        ops.psf_forward(cube.view(S, S, batch.L), batch.psf_t[g],
                        out=out[s0:s1].view(S, S, batch.L))
    return out


def forward_backward_per_galaxy(batch: RaggedBatch, coords, velocity, mass, metallicity, age,
                                target, weight):
    """``RaggedBatch.forward_backward`` galaxy by galaxy through ``DatacubeFunction``."""
    from .autograd import render_cube
    from .api import IFURenderer

    r = batch.r
    grads = [torch.zeros_like(mass), torch.zeros_like(metallicity), torch.zeros_like(age),
             torch.zeros(mass.shape[0], dtype=torch.float32, device=batch.device)]
    d_psf = torch.zeros(batch.n_gal, dtype=torch.float64, device=batch.device)
    d_lsf = torch.zeros((), dtype=torch.float64, device=batch.device)
    loss = torch.zeros((), dtype=torch.float32, device=batch.device)
    for g in range(batch.n_gal):
        p0, p1 = int(batch.t.poff[g]), int(batch.t.poff[g + 1])
        e0, e1 = int(batch.t.eoff[g]), int(batch.t.eoff[g + 1])
        S = int(batch.t.sbin[g])
        s0, s1 = int(batch.t.seg_base[g]), int(batch.t.seg_base[g + 1])
        rg = IFURenderer.__new__(IFURenderer)
        rg.__dict__.update(r.__dict__)
        rg.edges = batch.d_edges[e0:e1]
        rg.sbin = S
        m = mass[p0:p1].detach().clone().requires_grad_()
        z = metallicity[p0:p1].detach().clone().requires_grad_()
        a = age[p0:p1].detach().clone().requires_grad_()
        v = velocity[p0:p1].detach().clone().requires_grad_()
        sp = torch.tensor(float(batch.psf_sigma[g]), dtype=torch.float64, device=batch.device,
                          requires_grad=True)
        sl = torch.tensor(batch.lsf_sigma, dtype=torch.float64, device=batch.device,
                          requires_grad=True)
        cube = render_cube(rg, coords[p0:p1], v, m, z, a, sp, sl, int(batch.psf_size[g]),
                           batch.wave_res)
        tg = target[s0:s1].view(S, S, batch.L)
        wg = weight[s0:s1].view(S, S, batch.L)
        diff = cube - tg
        lg = (wg * diff * diff).sum()
        lg.backward()
        loss = loss + lg.detach()
        grads[0][p0:p1] = m.grad
        grads[1][p0:p1] = z.grad
        grads[2][p0:p1] = a.grad
        grads[3][p0:p1] = v.grad[:, r.velocity_axis]
        d_psf[g] = sp.grad
        d_lsf = d_lsf + sl.grad
    return loss, tuple(grads), d_psf, d_lsf
