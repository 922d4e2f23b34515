"""Parity on the 10^7-particle workload the throughput target is stated on.

Workload ``large``: an exponential disk plus a Plummer bulge (a = 1 kpc) holding 30 %
of the particles, 10^7 particles (plus the edge-case particles), 300 x 300 spaxels x
3721 wavelengths (a 1.34 GB float32 cube), SSP grid 221 ages x 6 metallicities x 1221
wavelengths, PSF 15 x 15 with sigma 1.5 spaxel, LSF sigma 1.2 A, noise at S/N 20.
The bulge puts ~1.5e5 particles into each central spaxel: the deepest chunked merges
of the accumulate kernel.

Checked here, with the error of every comparison printed:
* spaxel indices and the aperture mask of all particles, bit-exact against the oracle's
  square_spaxel_assignment / mask (rubix/telescope/utils.py:78-178);
* the sort: stable permutation and segment offsets against numpy's stable argsort;
* the accumulated cube (lookup, mass, Doppler, resampling, per-spaxel sum:
  rubix/core/ifu.py:63-341, rubix/spectra/ifu.py:168-288) within 1e-5 of the float64
  oracle on 32 spaxels: the 5 densest bulge spaxels and 27 seeded random non-empty
  ones, normwise per spaxel and elementwise;
* run-to-run bitwise equality of the whole cube;
* PSF and LSF (rubix/telescope/psf/psf.py:33-58, rubix/telescope/lsf/lsf.py:29-105) of
  the full-size cube against the oracle's convolutions of the same accumulated cube on
  two windows (the bulge centre, and the cube corner where the zero padding acts);
* the noise step: rubix takes the median of where(flux > 0, flux, nan), which is NaN
  when any spaxel is empty -- as here -- so no noise is added (the cube is unchanged).
"""

import numpy as np
import pytest

import oracle
from helpers import CUBE_RTOL, to_dev, workload

pytestmark = pytest.mark.gpu

N_DENSE, N_RANDOM = 5, 27


@pytest.fixture(scope="module")
def large(rubix_lib):
    import torch

    from rubix_gb300.api import IFURenderer

    w = workload("large")
    p = w.particles
    r = IFURenderer.from_workload(w)
    d = [to_dev(a) for a in (p.coords, p.velocity, p.mass, p.metallicity, p.age)]
    idx, mask = r.assign(d[0])
    perm, offs = r.sort(idx, mask)
    raw = r.accumulate(d[2], d[3], d[4], d[1], perm, offs)
    raw_again = r.accumulate(d[2], d[3], d[4], d[1], perm, offs)
    same = bool(torch.equal(raw, raw_again))
    del raw_again
    fused = r.accumulate(d[2], d[3], d[4], d[1], perm, offs, with_lsf=True)
    final = r.psf(fused)
    del fused
    noisy = r.noise_(final.clone())
    torch.cuda.synchronize()
    idx_ref = oracle.square_spaxel_assignment(p.coords, w.edges)
    mask_ref = oracle.mask_particles_outside_aperture(p.coords, w.edges)
    return dict(w=w, r=r, idx=idx, mask=mask, perm=perm, offs=offs, raw=raw, same=same,
                final=final, noisy=noisy, idx_ref=idx_ref, mask_ref=mask_ref)


def test_large_indices_bit_exact(large):
    idx = large["idx"].cpu().numpy()
    mask = large["mask"].cpu().numpy().astype(bool)
    n_idx = int(np.sum(idx != large["idx_ref"]))
    n_mask = int(np.sum(mask != large["mask_ref"]))
    print(f"large: {idx.size} particles, spaxel index mismatches {n_idx}, mask mismatches "
          f"{n_mask}")
    assert n_idx == 0 and n_mask == 0


def test_large_sort_stable(large):
    w = large["w"]
    nseg = w.sbin * w.sbin
    idx, keep = large["idx_ref"], large["mask_ref"]
    valid = keep & (idx >= 0) & (idx < nseg)
    key = np.where(valid, idx, nseg)
    order = np.argsort(key, kind="stable")
    nv = int(valid.sum())
    perm = large["perm"].cpu().numpy()
    offs = large["offs"].cpu().numpy()
    assert offs[0] == 0 and offs[nseg] == nv
    assert np.array_equal(np.diff(offs), np.bincount(key[valid], minlength=nseg))
    assert np.array_equal(perm[:nv], order[:nv])


def _sampled_spaxels(large):
    w = large["w"]
    nseg = w.sbin * w.sbin
    idx, keep = large["idx_ref"], large["mask_ref"]
    counts = np.bincount(idx[keep], minlength=nseg)
    dense = np.argsort(-counts, kind="stable")[:N_DENSE]
    others = np.setdiff1d(np.nonzero(counts)[0], dense)
    rnd = np.random.default_rng(5).choice(others, N_RANDOM, replace=False)
    return np.concatenate([dense, np.sort(rnd)]), counts


def test_large_cube_sampled_spaxels_vs_oracle(large):
    from oracle import pool

    w = large["w"]
    p = w.particles
    L = w.wave_t.size
    segs, counts = _sampled_spaxels(large)
    idx, keep = large["idx_ref"], large["mask_ref"]
    order = np.argsort(idx, kind="stable")
    starts = np.searchsorted(idx[order], segs)
    groups = []
    for s, b in zip(segs, starts):
        j = order[b:b + np.count_nonzero(idx == s)]
        j = j[keep[j]]
        groups.append((p.mass[j], p.metallicity[j], p.age[j], p.velocity[j, 2]))
    want = pool.spaxel_spectra(groups, w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z,
                               w.wave_t)
    got = large["raw"].view(-1, L)[to_dev(segs.astype(np.int64))].cpu().numpy()
    per = []
    for k, s in enumerate(segs):
        scale = np.abs(want[k]).max()
        per.append(np.abs(got[k] - want[k]).max() / scale if scale > 0 else
                   np.abs(got[k]).max())
    norm, elem = oracle.cube_rel_error(got, want)
    print(f"large cube, {len(segs)} spaxels ({int(counts[segs].sum())} particles; densest "
          f"{counts[segs[:N_DENSE]].tolist()}): normwise {norm:.2e}, elementwise {elem:.2e}, "
          f"worst per-spaxel normwise {max(per):.2e}")
    assert max(per) <= CUBE_RTOL
    assert norm <= CUBE_RTOL and elem <= CUBE_RTOL


def test_large_cube_bitwise_reproducible(large):
    assert large["same"], "two accumulate launches on the same inputs differ"


@pytest.mark.parametrize("where", ["bulge_centre", "corner"])
def test_large_psf_lsf_windows(large, where):
    w = large["w"]
    S, L = w.sbin, w.wave_t.size
    h = (w.psf_size - 1) // 2
    if where == "corner":
        y0, x0, n = 0, 0, 4 * h
        inner = (slice(0, 3 * h), slice(0, 3 * h))  # cube edges are real edges here
    else:
        segs, _ = _sampled_spaxels(large)
        cy, cx = divmod(int(segs[0]), S)
        y0, x0, n = cy - 2 * h, cx - 2 * h, 4 * h + 1
        inner = (slice(h, n - h), slice(h, n - h))
    raw = large["raw"][y0:y0 + n, x0:x0 + n].cpu().numpy().astype(np.float64)
    K = oracle.gaussian_kernel_2d(w.psf_size, w.psf_size, w.psf_sigma)
    want = oracle.apply_lsf(oracle.apply_psf(raw, K), w.lsf_sigma, w.wave_res)[inner]
    got = large["final"][y0:y0 + n, x0:x0 + n].cpu().numpy()[inner]
    norm, elem = oracle.cube_rel_error(got, want)
    print(f"large PSF+LSF window at {where} ({y0},{x0}): normwise {norm:.2e}, "
          f"elementwise {elem:.2e}")
    assert np.abs(want).max() > 0
    assert norm <= CUBE_RTOL and elem <= CUBE_RTOL


def test_large_noise_follows_rubix_median_rule(large):
    import torch

    from rubix_gb300 import ops

    flux = ops.flux_image(large["final"])
    n_empty = int((flux <= 0).sum())
    print(f"large: {n_empty} of {flux.numel()} spaxels have no flux after the PSF")
    assert n_empty > 0
    assert torch.equal(large["noisy"], large["final"])
