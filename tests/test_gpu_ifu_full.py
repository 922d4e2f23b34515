"""Every spaxel of the 10^6-particle IFU workload against the float64 oracle.

Workload ``ifu``: 10^6 particles (exponential disk) plus the edge-case particles,
150 x 150 spaxels x 3721 wavelengths, SSP grid 221 ages x 6 metallicities x 1221
wavelengths, PSF 15 x 15 sigma 1.5, LSF sigma 1.2 A.  The oracle's per-spaxel sums of
all particles (rubix/core/ifu.py:63-341, rubix/spectra/ifu.py:168-288) run on every
host core (oracle/pool.py); the whole accumulated cube and the whole final cube (PSF
and LSF: rubix/telescope/psf/psf.py:33-58, rubix/telescope/lsf/lsf.py:29-105, applied
by the oracle to its own cube) are compared within 1e-5, normwise and elementwise,
with the errors printed.
"""

import numpy as np
import pytest

import oracle
from helpers import CUBE_RTOL, to_dev, workload

pytestmark = pytest.mark.gpu


def test_ifu_whole_cube_vs_oracle(rubix_lib):
    import torch

    from oracle import pool
    from rubix_gb300.api import IFURenderer

    w = workload("ifu")
    p = w.particles
    S, L = w.sbin, w.wave_t.size
    r = IFURenderer.from_workload(w)
    d = [to_dev(a) for a in (p.coords, p.velocity, p.mass, p.metallicity, p.age)]
    idx, mask = r.assign(d[0])
    perm, offs = r.sort(idx, mask)
    raw = r.accumulate(d[2], d[3], d[4], d[1], perm, offs)
    final = r.psf(r.accumulate(d[2], d[3], d[4], d[1], perm, offs, with_lsf=True))
    torch.cuda.synchronize()

    # the oracle cube, spaxel by spaxel (filter_particles applied; ids >= S^2 dropped)
    li = oracle.square_spaxel_assignment(p.coords, w.edges)
    keep = oracle.mask_particles_outside_aperture(p.coords, w.edges) & (li < S * S)
    order = np.argsort(np.where(keep, li, S * S), kind="stable")
    counts = np.bincount(li[keep], minlength=S * S)
    segs = np.nonzero(counts)[0]
    starts = np.concatenate([[0], np.cumsum(counts)])
    groups = []
    for s in segs:
        j = order[starts[s]:starts[s + 1]]
        groups.append((p.mass[j], p.metallicity[j], p.age[j], p.velocity[j, 2]))
    sums = pool.spaxel_spectra(groups, w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z,
                               w.wave_t)
    want = np.zeros((S * S, L))
    want[segs] = sums
    want = want.reshape(S, S, L)

    got = raw.cpu().numpy()
    norm, elem = oracle.cube_rel_error(got, want)
    empty = ~np.isin(np.arange(S * S), segs)
    print(f"ifu accumulated cube, all {S * S} spaxels ({int(keep.sum())} particles): "
          f"normwise {norm:.2e}, elementwise {elem:.2e}; empty spaxels all zero: "
          f"{not got.reshape(S * S, L)[empty].any()}")
    assert norm <= CUBE_RTOL and elem <= CUBE_RTOL
    assert not got.reshape(S * S, L)[empty].any()

    K = oracle.gaussian_kernel_2d(w.psf_size, w.psf_size, w.psf_sigma)
    want_f = oracle.apply_lsf(oracle.apply_psf(want, K), w.lsf_sigma, w.wave_res)
    norm_f, elem_f = oracle.cube_rel_error(final.cpu().numpy(), want_f)
    print(f"ifu final cube (LSF in the accumulate epilogue, then PSF): normwise "
          f"{norm_f:.2e}, elementwise {elem_f:.2e}")
    assert norm_f <= CUBE_RTOL and elem_f <= CUBE_RTOL
