"""Process-pool runner of the oracle over many particles (TEST INFRASTRUCTURE ONLY).

The float64 oracle renders about 3000 particles per second on one host core, so the
parity checks of the 10^7-particle workload (a spaxel of its bulge holds ~1.5e5
particles) spread the per-spaxel sums over the host cores.  The pool is started with
the ``spawn`` method, which is safe in a process that has already initialised CUDA
(a forked child of such a process can hang).  Each worker receives the SSP grid and
the wavelength grids once, through the pool initializer.
"""

from __future__ import annotations

import multiprocessing as mp
import os

import numpy as np

from .ifu_oracle import particle_spectra

_GRID = {}


def _init(ssp_metallicity, ssp_age, ssp_flux, wave_z, wave_t):
    _GRID.update(ssp_metallicity=ssp_metallicity, ssp_age=ssp_age, ssp_flux=ssp_flux,
                 wave_z=wave_z, wave_t=wave_t)


def _sum_job(job):
    """Per-group sums of the float64 resampled, mass-scaled spectra of one block of
    particles (the per-spaxel segment sum of calculate_cube, rubix/spectra/ifu.py:
    270-288); returns (group ids, sums)."""
    gid, mass, met, age, vz = job
    g = _GRID
    uniq, inv = np.unique(gid, return_inverse=True)
    tot = np.zeros((uniq.size, g["wave_t"].size))
    for s in range(0, mass.size, 512):
        sp = particle_spectra(mass[s:s + 512], met[s:s + 512], age[s:s + 512], vz[s:s + 512],
                              g["ssp_metallicity"], g["ssp_age"], g["ssp_flux"], g["wave_z"],
                              g["wave_t"])
        np.add.at(tot, inv[s:s + 512], sp)
    return uniq, tot


def spaxel_spectra(groups, ssp_metallicity, ssp_age, ssp_flux, wave_z, wave_t,
                   processes=None, block=4096):
    """float64 oracle spectrum of each group of particles, summed over the group.

    ``groups``: list of (mass, metallicity, age, v_los) arrays, one tuple per spaxel
    (the particles assigned to it, filter_particles already applied).  Returns an
    (n_groups, L) float64 array.  The particles of all groups, in group order, are cut
    into blocks of ``block`` that run in parallel on ``processes`` workers (default:
    every host core); a block may hold many small groups or part of a large one."""
    L = np.asarray(wave_t).size
    out = np.zeros((len(groups), L))
    sizes = np.array([np.size(gr[0]) for gr in groups], dtype=np.int64)
    if sizes.sum() == 0:
        return out
    gid = np.repeat(np.arange(len(groups)), sizes)
    cols = [np.concatenate([np.asarray(gr[k], dtype=np.float32) for gr in groups])
            for k in range(4)]
    jobs = [(gid[s:s + block], *(c[s:s + block] for c in cols))
            for s in range(0, gid.size, block)]
    n_proc = max(1, min(processes or os.cpu_count() or 1, len(jobs)))
    grid = (np.asarray(ssp_metallicity), np.asarray(ssp_age), np.asarray(ssp_flux),
            np.asarray(wave_z), np.asarray(wave_t))
    if n_proc == 1:
        _init(*grid)
        res = [_sum_job(j) for j in jobs]
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(n_proc, initializer=_init, initargs=grid) as pool:
            res = pool.map(_sum_job, jobs, chunksize=1)
    for uniq, tot in res:
        out[uniq] += tot
    return out
