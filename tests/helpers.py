"""Shared helpers for the test-suite (workload caching, oracle runs, device upload)."""

from __future__ import annotations

import functools

import numpy as np

import oracle
from rubix_gb300 import synth

# Tolerance of every FP32-vs-FP64-oracle cube comparison: relative error 1e-5,
# normwise (max |gpu - oracle| / max |oracle|) and elementwise on the elements
# whose oracle value exceeds 1e-3 of the cube maximum.
CUBE_RTOL = 1e-5


@functools.lru_cache(maxsize=8)
def workload(name: str, n: int | None = None, n_wave_t: int | None = None, edge_cases=True):
    return synth.make_workload(name, n=n, n_wave_t=n_wave_t, edge_cases=edge_cases)


@functools.lru_cache(maxsize=8)
def oracle_stages(name: str, n: int | None = None, n_wave_t: int | None = None,
                  edge_cases=True, with_psf_lsf=True):
    w = workload(name, n, n_wave_t, edge_cases)
    p = w.particles
    return oracle.render_cube(
        p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges, w.sbin,
        w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.ssp.wavelength, w.dist_z, w.wave_t,
        psf_size=w.psf_size if with_psf_lsf else None, psf_sigma=w.psf_sigma,
        lsf_sigma=w.lsf_sigma if with_psf_lsf else None, wave_res=w.wave_res,
    )


def to_dev(a, dtype=None):
    import torch

    t = torch.as_tensor(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def assert_cube_close(test, ref, rtol=CUBE_RTOL, what="cube"):
    norm, elem = oracle.cube_rel_error(test, ref)
    assert norm <= rtol and elem <= rtol, (
        f"{what}: normwise rel err {norm:.3e}, elementwise rel err {elem:.3e} > {rtol:g}"
    )
    return norm, elem
