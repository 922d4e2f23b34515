"""Edge cases of the CUDA path against the oracle: empty inputs, no particle inside the
aperture, one particle, particles outside the SSP grid, zero masses, the maximum
telescope grid, non-uniform telescope grids, a spaxel holding many chunks, and the
argument checks of the C ABI."""

import numpy as np
import pytest

import oracle
from helpers import assert_cube_close, to_dev, workload

pytestmark = pytest.mark.gpu


def _render(w, p, **kw):
    from rubix_gb300.api import IFURenderer

    r = IFURenderer.from_workload(w, **kw)
    return r.render(to_dev(p.coords), to_dev(p.velocity), to_dev(p.mass),
                    to_dev(p.metallicity), to_dev(p.age))


def _oracle(w, p, psf=True, lsf=True):
    return oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                              w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux,
                              w.ssp.wavelength, w.dist_z, w.wave_t,
                              psf_size=w.psf_size if psf else None, psf_sigma=w.psf_sigma,
                              lsf_sigma=w.lsf_sigma if lsf else None, wave_res=w.wave_res)


def _subset(p, sel):
    from rubix_gb300.synth import ParticleData

    return ParticleData(coords=p.coords[sel], velocity=p.velocity[sel], mass=p.mass[sel],
                        metallicity=p.metallicity[sel], age=p.age[sel])


def test_no_particles():
    w = workload("small", n=50, n_wave_t=256, edge_cases=False)
    p = _subset(w.particles, np.zeros(0, dtype=np.int64))
    st = _render(w, p)
    assert st.final.shape == (w.sbin, w.sbin, 256) and not st.final.any()


def test_all_outside_the_aperture():
    w = workload("small", n=200, n_wave_t=256, edge_cases=False)
    p = _subset(w.particles, np.arange(200))
    p.coords[:, 0] = float(w.edges[-1]) * 3.0  # everything to the right of the field
    st = _render(w, p)
    assert not st.final.any() and not st.mask.any()


def test_single_particle_and_edge_cases():
    w = workload("small", n=0, n_wave_t=512)  # only the 14 edge-case particles
    p = w.particles
    ref = _oracle(w, p)
    assert_cube_close(_render(w, p).final.cpu().numpy(), ref["final"], what="edge cases")
    one = _subset(p, np.array([8]))  # on interior grid nodes, receding 300 km/s
    ref1 = _oracle(w, one)
    assert_cube_close(_render(w, one).final.cpu().numpy(), ref1["final"], what="one particle")


def test_outside_ssp_grid_and_zero_mass_contribute_nothing():
    w = workload("small", n=0, n_wave_t=256)
    p = w.particles
    # edge cases 9 (older than the grid), 10/11 (Z outside), 12 (zero mass)
    sub = _subset(p, np.array([9, 10, 11, 12]))
    st = _render(w, sub, psf=False, lsf=False)
    assert not st.final.any()


def test_non_uniform_telescope_grid():
    from rubix_gb300 import synth

    w = synth.make_workload("small", n=800)
    # log-spaced telescope grid with bins from 0.9 to 2.2 A: the general walk
    wt = np.geomspace(4700.0, 9300.0, 2000).astype(np.float32)
    w.wave_t = wt
    p = w.particles
    ref = oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                             w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.ssp.wavelength,
                             w.dist_z, wt)
    got = _render(w, p, psf=False, lsf=False).final.cpu().numpy()
    assert_cube_close(got, ref["final"], what="log-spaced telescope grid")


def test_maximum_telescope_grid():
    from rubix_gb300 import synth

    w = synth.make_workload("small", n=300)
    w.wave_t = np.linspace(4000.0, 9500.0, 4096).astype(np.float32)  # kMaxWaveT
    p = w.particles
    ref = oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                             w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.ssp.wavelength,
                             w.dist_z, w.wave_t)
    got = _render(w, p, psf=False, lsf=False).final.cpu().numpy()
    assert_cube_close(got, ref["final"], what="4096 telescope wavelengths")


def test_dense_spaxel_many_chunks():
    """Thousands of particles in one spaxel: chunks, partial spectra and their merge."""
    from rubix_gb300 import synth

    w = synth.make_workload("small", n=5000, n_wave_t=256, edge_cases=False)
    p = w.particles
    c = 0.5 * (w.edges[12] + w.edges[13])
    p.coords[:3000, 0] = c
    p.coords[:3000, 1] = c
    ref = _oracle(w, p, psf=False, lsf=False)
    got = _render(w, p, psf=False, lsf=False).final.cpu().numpy()
    assert_cube_close(got, ref["final"], what="dense spaxel")


def test_capi_rejects_bad_arguments():
    import torch

    from rubix_gb300 import _lib, ops

    w = workload("small", n=10, n_wave_t=64)
    dev = [to_dev(x) for x in (w.ssp.flux, w.ssp.metallicity, w.ssp.age, w.wave_z, w.wave_t)]
    idx = torch.zeros(4, dtype=torch.int32, device="cuda")
    perm, offs = ops.spaxel_sort(idx, 1)
    m = torch.ones(4, device="cuda")
    v = torch.zeros(4, 3, device="cuda")
    too_many = torch.zeros(5000, device="cuda")
    with pytest.raises(_lib.RubixError):  # more telescope wavelengths than supported
        ops.cube_forward(*dev[:4], too_many, m, m, m, v, 2, perm, offs, 1)
    with pytest.raises(_lib.RubixError):  # velocity component outside the row
        ops.cube_forward(*dev, m, m, m, v, 3, perm, offs, 1)
    with pytest.raises(_lib.RubixError):  # PSF kernel wider than supported
        ops.psf_forward(torch.zeros(4, 4, 8, device="cuda"), np.ones(65))
    with pytest.raises(ValueError):  # CPU tensors never reach the library
        ops.psf_forward(torch.zeros(4, 4, 8), np.ones(3))


def test_fma_probe_runs():
    """bench.py's FP32 rate probe (a bench-only library) launches, writes one finite value
    per thread and reports its FMA count."""
    import os
    import sys

    import torch

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    n_fma, out = bench.fma_probe("cuda", iters=8)
    torch.cuda.synchronize()
    assert n_fma == out.numel() * 8 * 128
    assert torch.isfinite(out).all()
