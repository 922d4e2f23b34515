"""SSP grids too large for the staged shared-memory layout: the accumulate kernel reads
corner entries and SSP wavelengths through L1/L2 (one or two rows in the pool), the
adjoint likewise.  Parity with the oracle at 2500 (staged, one block per SM), 6000 and
12 000 SSP wavelengths, gradients at 6000, and the refusal beyond the limits."""

import dataclasses

import numpy as np
import pytest

import oracle
from helpers import assert_cube_close, to_dev, workload

pytestmark = pytest.mark.gpu


def _large_workload(n_wave, n=1500):
    from rubix_gb300 import synth

    base = workload("small", n=n)
    ssp = synth.make_ssp(8, 4, n_wave, seed=11)
    return dataclasses.replace(base, ssp=ssp,
                               wave_z=oracle.cosmological_doppler_shift(base.dist_z,
                                                                        ssp.wavelength))


def _cube(w):
    import torch

    from rubix_gb300 import ops

    p = w.particles
    idx = oracle.square_spaxel_assignment(p.coords, w.edges)
    nseg = w.sbin * w.sbin
    perm, offs = ops.spaxel_sort(to_dev(idx, torch.int32), nseg)
    cube = ops.cube_forward(to_dev(w.ssp.flux), to_dev(w.ssp.metallicity), to_dev(w.ssp.age),
                            to_dev(w.wave_z), to_dev(w.wave_t), to_dev(p.mass),
                            to_dev(p.metallicity), to_dev(p.age), to_dev(p.velocity), 2, perm,
                            offs, nseg, check=True)
    return cube.reshape(w.sbin, w.sbin, -1).cpu().numpy(), idx, perm, offs


@pytest.mark.parametrize("n_wave", [2500, 6000, 12000])
def test_large_grid_forward(n_wave):
    w = _large_workload(n_wave)
    p = w.particles
    got, *_ = _cube(w)
    ref = oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                             w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux,
                             w.ssp.wavelength, w.dist_z, w.wave_t, apply_filter=False)
    assert_cube_close(got, ref["cube"], what=f"cube with {n_wave} SSP wavelengths")


def test_large_grid_adjoint():
    import torch

    from rubix_gb300 import ops
    from test_gpu_grad import _compare

    w = _large_workload(6000, n=1200)
    p = w.particles
    L = w.wave_t.size
    _, idx, perm, offs = _cube(w)
    nseg = w.sbin * w.sbin
    adj = np.random.default_rng(5).standard_normal((nseg, L)).astype(np.float32)
    got = ops.cube_backward(to_dev(w.ssp.flux), to_dev(w.ssp.metallicity), to_dev(w.ssp.age),
                            to_dev(w.wave_z), to_dev(w.wave_t), to_dev(p.mass),
                            to_dev(p.metallicity), to_dev(p.age), to_dev(p.velocity), 2, perm,
                            offs, nseg, to_dev(adj))
    want = oracle.particle_grads(p.mass, p.metallicity, p.age, p.velocity[:, 2],
                                 w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z, w.wave_t,
                                 adj.astype(np.float64)[idx.astype(np.int64)])
    for name, g, wv in zip(("mass", "metallicity", "age", "v_los"), got, want):
        _compare(f"dL/d{name} ({w.ssp.wavelength.size} SSP wavelengths)", g.cpu().numpy(), wv)


def test_too_large_grids_are_refused():
    from rubix_gb300 import _lib, ops

    w = _large_workload(16000, n=50)
    with pytest.raises(_lib.RubixError, match="shared memory"):
        _cube(w)
    w = _large_workload(7000, n=50)
    _, idx, perm, offs = _cube(w)
    p = w.particles
    nseg = w.sbin * w.sbin
    adj = to_dev(np.zeros((nseg, w.wave_t.size), np.float32))
    with pytest.raises(_lib.RubixError, match="shared memory"):
        ops.cube_backward(to_dev(w.ssp.flux), to_dev(w.ssp.metallicity), to_dev(w.ssp.age),
                          to_dev(w.wave_z), to_dev(w.wave_t), to_dev(p.mass),
                          to_dev(p.metallicity), to_dev(p.age), to_dev(p.velocity), 2, perm,
                          offs, nseg, adj)
