"""GPU parity of each kernel against the oracle, through the C ABI (via rubix_gb300.ops)."""

import numpy as np
import pytest

import oracle
from helpers import assert_cube_close, oracle_stages, to_dev, workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ops(rubix_lib):
    from rubix_gb300 import ops as _ops

    return _ops


def test_spaxel_assign_bit_exact(ops):
    w = workload("small")
    p = w.particles
    got = ops.spaxel_assign(to_dev(p.coords), to_dev(w.edges)).cpu().numpy()
    ref = oracle.square_spaxel_assignment(p.coords, w.edges)
    assert got.dtype == np.int32
    assert np.array_equal(got, ref), f"{np.sum(got != ref)} spaxel index mismatches"


def test_spaxel_assign_reference_example(ops):
    # tests/test_telescope_utils.py:20-35 of rubix: two particles -> [4, 14]
    import torch

    coords = torch.tensor([[0.5, 1.5], [2.5, 3.5]], dtype=torch.float32).cuda()
    edges = torch.tensor([0, 1, 2, 3, 4], dtype=torch.float32).cuda()
    assert ops.spaxel_assign(coords, edges).cpu().tolist() == [4, 14]


def test_aperture_mask_bit_exact(ops):
    w = workload("small")
    p = w.particles
    got = ops.aperture_mask(to_dev(p.coords), to_dev(w.edges)).cpu().numpy().astype(bool)
    ref = oracle.mask_particles_outside_aperture(p.coords, w.edges)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("n,nseg", [(0, 10), (1, 1), (1000, 7), (100_003, 625), (300_000, 90_000)])
def test_spaxel_sort_stable(ops, n, nseg):
    import torch

    rng = np.random.default_rng(n + nseg)
    idx = rng.integers(-2, nseg + 3, n).astype(np.int32)
    keep = (rng.random(n) > 0.1).astype(np.uint8)
    perm, offs = ops.spaxel_sort(to_dev(idx), nseg, to_dev(keep))
    perm, offs = perm.cpu().numpy(), offs.cpu().numpy()
    valid = (keep != 0) & (idx >= 0) & (idx < nseg)
    key = np.where(valid, idx, nseg)
    order = np.argsort(key, kind="stable")
    nv = int(valid.sum())
    assert offs[nseg] == nv
    assert np.array_equal(perm[:nv], order[:nv])
    counts = np.bincount(key[valid], minlength=nseg)
    assert np.array_equal(np.diff(offs), counts)
    assert offs[0] == 0
    torch.cuda.synchronize()


def _cube_small(ops, w, keep=True):
    import torch

    p = w.particles
    dev_coords = to_dev(p.coords)
    edges = to_dev(w.edges)
    idx = ops.spaxel_assign(dev_coords, edges)
    mask = ops.aperture_mask(dev_coords, edges) if keep else None
    nseg = w.sbin * w.sbin
    perm, offs = ops.spaxel_sort(idx, nseg, mask)
    cube = ops.cube_forward(
        to_dev(w.ssp.flux), to_dev(w.ssp.metallicity), to_dev(w.ssp.age), to_dev(w.wave_z),
        to_dev(w.wave_t), to_dev(p.mass), to_dev(p.metallicity), to_dev(p.age),
        to_dev(p.velocity), 2, perm, offs, nseg,
    )
    torch.cuda.synchronize()
    return cube.reshape(w.sbin, w.sbin, -1)


def test_cube_forward_small_parity(ops):
    w = workload("small")
    ref = oracle_stages("small")
    cube = _cube_small(ops, w).cpu().numpy()
    assert_cube_close(cube, ref["cube"], what="accumulated cube")


def test_cube_forward_deterministic(ops):
    w = workload("small")
    a = _cube_small(ops, w).cpu().numpy()
    b = _cube_small(ops, w).cpu().numpy()
    assert a.tobytes() == b.tobytes()


def test_psf_parity(ops):
    import torch
    from rubix_gb300 import telescope as tel

    w = workload("small")
    ref = oracle_stages("small")
    cube = to_dev(ref["cube"].astype(np.float32))
    g = tel.gaussian_taps_1d(w.psf_size, w.psf_sigma)
    out = ops.psf_forward(cube, g)
    torch.cuda.synchronize()
    want = oracle.apply_psf(ref["cube"].astype(np.float32), oracle.gaussian_kernel_2d(w.psf_size, w.psf_size, w.psf_sigma))
    assert_cube_close(out.cpu().numpy(), want, what="psf")


def test_lsf_parity(ops):
    import torch
    from rubix_gb300 import telescope as tel

    w = workload("small")
    ref = oracle_stages("small")
    cube = to_dev(ref["cube_psf"].astype(np.float32))
    taps = tel.lsf_taps(w.lsf_sigma, w.wave_res)
    out = ops.lsf_forward(cube, taps, 12)
    torch.cuda.synchronize()
    want = oracle.apply_lsf(ref["cube_psf"].astype(np.float32), w.lsf_sigma, w.wave_res)
    assert_cube_close(out.cpu().numpy(), want, what="lsf")


def test_full_chain_small(ops):
    import torch
    from rubix_gb300 import telescope as tel

    w = workload("small")
    ref = oracle_stages("small")
    cube = _cube_small(ops, w)
    g = tel.gaussian_taps_1d(w.psf_size, w.psf_sigma)
    c2 = ops.psf_forward(cube, g)
    c3 = ops.lsf_forward(c2, tel.lsf_taps(w.lsf_sigma, w.wave_res), 12)
    torch.cuda.synchronize()
    assert_cube_close(c3.cpu().numpy(), ref["final"], what="final cube")
