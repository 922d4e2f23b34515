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
        to_dev(p.velocity), 2, perm, offs, nseg, check=True,
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


def _cube_for(ops, w):
    import torch

    p = w.particles
    c = to_dev(p.coords)
    e = to_dev(w.edges)
    nseg = w.sbin * w.sbin
    perm, offs = ops.spaxel_sort(ops.spaxel_assign(c, e), nseg, ops.aperture_mask(c, e))
    cube = ops.cube_forward(
        to_dev(w.ssp.flux), to_dev(w.ssp.metallicity), to_dev(w.ssp.age), to_dev(w.wave_z),
        to_dev(w.wave_t), to_dev(p.mass), to_dev(p.metallicity), to_dev(p.age),
        to_dev(p.velocity), 2, perm, offs, nseg, check=True)
    torch.cuda.synchronize()
    return cube.reshape(w.sbin, w.sbin, -1).cpu().numpy(), offs.cpu().numpy()


def test_cube_general_walk_fine_ssp_grid(ops):
    """SSP grid finer than the telescope bins (the walk may cross several SSP nodes per
    bin) plus particles beyond +-10^4 km/s."""
    import dataclasses

    from rubix_gb300 import synth

    base = workload("small", n=3000)
    rng = np.random.default_rng(7)
    wave = np.linspace(4000.0, 5400.0, 1400).astype(np.float32)
    ssp = synth.make_ssp(12, 5, 1400, seed=9)
    ssp = dataclasses.replace(ssp, wavelength=wave)
    p = base.particles
    vel = p.velocity.copy()
    vel[:40, 2] = rng.uniform(-30000, 30000, 40).astype(np.float32)
    p2 = dataclasses.replace(p, velocity=vel)
    wave_t = np.arange(4700.15, 5300.0, 1.25, dtype=np.float32)
    w = dataclasses.replace(base, particles=p2, ssp=ssp, wave_t=wave_t,
                            wave_z=oracle.cosmological_doppler_shift(base.dist_z, wave))
    got, _ = _cube_for(ops, w)
    ref = oracle.render_cube(p2.coords, p2.velocity, p2.mass, p2.metallicity, p2.age, w.edges,
                             w.sbin, ssp.metallicity, ssp.age, ssp.flux, wave, w.dist_z, wave_t)
    assert_cube_close(got, ref["cube"], what="general-walk cube")


def test_cube_ifu_sampled_spaxels(ops):
    """Full 10^6-particle IFU workload; the oracle recomputes a sample of spaxels
    (including the densest ones, which are split into several chunks and merged)."""
    w = workload("ifu", edge_cases=False)
    p = w.particles
    got, offs = _cube_for(ops, w)
    counts = np.diff(offs)
    dense = np.argsort(counts)[-3:]
    rng = np.random.default_rng(3)
    occupied = np.nonzero(counts)[0]
    sample = np.unique(np.concatenate([dense, rng.choice(occupied, 5, replace=False)]))
    assert counts[dense].max() > 512, "workload should contain multi-chunk spaxels"
    idx = oracle.square_spaxel_assignment(p.coords, w.edges)
    inside = oracle.mask_particles_outside_aperture(p.coords, w.edges)
    for s in sample:
        sel = np.nonzero((idx == s) & inside)[0]
        spec = oracle.particle_spectra(p.mass[sel], p.metallicity[sel], p.age[sel],
                                       p.velocity[sel, 2], w.ssp.metallicity, w.ssp.age,
                                       w.ssp.flux, w.wave_z, w.wave_t).sum(axis=0)
        iy, ix = divmod(int(s), w.sbin)
        assert_cube_close(got[iy, ix], spec, what=f"spaxel {s} ({sel.size} particles)")


def test_renderer_fused_lsf_matches_oracle(ops):
    """Accumulate with the LSF epilogue, then PSF (the renderer's default order)."""
    import torch

    from rubix_gb300.api import IFURenderer

    w = workload("small")
    ref = oracle_stages("small")
    p = w.particles
    r = IFURenderer.from_workload(w, device="cuda")
    st = r.render(*(to_dev(a) for a in (p.coords, p.velocity, p.mass, p.metallicity, p.age)))
    torch.cuda.synchronize()
    assert st.lsf_fused
    assert_cube_close(st.final.cpu().numpy(), ref["final"], what="fused final cube")
    st2 = r.render(*(to_dev(a) for a in (p.coords, p.velocity, p.mass, p.metallicity, p.age)),
                   fuse_lsf=False)
    assert_cube_close(st2.final.cpu().numpy(), ref["final"], what="unfused final cube")


@pytest.mark.parametrize("m", [1, 3, 7, 15, 17, 19])
def test_psf_packed_kernel_equals_scalar_kernel(ops, m):
    """Host taps run the packed two-lane FMA kernel (up to 17 taps), device taps the
    scalar one: same products in the same order, so the cubes are bit-identical; ragged
    x and wavelength edges and padded spaxel strides included (strides that are a
    multiple of 4 floats stage the host-tap kernel's rows by TMA)."""
    import torch

    rng = np.random.default_rng(m)
    g = rng.uniform(0.1, 1.0, m).astype(np.float32)
    for ny, nx, L, pad in ((40, 37, 45, 0), (25, 25, 3721, 0), (9, 70, 33, 5),
                           (40, 37, 45, 3), (25, 25, 3721, 3), (9, 70, 33, 3), (33, 64, 128, 0)):
        base = torch.from_numpy(rng.standard_normal((ny, nx, L + pad)).astype(np.float32)).cuda()
        cube = base[:, :, :L]
        a = ops.psf_forward(cube, g)
        b = ops.psf_forward(cube, torch.from_numpy(g).cuda())
        torch.cuda.synchronize()
        assert torch.equal(a, b), (m, ny, nx, L, pad)
    want = oracle.apply_psf(base[:, :, :L].cpu().numpy().astype(np.float64), np.outer(g, g))
    np.testing.assert_allclose(a.cpu().numpy(), want, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("m", [1, 5, 15, 17])
def test_psf_tma_staged_rows_equal_copy_staged_rows(ops, m):
    """A spaxel stride that is a multiple of 4 floats (16-byte rows) stages the PSF's
    input rows with tiled TMA copies, any other stride with 4-byte cp.async copies; the
    arithmetic is the same, so the cubes are bit-identical.  Cases: strips and
    wavelength tiles cut at the cube's edges (x, y and L not multiples of the 32 x 32
    tile), fewer rows than the ring holds, and the renderer's padded layout (L = 3721 on
    a 3724-float stride).  The kernel's device error word stays 0."""
    import torch

    rng = np.random.default_rng(100 + m)
    g = rng.uniform(0.1, 1.0, m).astype(np.float32)
    for ny, nx, L in ((40, 37, 45), (3, 70, 33), (25, 25, 3721), (50, 33, 3721), (1, 1, 7)):
        Lp = (L + 3) // 4 * 4
        dense = torch.from_numpy(rng.standard_normal((ny, nx, L)).astype(np.float32)).cuda()
        pad = torch.full((ny, nx, Lp + 4), float("nan"), device="cuda")  # never read
        pad[:, :, :L] = dense
        a = ops.psf_forward(pad[:, :, :L], g)      # 16-byte rows: TMA
        so = L + 1 if (L + 1) % 4 else L + 2  # not a multiple of 4 floats: cp.async
        odd = torch.full((ny, nx, so), float("nan"), device="cuda")
        odd[:, :, :L] = dense
        b = ops.psf_forward(odd[:, :, :L], g)
        c = ops.psf_forward(dense, g)              # stride L, L % 4 != 0 here: cp.async
        torch.cuda.synchronize()
        assert torch.equal(a, b) and torch.equal(a, c), (m, ny, nx, L)
        assert not torch.isnan(a).any()
    assert ops.psf_status() == 0
    want = oracle.apply_psf(dense.cpu().numpy().astype(np.float64), np.outer(g, g))
    np.testing.assert_allclose(a.cpu().numpy(), want, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("m", [1, 7, 15, 21])
def test_psf_dot_equals_dot_of_psf(ops, m):
    """<w, PSF(cube)> fused (the convolution never written) against psf_forward followed
    by the dot product, with device taps, unequal x and y taps, ragged strips and
    wavelength tiles and a padded spaxel stride: the convolutions are the same float32
    numbers, only the order of the float64-finished sum differs."""
    import torch

    rng = np.random.default_rng(200 + m)
    ty = torch.from_numpy(rng.uniform(0.1, 1.0, m).astype(np.float32)).cuda()
    tx = torch.from_numpy(rng.uniform(-0.5, 1.0, m).astype(np.float32)).cuda()
    for ny, nx, L, pad in ((50, 50, 3721, 0), (9, 70, 33, 3), (40, 37, 45, 0)):
        base = torch.from_numpy(rng.standard_normal((ny, nx, L + pad)).astype(np.float32)).cuda()
        cube = base[:, :, :L]
        w = torch.from_numpy(rng.standard_normal((ny, nx, L)).astype(np.float32)).cuda()
        got = ops.psf_dot(cube, ty, tx, w)
        want = ops.dot(w, ops.psf_forward(cube, ty, tx))
        torch.cuda.synchronize()
        g, v = float(got), float(want)
        scale = float(w.abs().sum()) * float(ops.psf_forward(cube, ty, tx).abs().max())
        assert abs(g - v) <= 1e-6 * scale, (m, ny, nx, L, g, v)


@pytest.mark.parametrize("k", [3, 13, 28])
def test_lsf_dot_equals_dot_of_lsf(ops, k):
    """<w, LSF(rows)> fused against lsf_forward followed by the dot product (device taps,
    a padded row stride included)."""
    import torch

    rng = np.random.default_rng(300 + k)
    taps = torch.from_numpy(rng.uniform(0.05, 1.0, k).astype(np.float32)).cuda()
    crop = (k - 1) // 2
    for rows, L, pad in ((2500, 3721, 0), (37, 45, 3)):
        base = torch.from_numpy(rng.standard_normal((rows, L + pad)).astype(np.float32)).cuda()
        a = base[:, :L]
        w = torch.from_numpy(rng.standard_normal((rows, L)).astype(np.float32)).cuda()
        got = ops.lsf_dot(a, taps, crop, w)
        conv = ops.lsf_forward(a, taps, crop)
        want = ops.dot(w, conv)
        torch.cuda.synchronize()
        scale = float(w.abs().sum()) * float(conv.abs().max())
        assert abs(float(got) - float(want)) <= 1e-6 * scale, (k, rows, L)
