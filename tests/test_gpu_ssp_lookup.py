"""The SSP lookup's interpolation rules on the GPU, against the oracle.

rubix looks templates up with interpax's interp2d (rubix/spectra/ssp/grid.py:113-120,
called from rubix/core/ifu.py:63-121); this package implements its ``method="linear"``
branch with ``extrap=0``: bilinear on the cell clip(searchsorted(grid, q, 'right'), 1,
n-1), in linear metallicity and linear age, 0 outside the inclusive box
[Z_0, Z_last] x [A_0, A_last].  No reference vector covers that branch (rubix's tests use
method="cubic" on a template file it does not ship), so these checks pin its rules on
the 221 ages x 6 metallicities grid: every node is reproduced, the outer boundary is
inside (it returns the edge node), and the nearest float32 values just outside return
0 -- for the materialised lookup (rubix_ssp_lookup) and through the fused cube kernel.
"""

import numpy as np
import pytest

import oracle
from helpers import CUBE_RTOL, assert_cube_close, to_dev

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grid():
    from rubix_gb300 import synth

    ssp = synth.make_ssp(221, 6, 1221, seed=2)
    zg, ag = ssp.metallicity, ssp.age
    Z, A = np.meshgrid(zg, ag, indexing="ij")
    nodes = (Z.reshape(-1), A.reshape(-1))  # (z, a) order matches flux[z, a]
    up, down = np.float32(np.inf), np.float32(-np.inf)
    outside = (np.array([np.nextafter(zg[0], down), np.nextafter(zg[-1], up), zg[2], zg[3]],
                        dtype=np.float32),
               np.array([ag[100], ag[50], np.nextafter(ag[0], down), np.nextafter(ag[-1], up)],
                        dtype=np.float32))
    return ssp, nodes, outside


def test_lookup_reproduces_every_node(rubix_lib, grid):
    from rubix_gb300 import ops

    ssp, (z, a), _ = grid
    got = ops.ssp_lookup(to_dev(ssp.flux), to_dev(ssp.metallicity), to_dev(ssp.age),
                         to_dev(z), to_dev(a)).cpu().numpy()
    want = ssp.flux.reshape(-1, ssp.flux.shape[-1])
    ref = oracle.interp2d_linear(z, a, ssp.metallicity, ssp.age, ssp.flux)
    rel = np.abs(got - want) / np.abs(want)
    print(f"lookup at all {z.size} nodes: max rel err vs the node spectra {rel.max():.2e}, "
          f"exact {np.mean(got == want):.4f} of elements")
    assert rel.max() <= 1e-6
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()
    # interior nodes and the lower boundary are exact: weight (1, 0) on the node
    interior = (z < ssp.metallicity[-1]) & (a < ssp.age[-1])
    assert np.array_equal(got[interior], want[interior])


def test_lookup_outer_boundary_inclusive_and_outside_zero(rubix_lib, grid):
    from rubix_gb300 import ops

    ssp, _, (z, a) = grid
    zg, ag = ssp.metallicity, ssp.age
    qz = np.concatenate([z, [zg[0], zg[-1], zg[-1], zg[0]]]).astype(np.float32)
    qa = np.concatenate([a, [ag[0], ag[-1], ag[0], ag[-1]]]).astype(np.float32)
    got = ops.ssp_lookup(to_dev(ssp.flux), to_dev(zg), to_dev(ag), to_dev(qz),
                         to_dev(qa)).cpu().numpy()
    assert not got[:4].any(), "just outside the grid must give 0"
    corners = [ssp.flux[0, 0], ssp.flux[-1, -1], ssp.flux[-1, 0], ssp.flux[0, -1]]
    for k, want in enumerate(corners):
        np.testing.assert_allclose(got[4 + k], want, rtol=1e-6)
    ref = oracle.interp2d_linear(qz, qa, zg, ag, ssp.flux)
    assert not ref[:4].any()
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=0)


def test_fused_kernel_nodes_and_outside(rubix_lib, grid):
    """Each node (and each just-outside point) as one particle in its own spaxel,
    through the fused lookup/resample/sum kernel."""
    from rubix_gb300 import synth
    from rubix_gb300 import telescope as tel
    from rubix_gb300.api import IFURenderer

    ssp, (nz, na), (oz, oa) = grid
    z = np.concatenate([nz, oz]).astype(np.float32)
    a = np.concatenate([na, oa]).astype(np.float32)
    n = z.size
    S = int(np.ceil(np.sqrt(n)))
    edges = np.arange(S + 1, dtype=np.float32)
    k = np.arange(n)
    coords = np.stack([k % S + 0.5, k // S + 0.5, np.zeros(n)], axis=1).astype(np.float32)
    rng = np.random.default_rng(9)
    vel = np.zeros((n, 3), dtype=np.float32)
    vel[:, 2] = rng.normal(0.0, 80.0, n).astype(np.float32)
    mass = np.full(n, 1e5, dtype=np.float32)
    wave_t = tel.calculate_wave_seq(synth.WAVE_RANGE, synth.WAVE_RES)
    r = IFURenderer(ssp.age, ssp.metallicity, ssp.wavelength, ssp.flux, wave_t, edges, S,
                    synth.DIST_Z)
    st = r.render(to_dev(coords), to_dev(vel), to_dev(mass), to_dev(z), to_dev(a))
    got = st.cube.cpu().numpy()
    ref = oracle.render_cube(coords, vel, mass, z, a, edges, S, ssp.metallicity, ssp.age,
                             ssp.flux, ssp.wavelength, synth.DIST_Z, wave_t)["cube"]
    norm, elem = assert_cube_close(got, ref, rtol=CUBE_RTOL, what="fused kernel at SSP nodes")
    print(f"fused kernel, {nz.size} nodes + {oz.size} outside points: normwise {norm:.2e}, "
          f"elementwise {elem:.2e}")
    flat = got.reshape(S * S, -1)
    assert not flat[nz.size:n].any(), "particles just outside the grid must contribute 0"
    assert flat[:nz.size].min(axis=1).min() > 0
