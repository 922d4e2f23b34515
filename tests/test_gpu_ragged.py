"""Ragged batches on the GPU: one launch per kernel for several galaxies, against the
single-galaxy launches (bit-identical cubes), the oracle, the per-galaxy gradients,
a CUDA-graph replay and the autotuner."""

import numpy as np
import pytest

import oracle
from helpers import assert_cube_close, to_dev

pytestmark = pytest.mark.gpu

COUNTS = [300, 2000, 50, 1200, 0, 800]
SBINS = [16, 25, 18, 32, 17, 20]
SIGMAS = [0.8, 1.5, 2.0, 1.1, 1.0, 1.7]


@pytest.fixture(scope="module")
def batch_case():
    from rubix_gb300 import ragged, synth
    from rubix_gb300 import telescope as tel
    from rubix_gb300.api import IFURenderer

    ssp = synth.make_ssp(20, 6, 1000, seed=1)
    wave_t = tel.calculate_wave_seq(synth.WAVE_RANGE, synth.WAVE_RES)
    edges = [ragged.galaxy_edges(s, synth.DIST_Z) for s in SBINS]
    gals = []
    for g, (n, e) in enumerate(zip(COUNTS, edges)):
        p = synth.make_galaxy(n, seed=50 + g)
        p.coords *= float(e[-1]) / 8.0  # spread over the field, some outside
        gals.append(p)
    cat = {k: np.concatenate([getattr(p, k) for p in gals]) for k in
           ("coords", "velocity", "mass", "metallicity", "age")}
    r = IFURenderer(ssp.age, ssp.metallicity, ssp.wavelength, ssp.flux, wave_t, edges[0],
                    SBINS[0], synth.DIST_Z)
    sizes = [2 * int(np.ceil(3 * s)) + 1 for s in SIGMAS]
    b = ragged.RaggedBatch(r, COUNTS, SBINS, edges, SIGMAS, sizes, synth.LSF_SIGMA,
                           synth.WAVE_RES)
    dev = {k: to_dev(v) for k, v in cat.items()}
    return b, ssp, wave_t, edges, gals, cat, dev


def test_ragged_assign_matches_oracle(batch_case):
    b, _, _, edges, gals, cat, dev = batch_case
    idx, keep = b.assign(dev["coords"])
    idx, keep = idx.cpu().numpy(), keep.cpu().numpy().astype(bool)
    for g, p in enumerate(gals):
        p0, p1 = int(b.t.poff[g]), int(b.t.poff[g + 1])
        local = oracle.square_spaxel_assignment(p.coords, edges[g])
        inside = oracle.mask_particles_outside_aperture(p.coords, edges[g])
        k = inside & (local < SBINS[g] ** 2)
        assert np.array_equal(keep[p0:p1], k)
        assert np.array_equal(idx[p0:p1][k], local[k] + int(b.t.seg_base[g]))


def test_ragged_render_equals_single_galaxy_launches(batch_case):
    import torch

    from rubix_gb300 import ragged

    b, *_, dev = batch_case
    args = (dev["coords"], dev["velocity"], dev["mass"], dev["metallicity"], dev["age"])
    batched = b.render(*args)
    looped = ragged.render_per_galaxy(b, *args)
    torch.cuda.synchronize()
    assert torch.equal(batched, looped)


def test_ragged_galaxy_matches_oracle(batch_case):
    b, ssp, wave_t, edges, gals, cat, dev = batch_case
    out = b.render(dev["coords"], dev["velocity"], dev["mass"], dev["metallicity"], dev["age"])
    g = 1
    p = gals[g]
    ref = oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, edges[g],
                             SBINS[g], ssp.metallicity, ssp.age, ssp.flux, ssp.wavelength,
                             0.1, wave_t, psf_size=2 * int(np.ceil(3 * SIGMAS[g])) + 1,
                             psf_sigma=SIGMAS[g], lsf_sigma=1.2, wave_res=1.25)
    assert_cube_close(b.galaxy_view(out, g).cpu().numpy(), ref["final"], what="ragged galaxy")
    # the empty galaxy renders zeros
    assert not b.galaxy_view(out, 4).any()


def test_ragged_forward_backward(batch_case):
    import torch

    from rubix_gb300 import ragged

    b, *_, dev = batch_case
    args = (dev["coords"], dev["velocity"], dev["mass"], dev["metallicity"], dev["age"])
    rng = np.random.default_rng(2)
    cube0 = b.render(*args)
    target = (cube0 * to_dev(rng.uniform(0.9, 1.1, cube0.shape).astype(np.float32))).contiguous()
    weight = 1.0 / (target * target / 400.0 + 1e-3 * float(target.abs().max()) ** 2)
    loss, grads, d_psf, d_lsf, _ = b.forward_backward(*args, target, weight)
    loss2, grads2, d_psf2, d_lsf2 = ragged.forward_backward_per_galaxy(b, *args, target, weight)
    torch.cuda.synchronize()
    # particle gradients: same per-particle arithmetic, same adjoint rows
    for a, c, name in zip(grads, grads2, ("mass", "Z", "age", "v")):
        a, c = a.cpu().numpy(), c.detach().cpu().numpy()
        scale = np.abs(c).max()
        assert np.max(np.abs(a - c)) <= 1e-6 * scale, name
    np.testing.assert_allclose(d_psf.cpu().numpy(), d_psf2.cpu().numpy(), rtol=1e-6)
    np.testing.assert_allclose(float(d_lsf), float(d_lsf2), rtol=1e-6)
    np.testing.assert_allclose(float(loss), float(loss2), rtol=1e-5)


def test_ragged_graph_replay(batch_case):
    import torch

    b, *_, dev = batch_case
    args = (dev["coords"], dev["velocity"], dev["mass"], dev["metallicity"], dev["age"])
    cube0 = b.render(*args)
    target = (cube0 * 1.03).contiguous()
    weight = torch.ones_like(target)
    eager = b.forward_backward(*args, target, weight)
    graph, out = b.capture(b.forward_backward, *args, target, weight)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out[4], eager[4])  # cube
    for a, c in zip(out[1], eager[1]):
        assert torch.equal(a, c)
    assert torch.equal(out[2], eager[2])


def test_autotune_picks_a_candidate(batch_case):
    import torch

    from rubix_gb300 import autotune

    b, *_, dev = batch_case
    args = (dev["coords"], dev["velocity"], dev["mass"], dev["metallicity"], dev["age"])
    ref = b.render(*args).clone()
    res = autotune.autotune(lambda: b.render(*args), key=("test", 6),
                            candidates=((256, 64), (64, 16)), repeats=2)
    assert res["best"] in ((256, 64), (64, 16)) and len(res["times_ms"]) == 2
    assert autotune.get_tuning(0) == res["best"]
    out = b.render(*args)
    torch.cuda.synchronize()
    scale = float(ref.abs().max())
    assert float((out - ref).abs().max()) <= 1e-6 * scale
    again = autotune.autotune(lambda: None, key=("test", 6))
    assert again["cached"] and again["best"] == res["best"]
    autotune.set_tuning(0, None)
    assert autotune.get_tuning(0) == (256, 64)
