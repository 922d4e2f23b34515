"""apply_noise: the Philox generator (host, no GPU), the noise statistics against the
oracle's restatement of calculate_S2N, the median's NaN rule, the step's config checks."""

import numpy as np
import pytest

import oracle
from helpers import to_dev


def test_philox_restatement_known_answers():
    # Random123 known-answer vector for philox4x32-10, counter = key = 0
    assert oracle.philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C,
                                                           0x9B00DBD8]
    m = 0xFFFFFFFF
    assert oracle.philox4x32_10([m] * 4, [m] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                       0x6D5451FD]


def test_library_philox_matches_restatement(rubix_lib):
    from rubix_gb300 import ops

    rng = np.random.default_rng(0)
    for _ in range(20):
        c = [int(x) for x in rng.integers(0, 2**32, 4, dtype=np.uint64)]
        k = [int(x) for x in rng.integers(0, 2**32, 2, dtype=np.uint64)]
        assert ops.philox4x32_10(c, k) == oracle.philox4x32_10(c, k)


def test_vectorised_philox_matches_restatement():
    rng = np.random.default_rng(3)
    c = rng.integers(0, 2**32, (4, 16), dtype=np.uint64)
    k = [int(x) for x in rng.integers(0, 2**32, 2, dtype=np.uint64)]
    got = oracle.philox4x32_10_arrays(*c, *k)
    for i in range(16):
        assert [int(x[i]) for x in got] == oracle.philox4x32_10([int(v) for v in c[:, i]], k)


def test_noise_draws_counter_mapping():
    # element (s, t) -> index e = s*L + t -> output e % 4 of the call with counter e // 4
    seed = (7 << 32) | 11
    z = oracle.noise_draws(3, 9, seed, "uniform")
    for s_, t in ((0, 0), (0, 8), (1, 0), (2, 5)):
        e = s_ * 9 + t
        bits = oracle.philox4x32_10([e // 4, 0, 0, 0], [11, 7])[e % 4]
        assert z[s_, t] == (bits >> 8) / 2.0**24
    n = oracle.noise_draws(64, 3721, 1, "normal")
    assert abs(n.mean()) < 5 / np.sqrt(n.size) and abs(n.std() - 1) < 5e-3


def test_noise_sigma_nan_rule():
    cube = np.ones((3, 3, 4))
    s, med = oracle.noise_sigma(cube, 10.0)
    assert med == 4.0 and np.allclose(s, np.sqrt(4.0) / 10.0 / 2.0)
    cube[0, 0, :] = 0.0  # one empty spaxel: the median becomes NaN -> 0, no noise anywhere
    s, med = oracle.noise_sigma(cube, 10.0)
    assert med == 0.0 and not s.any()


def test_apply_noise_config_messages():
    from rubix_gb300.core import get_apply_noise

    with pytest.raises(ValueError, match="Noise information not provided in telescope config"):
        get_apply_noise({"telescope": {}})
    with pytest.raises(ValueError, match="Signal to noise information not provided"):
        get_apply_noise({"telescope": {"noise": {}}})
    with pytest.raises(ValueError, match="Noise distribution not provided in noise config"):
        get_apply_noise({"telescope": {"noise": {"signal_to_noise": 1}}})
    f = get_apply_noise({"telescope": {"noise": {"signal_to_noise": 1,
                                                 "noise_distribution": "normal"}}})
    assert f.__name__ == "apply_noise"


@pytest.mark.gpu
def test_flux_image_and_median():
    import torch

    from rubix_gb300 import ops

    rng = np.random.default_rng(1)
    for n in (1, 2, 7, 1000, 22500):
        flux = rng.uniform(0.5, 2.0, n).astype(np.float32)
        med = float(ops.noise_median(to_dev(flux)))
        assert med == np.float32(np.median(flux.astype(np.float64))) or \
            abs(med - np.median(flux)) <= 1e-7 * np.median(flux)
    flux[3] = 0.0
    assert float(ops.noise_median(to_dev(flux))) == 0.0
    cube = rng.random((13, 11, 300)).astype(np.float32)
    got = ops.flux_image(to_dev(cube)).cpu().numpy()
    np.testing.assert_allclose(got, cube.sum(-1), rtol=1e-5)
    torch.cuda.synchronize()


@pytest.mark.gpu
@pytest.mark.parametrize("dist", ["normal", "uniform"])
def test_noise_statistics(dist):
    import torch

    from rubix_gb300 import ops

    rng = np.random.default_rng(2)
    S, L = 40, 3721
    base = rng.uniform(1.0, 3.0, (S, S, 1)) * np.ones((1, 1, L))
    base = base.astype(np.float32)
    sig, _ = oracle.noise_sigma(base, 20.0)
    cube = to_dev(base)
    ops.apply_noise_(cube, 20.0, dist, seed=123)
    again = to_dev(base)
    ops.apply_noise_(again, 20.0, dist, seed=123)
    other = to_dev(base)
    ops.apply_noise_(other, 20.0, dist, seed=124)
    torch.cuda.synchronize()
    got = cube.cpu().numpy()
    assert np.array_equal(got, again.cpu().numpy())
    assert not np.array_equal(got, other.cpu().numpy())
    z = (got.astype(np.float64) - base) / (base * sig[:, :, None])
    n = z.size
    if dist == "normal":
        assert abs(z.mean()) < 5 / np.sqrt(n) and abs(z.std() - 1.0) < 5e-3
        # Gaussian tails: |z| > 3 about 0.27 %
        assert abs(np.mean(np.abs(z) > 3) - 0.0027) < 5e-4
    else:
        # z recovered from float32 values: within rounding of [0, 1)
        assert abs(z.mean() - 0.5) < 5 / np.sqrt(12 * n)
        assert z.min() >= -1e-5 and z.max() < 1 + 1e-5


def _apply_noise_rows(rows, L, flux, median, dist, seed):
    """rubix_apply_noise on a [spaxels, >= L] float32 view (any row stride)."""
    from rubix_gb300 import _lib, ops

    _lib.call("rubix_apply_noise", ops._ptr(rows), rows.shape[0], L, rows.stride(0),
              ops._ptr(flux), ops._ptr(median), 20.0, {"normal": 0, "uniform": 1}[dist],
              seed, ops._stream(rows.device))


@pytest.mark.gpu
@pytest.mark.parametrize("dist", ["normal", "uniform"])
def test_noise_draws_match_counter_mapping(dist):
    """Every element's draw is the oracle's Philox output for its counter; the float4
    path (unpadded, aligned), the element path of a misaligned cube and of padded rows
    give bit-identical cubes."""
    import torch

    from rubix_gb300 import ops

    rng = np.random.default_rng(4)
    n_sp, L = 35, 37  # odd L: quads straddle spaxel rows
    seed = (5 << 32) | 99
    base = rng.uniform(1.0, 3.0, (n_sp, L)).astype(np.float32)
    cube = to_dev(base)
    flux = ops.flux_image(cube)
    med = ops.noise_median(flux)
    _apply_noise_rows(cube, L, flux, med, dist, seed)
    # misaligned start (element path) and padded rows (element path)
    buf = torch.zeros(n_sp * L + 1, dtype=torch.float32, device=cube.device)
    mis = buf[1:].view(n_sp, L)
    mis.copy_(to_dev(base))
    _apply_noise_rows(mis, L, flux, med, dist, seed)
    pad = torch.zeros(n_sp, L + 3, dtype=torch.float32, device=cube.device)
    pad[:, :L] = to_dev(base)
    _apply_noise_rows(pad, L, flux, med, dist, seed)
    torch.cuda.synchronize()
    got = cube.cpu().numpy()
    assert np.array_equal(got, mis.cpu().numpy())
    assert np.array_equal(got, pad[:, :L].cpu().numpy())
    assert not pad[:, L:].any()

    f = flux.cpu().numpy()
    scale = np.float32(np.sqrt(np.float32(med.item()))) * (np.float32(1) / np.float32(20))
    sig = (scale / np.sqrt(f)).astype(np.float32)
    z = oracle.noise_draws(n_sp, L, seed, dist)
    if dist == "uniform":
        w = (sig[:, None] * z.astype(np.float32)).astype(np.float32)
        want = (base.astype(np.float64) + base.astype(np.float64) * w).astype(np.float32)
        ulps = np.abs(got.view(np.int32).astype(np.int64) - want.view(np.int32))
        assert ulps.max() <= 1 and (ulps == 0).mean() > 0.99
    else:
        zg = (got.astype(np.float64) - base) / (base * sig[:, None].astype(np.float64))
        np.testing.assert_allclose(zg, z, rtol=0, atol=5e-4)
