"""Host logic of ragged batches: layout tables, tap padding, batch specification."""

import numpy as np
import pytest

import oracle
from rubix_gb300 import ragged


def test_build_tables():
    edges = [np.linspace(-1, 1, s + 1).astype(np.float32) for s in (16, 33, 20)]
    t = ragged.build_tables([10, 0, 5], [16, 33, 20], edges, 3721)
    assert t.poff.tolist() == [0, 10, 10, 15]
    assert t.eoff.tolist() == [0, 17, 51, 72]
    assert t.seg_base.tolist() == [0, 256, 256 + 1089, 256 + 1089 + 400]
    nl = (3721 + 31) // 32
    assert t.block_off.tolist() == [0, nl, nl + 2 * nl, nl + 2 * nl + nl]
    assert t.n_blocks == 4 * nl and t.n_segments == 1745 and t.n_gal == 3
    with pytest.raises(ValueError):
        ragged.build_tables([1], [4], [np.array([1.0, 0.0])], 10)  # descending edges
    with pytest.raises(ValueError):
        ragged.build_tables([1, 2], [4], edges[:1], 10)


@pytest.mark.parametrize("k,m", [(3, 7), (7, 13), (4, 9), (13, 13), (6, 7)])
def test_pad_taps_keeps_same_convolution(k, m):
    rng = np.random.default_rng(k * 100 + m)
    t = rng.random(k)
    cube = rng.standard_normal((12, 10, 2))
    ref = oracle.apply_psf(cube, np.outer(t, t), method="direct")
    p = ragged.pad_taps(t, m)
    got = oracle.apply_psf(cube, np.outer(p, p), method="direct")
    np.testing.assert_allclose(got, ref, atol=1e-12)


def test_padded_size_and_limits():
    assert ragged.padded_size([7, 13, 9]) == 13
    assert ragged.padded_size([4, 6]) == 7
    with pytest.raises(ValueError):
        ragged.padded_size([23])
    with pytest.raises(ValueError):
        ragged.pad_taps(np.ones(5), 4)


def test_synthetic_batch_spec():
    counts, sbins, sig, sizes = ragged.synthetic_batch_spec()
    assert counts.size == 256 and counts.min() >= 1000 and counts.max() <= 1_000_000
    assert sbins.min() >= 16 and sbins.max() <= 64
    assert sig.min() >= 0.8 and sig.max() <= 2.0
    assert np.all(sizes % 2 == 1) and ragged.padded_size(sizes) <= 13
    # log-uniform: total about 256 * (1e6 - 1e3) / ln(1e3)
    assert 2e7 < counts.sum() < 6e7
    again = ragged.synthetic_batch_spec()
    assert all(np.array_equal(a, b) for a, b in zip((counts, sbins, sig, sizes), again))
