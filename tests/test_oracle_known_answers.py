"""The oracle against the known answers of rubix's own tests for this path.

Each test restates the inputs and expectations of a rubix test (cited); together they
pin the oracle restatement to the reference's specified behaviour.
"""

import numpy as np
import pytest

import oracle

C = 299792.458


def test_cosmological_doppler_shift():  # tests/test_spectra_ifu.py:29-34
    w = np.array([5000.0, 6000.0, 7000.0], dtype=np.float32)
    np.testing.assert_allclose(oracle.cosmological_doppler_shift(0.1, w), w * 1.1, rtol=1e-6)


def test_calculate_diff():  # tests/test_spectra_ifu.py:37-50
    v = np.array([1.0, 2.0, 4.0, 7.0])
    assert np.array_equal(oracle.calculate_diff(v), [0, 1, 2, 3])
    assert np.array_equal(oracle.calculate_diff(v, pad_with_zero=False), [1, 2, 3])


def test_velocity_doppler_shift():  # tests/test_spectra_ifu.py:150-172 (direction "y")
    w = np.array([5000.0, 6000.0, 7000.0], dtype=np.float32)
    vel = np.array([[300.0, 400.0, 500.0], [600.0, 700.0, 800.0]], dtype=np.float32)
    got = oracle.velocity_doppler_shift32(w, vel[:, 1])
    want = np.stack([w * np.exp(vel[0, 1] / C), w * np.exp(vel[1, 1] / C)])
    np.testing.assert_allclose(got, want, rtol=1e-5)


def _resample_expected(F, lp, lt):
    in_range = (lp >= lt.min()) & (lp <= lt.max())
    total = np.sum(F * oracle.calculate_diff(lp) * in_range)
    lum = np.interp(lt, lp, F)
    new_total = np.sum(lum * oracle.calculate_diff(lt))
    return lum, total, new_total


def test_resample_spectrum():  # tests/test_spectra_ifu.py:175-199
    F = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    lp = np.array([4000.0, 5000.0, 6000.0, 7000.0, 8000.0])
    lt = np.array([4500.0, 5500.0, 6500.0, 7500.0])
    got = oracle.resample_spectrum(F, lp, lt)
    lum, total, new_total = _resample_expected(F, lp, lt)
    np.testing.assert_allclose(got, lum * total / new_total, rtol=1e-5)
    assert not np.any(np.isnan(got))
    got_rows, _ = oracle.resample_spectra(F[None], lp[None].astype(np.float32),
                                          lt.astype(np.float32))
    np.testing.assert_allclose(got_rows[0], got, rtol=1e-12)


def test_resample_spectrum_if_spec_is_zero():  # tests/test_spectra_ifu.py:202-228
    F = np.zeros(5)
    lp = np.array([4000.0, 5000.0, 6000.0, 7000.0, 8000.0])
    lt = np.array([4500.0, 5500.0, 6500.0, 7500.0])
    got = oracle.resample_spectrum(F, lp, lt)
    assert not np.any(np.isnan(got))
    assert (got == 0).all()


def test_calculate_cube():  # tests/test_spectra_ifu.py:231-257
    spectra = np.array([[100, 200, 300], [400, 500, 600], [700, 800, 900], [1, 2, 3]],
                       dtype=np.float32)
    idx = np.array([0, 1, 1, 3], dtype=np.int32)
    expected = np.array([[[100, 200, 300], [1100, 1300, 1500]], [[0, 0, 0], [1, 2, 3]]])
    assert np.array_equal(oracle.calculate_cube(spectra, idx, 2), expected)


def test_calculate_cube_drops_ids_beyond_segments():  # jax.ops.segment_sum semantics
    spectra = np.ones((3, 2), dtype=np.float32)
    cube = oracle.calculate_cube(spectra, np.array([0, 4, 7]), 2)
    assert cube.sum() == 2.0 and cube[0, 0].tolist() == [1.0, 1.0]


def test_square_spaxel_assignment():  # tests/test_telescope_utils.py:20-35
    coords = np.array([[0.5, 1.5], [2.5, 3.5]])
    edges = np.array([0, 1, 2, 3, 4])
    assert oracle.square_spaxel_assignment(coords, edges).tolist() == [4, 14]


def test_no_particles():  # tests/test_telescope_utils.py:38-42
    assert len(oracle.mask_particles_outside_aperture(np.zeros((0, 3)), np.array([0, 1]))) == 0


@pytest.mark.parametrize("coords,n_inside", [
    ([[0.5, 0.5, 0], [0.2, 0.2, 0]], 2),                             # :45-51
    ([[1.5, 1.5, 0], [-0.1, -0.1, 0]], 0),                           # :54-59
    ([[0, 0, 0], [1, 1, 0], [0, 1, 0], [1, 0, 0]], 4),               # :62-68 boundary inclusive
    ([[0.5, 0.5, 0], [1.5, 1.5, 0], [0, 0, 0], [-0.1, -0.1, 0]], 2),  # :71-79
])
def test_mask_particles_outside_aperture(coords, n_inside):
    m = oracle.mask_particles_outside_aperture(np.array(coords, dtype=np.float32),
                                               np.array([0, 1]))
    assert int(m.sum()) == n_inside


def test_calculate_spatial_bin_edges():  # tests/test_telescope_utils.py:82-99
    edges, size = oracle.calculate_spatial_bin_edges(1.0, np.int64(10), 2.0)
    assert size == 0.2
    np.testing.assert_allclose(edges, np.arange(-1.0, 1.0 + 0.2, 0.2), atol=1e-6)


def test_gaussian_kernel_properties():  # tests/test_telescope_psf_kernels.py:6-28
    k = oracle.gaussian_kernel_2d(5, 5, 1.0)
    assert k.shape == (5, 5) and (k >= 0).all()
    assert np.isclose(k.sum(), 1.0)
    assert k[2, 2] == k.max()


def test_get_psf_kernel_gaussian():  # tests/test_telescope_psf.py:8-13
    k = oracle.gaussian_kernel_2d(3, 3, 2.0)
    assert k.shape == (3, 3) and np.isclose(k.sum(), 1.0)


def _convolve2d_same(plane, K):
    from scipy.signal import convolve2d

    return convolve2d(plane, K, mode="same")


@pytest.mark.parametrize("nplanes", [1, 3])
def test_apply_psf_planes(nplanes):  # tests/test_telescope_psf.py:21-54
    cube = np.zeros((10, 10, nplanes))
    cube[5, 5, :] = 1.0
    K = np.ones((3, 3))
    got = oracle.apply_psf(cube, K)
    for i in range(nplanes):
        np.testing.assert_allclose(got[:, :, i], _convolve2d_same(cube[:, :, i], K), atol=1e-12)


def test_apply_psf_direct_equals_fft():
    rng = np.random.default_rng(0)
    cube = rng.random((9, 7, 5))
    K = oracle.gaussian_kernel_2d(5, 5, 1.3)
    np.testing.assert_allclose(oracle.apply_psf(cube, K, method="direct"),
                               oracle.apply_psf(cube, K, method="fft"), atol=1e-12)
    for i in range(5):
        np.testing.assert_allclose(oracle.apply_psf(cube, K)[:, :, i],
                                   _convolve2d_same(cube[:, :, i], K), atol=1e-12)


@pytest.mark.parametrize("positions", [[50], [20, 50, 75]])
def test_apply_lsf_delta(positions):  # tests/test_telescope_lsf.py:6-60
    spectra = np.zeros((len(positions), 100))
    for i, p in enumerate(positions):
        spectra[i, p] = 1.0
    got = oracle.apply_lsf(spectra, 2.0, 1.0)
    x = np.arange(100)
    for i, p in enumerate(positions):
        g = np.exp(-0.5 * (x - p) ** 2 / 4.0)
        np.testing.assert_allclose(got[i], g / g.sum(), atol=1e-5)


def test_apply_lsf_cube_shape_and_flux():  # tests/test_core_lsf.py:80-117
    cube = np.zeros((10, 10, 10))
    cube[:, :, 5] = 1.0
    got = oracle.apply_lsf(cube, 0.6, 1.25)
    assert got.shape == cube.shape
    assert np.all(got[:, :, 5] != 1)
    np.testing.assert_allclose(got.sum(axis=2), 1.0, rtol=1e-12)


def test_scale_spectrum_by_mass():  # tests/test_core_ifu.py:249-282
    spectra = np.arange(12, dtype=np.float32).reshape(1, 2, 6)
    mass = np.array([[0.5, 1.0]], dtype=np.float32)
    assert np.array_equal(spectra * mass[..., None], spectra * np.expand_dims(mass, -1))


def test_interp2d_linear_nodes_and_outside():
    # interpax linear: reproduces grid nodes, bilinear inside, 0 outside (inclusive box)
    x = np.array([0.001, 0.004, 0.02], dtype=np.float32)
    y = np.array([0.1, 1.0, 5.0, 13.0], dtype=np.float32)
    rng = np.random.default_rng(1)
    f = rng.random((3, 4, 7)).astype(np.float32)
    X, Y = np.meshgrid(x, y, indexing="ij")
    got = oracle.interp2d_linear(X.ravel(), Y.ravel(), x, y, f)
    np.testing.assert_allclose(got, f.reshape(12, 7), rtol=1e-6)
    mid = oracle.interp2d_linear([0.0025], [0.55], x, y, f)[0]
    want = 0.25 * (f[0, 0] + f[1, 0] + f[0, 1] + f[1, 1])
    np.testing.assert_allclose(mid, want, rtol=1e-6)
    out = oracle.interp2d_linear([0.05, 0.0005, 0.01, 0.01], [1.0, 1.0, 14.0, 0.05], x, y, f)
    assert (out == 0).all()


def test_calculate_spectra_outside_grid_is_zero():  # tests/test_core_ifu.py:207-246
    x = np.array([1e-4, 0.05], dtype=np.float32)
    y = np.array([0.1, 13.5], dtype=np.float32)
    f = np.ones((2, 2, 842), dtype=np.float32)
    spec = oracle.interp2d_linear([0.1], [4.5], x, y, f)
    assert spec.shape == (1, 842) and (spec == 0).all()
