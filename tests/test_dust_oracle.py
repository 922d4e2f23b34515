"""Dust extinction on the CPU: the oracle against rubix's known answers
(tests/test_dust_classes.py, tests/test_dust_extinction.py of rubix), hand-derived
properties of rubix's column-density algorithm, and the package's host-side curves and
dust-to-gas parameters against the oracle.  No GPU."""

import numpy as np
import pytest

from oracle import dust_oracle as do


# --- rubix tests/test_dust_classes.py:14-81, known answers ---------------------------

def test_power_law_known_answer():
    np.testing.assert_allclose(do.power_law_1d(np.array([1.0, 2.0, 3.0]), 2.0, 1.0, 1.0),
                               [2.0, 1.0, 0.66666667], rtol=1e-6)


def test_polynomial_known_answers():
    x = np.array([1.0, 2.0, 3.0])
    np.testing.assert_allclose(do.polynomial_1d(x, [1.0, 2.0, 3.0]), [6.0, 17.0, 34.0])
    np.testing.assert_allclose(do.polynomial_1d(x, [1.0]), [1.0, 1.0, 1.0])


def test_drude_known_answers():
    x = np.array([1.0, 2.0, 3.0])
    expected = [1.0, 0.30769232, 0.12328766]
    np.testing.assert_allclose(do.drude_1d(x, 1.0, 1.0, 1.0), expected, rtol=1e-6)
    np.testing.assert_allclose(do.modified_drude(x, 1.0, 1.0, 1.0, 0.0), expected, rtol=1e-6)
    with pytest.raises(ValueError, match="0 is not an allowed value for x_0"):
        do.drude_1d(x, 1.0, 0.0, 1.0)


def test_fm90_known_answer_and_bounds():
    x = np.array([4.0, 5.0, 6.0])
    np.testing.assert_allclose(do.fm90(x, 0.10, 0.70, 3.23, 0.41, 4.59, 0.95),
                               [4.1879544, 5.723751, 4.7574277], rtol=1e-6)
    for kw, msg in ((dict(C1=6.0), "C1 is out of bounds: 6.0"),
                    (dict(C2=-1.5), "C2 is out of bounds: -1.5"),
                    (dict(C3=7.0), "C3 is out of bounds: 7.0"),
                    (dict(C4=-1.5), "C4 is out of bounds: -1.5"),
                    (dict(xo=5.5), "xo is out of bounds: 5.5"),
                    (dict(gamma=0.1), "gamma is out of bounds: 0.1")):
        args = dict(C1=0.0, C2=0.5, C3=3.0, C4=0.5, xo=4.5, gamma=0.5)
        args.update(kw)
        if "gamma" not in kw:
            args["gamma"] = 0.95
        with pytest.raises(ValueError, match=msg):
            do.fm90(x, **args)


def test_model_curves_in_range():
    """rubix tests/test_dust_classes.py:112-166: shapes and 0 <= A(x)/A(V) <= 10."""
    w = np.array([0.5, 1.0, 2.0, 3.0, 5.0, 8.0, 10.0])
    r = do.cardelli89(w, 3.1)
    assert r.shape == w.shape and np.all(r >= 0) and np.all(r <= 10)
    w = np.array([0.1, 0.3, 0.5, 1.0, 2.0, 5.0, 10.0, 20.0, 30.0])
    r = do.gordon23(w, 3.1)
    assert r.shape == w.shape and np.all(r >= 0) and np.all(r <= 10)


def test_extinguish_formula():
    """rubix tests/test_dust_classes.py:136-151: 10^(-0.4 A(x)/A(V) Av)."""
    w = np.array([0.5, 1.0, 2.0, 3.0, 5.0, 8.0, 10.0])
    ax = do.cardelli89(w, 3.1)
    np.testing.assert_allclose(do.extinguish(ax, 3.1)[0], 10.0 ** (-0.4 * ax * 3.1), rtol=1e-6)


@pytest.mark.parametrize("model", ["power law slope free", "broken power law fit"])
@pytest.mark.parametrize("xco", ["MW", "Z"])
def test_dust_to_gas_ratio(model, xco):
    """rubix tests/test_dust_extinction.py:156-189: shape and positivity."""
    r = do.dust_to_gas_ratio(np.array([8.0, 8.5]), model, xco)
    assert r.shape == (2,) and np.all(r >= 0)


def test_dust_to_gas_fixed_slope_not_implemented():
    with pytest.raises(NotImplementedError):
        do.dust_to_gas_ratio(np.array([8.0]), "power law slope fixed", "MW")


def test_reference_mock_extinction():
    """rubix tests/test_dust_extinction.py:15-106: the two-cell mock of rubix's tests
    gives (1, 2, 2) non-negative spectra for both models."""
    gas = dict(coords=np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]]), pixel_assignment=[0, 1],
               metals=np.array([[0.01, 0.02, 0.03, 0.04, 0.05], [0.06, 0.07, 0.08, 0.09, 0.1]]),
               mass=np.array([1.0, 2.0]))
    stars = dict(coords=np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]]), pixel_assignment=[0, 1])
    spectra = np.array([[[1.0, 2.0], [3.0, 4.0]]])
    for model in ("Cardelli89", "Gordon23"):
        dust = dict(extinction_model=model, Rv=3.1, dust_grain_density=3.0,
                    dust_to_gas_model="power law slope free", Xco="MW")
        out, av, T = do.apply_spaxel_extinction(spectra, np.array([5000.0, 6000.0]), gas, stars,
                                                2, 1.0, dust)
        assert out.shape == (1, 2, 2) and np.all(out >= 0)
        assert np.all((T > 0) & (T <= 1))
    with pytest.raises(ValueError, match="Extinction model 'InvalidModel' is not available"):
        do.apply_spaxel_extinction(spectra, np.array([5000.0, 6000.0]), gas, stars, 2, 1.0,
                                   dict(extinction_model="InvalidModel"))


# --- properties of rubix's column-density algorithm, derived by hand ----------------

def test_column_density_hand_case():
    """One spaxel, cells at z = -1, 0, 1 with extinction 1, 2, 3 (cumulative 1, 3, 6):
    interpolation inside, clamp on the right, linear extrapolation on the left."""
    gz = np.array([0.0, -1.0, 1.0], np.float32)
    gext = np.array([2.0, 1.0, 3.0], np.float32)
    sz = np.array([-0.5, 0.5, 2.0, -3.0], np.float32)
    av = do.spaxel_av(gz, [0, 0, 0], gext, sz, [0, 0, 0, 0], 1)
    np.testing.assert_allclose(av, [2.0, 4.5, 6.0, -3.0], rtol=1e-6)


def test_column_density_other_spaxels_move_far():
    """A cell of another spaxel at negative z becomes (z * 1e30, 0): a star below its
    own spaxel's cells then interpolates towards that far node, i.e. takes (almost)
    the first cumulative value instead of extrapolating."""
    gz = np.array([-1.0, 0.0, -0.2], np.float32)
    gpa = [0, 0, 1]
    gext = np.array([1.0, 2.0, 5.0], np.float32)
    av = do.spaxel_av(gz, gpa, gext, np.array([-3.0, -0.1], np.float32), [0, 1], 2)
    np.testing.assert_allclose(av[0], 1.0, rtol=1e-6)
    # star of spaxel 1 above its only cell (cumulative 5): the far positive node is
    # spaxel 0's z = 0 cell at 0 * 1e30 = 0 with value 0 -> interpolation towards 0
    np.testing.assert_allclose(av[1], 5.0 * (0.0 - (-0.1)) / (0.0 - (-0.2)), rtol=1e-6)


def test_column_density_no_gas_in_spaxel():
    gz = np.array([0.5, -0.5], np.float32)
    av = do.spaxel_av(gz, [1, 1], np.array([1.0, 1.0], np.float32),
                      np.array([0.0, 3.0, -2.0], np.float32), [0, 0, 0], 2)
    np.testing.assert_array_equal(av, [0.0, 0.0, 0.0])


# --- the package's host-side curves and parameters against the oracle ----------------

def test_host_curves_match_oracle():
    from rubix_gb300 import dust

    w = np.concatenate([np.linspace(0.05, 40.0, 40001),
                        [0.09, 0.3, 0.33, 0.9, 1.0, 1.1, 3.3, 5.9, 8.0, 10.0, 35.0]])
    for Rv in (2.3, 3.1, 5.6):
        for ref, got in ((do.cardelli89, dust.cardelli89), (do.gordon23, dust.gordon23)):
            a, b = ref(w, Rv), got(w, Rv)
            ok = np.isfinite(a)
            assert np.array_equal(ok, np.isfinite(b))
            np.testing.assert_allclose(b[ok], a[ok], rtol=1e-12, atol=1e-12)


def test_host_exponent_and_scale():
    from rubix_gb300 import dust, telescope

    wt = telescope.calculate_wave_seq((4700.15, 9351.4), 1.25)
    for model in dust.RV_MODELS:
        e = dust.extinction_exponent(wt, model, 3.1)
        ax = do.axav(model, (wt.astype(np.float32) / np.float32(1e4)).astype(np.float64), 3.1)
        np.testing.assert_allclose(e, -0.4 * np.log2(10.0) * ax, rtol=1e-6)
        np.testing.assert_allclose(2.0 ** (e.astype(np.float64) * 1.7),
                                   do.extinguish(ax, 1.7)[0], rtol=2e-6)
    assert dust.extinction_scale(3.5) == pytest.approx(do.extinction_scale(3.5), rel=1e-15)
    with pytest.raises(ValueError, match="Extinction model 'Fitz99' is not available"):
        dust.axav("Fitz99", wt, 3.1)


@pytest.mark.parametrize("model", ["power law slope free", "broken power law fit"])
@pytest.mark.parametrize("xco", ["MW", "Z"])
def test_host_dust_to_gas_params(model, xco):
    from rubix_gb300 import dust

    p, broken = dust.dust_to_gas_params(model, xco)
    g = np.linspace(6.0, 10.0, 81).astype(np.float32)
    y = np.where((g > np.float32(p[5])) | (not broken),
                 np.float32(p[1]) + np.float32(p[2]) * (np.float32(p[0]) - g),
                 np.float32(p[3]) + np.float32(p[4]) * (np.float32(p[0]) - g))
    np.testing.assert_allclose(1.0 / 10.0 ** y.astype(np.float64),
                               do.dust_to_gas_ratio(g, model, xco), rtol=2e-6)


def test_get_extinction_config_errors():
    """rubix tests/test_dust_extinction.py:209-227."""
    from rubix_gb300.core import get_extinction

    with pytest.raises(ValueError, match="Dust configuration not found in config file."):
        get_extinction({"ssp": {}, "galaxy": {"dist_z": 0.1}})
    with pytest.raises(ValueError, match="Extinction model not found in dust configuration."):
        get_extinction({"ssp": {"dust": {}}, "galaxy": {"dist_z": 0.1}})


def test_float64_mode_follows_the_float32_restatement():
    """The float64 evaluation (used for differences) takes the same steps: A_V and the
    per-cell extinction agree with the float32 restatement to float32 rounding."""
    from rubix_gb300 import synth

    rng = np.random.Generator(np.random.PCG64(11))
    gz = rng.normal(0.0, 1.0, 400).astype(np.float32)
    sz = rng.normal(0.0, 1.5, 600).astype(np.float32)
    gpa = rng.integers(0, 9, 400).astype(np.int32)
    spa = rng.integers(0, 9, 600).astype(np.int32)
    gext = rng.uniform(0.0, 0.2, 400).astype(np.float32)
    a32 = do.spaxel_av(gz, gpa, gext, sz, spa, 9)
    a64 = do.spaxel_av(gz, gpa, gext, sz, spa, 9, dtype=np.float64)
    assert a64.dtype == np.float64
    assert np.max(np.abs(a64 - a32)) <= 1e-5 * np.max(np.abs(a32))
    g = synth.make_gas(1000, seed=2)
    e32 = do.gas_extinction(g.mass, g.metals, 0.1)
    e64 = do.gas_extinction(g.mass, g.metals, 0.1, dtype=np.float64)
    np.testing.assert_allclose(e64, e32, rtol=1e-5)
