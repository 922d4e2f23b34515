"""CPU checks of the gradient restatement: the oracle's analytic particle gradients
against central/one-sided finite differences of the oracle itself, the PSF/LSF tap
derivatives, and the adjoint identities the backward pass relies on."""

import numpy as np
import pytest

import oracle
from helpers import workload
from rubix_gb300 import autograd as rag

N_FD = 96


@pytest.fixture(scope="module")
def fd_case():
    w = workload("small", n=400)
    p = w.particles
    rng = np.random.default_rng(3)
    sel = rng.choice(p.n - 14, N_FD, replace=False)  # regular particles, not the edge cases
    adj = rng.standard_normal((N_FD, w.wave_t.size))
    q = {k: getattr(p, k)[sel].astype(np.float64) for k in ("mass", "metallicity", "age")}
    q["v"] = p.velocity[sel, 2].astype(np.float64)
    args = (w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z, w.wave_t, adj)
    return q, args


def _objective(q, args, **over):
    d = dict(q)
    d.update(over)
    return oracle.particle_objective(d["mass"], d["metallicity"], d["age"], d["v"], *args,
                                     smooth=True)


@pytest.mark.parametrize("name,idx,rel_step", [
    ("mass", 0, 1e-4), ("metallicity", 1, 1e-6), ("age", 2, 1e-6), ("v", 3, None)])
def test_particle_grads_vs_finite_differences(fd_case, name, idx, rel_step):
    q, args = fd_case
    g = oracle.particle_grads(q["mass"], q["metallicity"], q["age"], q["v"], *args, smooth=True)
    base = q[name]
    h = np.full_like(base, 0.002) if rel_step is None else rel_step * np.abs(base)
    f0 = _objective(q, args)
    fp = _objective(q, args, **{name: base + h})
    fm = _objective(q, args, **{name: base - h})
    central, right, left = (fp - fm) / (2 * h), (fp - f0) / h, (f0 - fm) / h
    scale = np.max(np.abs(central))
    # a telescope wavelength sitting on an SSP node is a kink of I(v): the analytic
    # derivative then equals one of the one-sided differences
    err = np.min(np.abs(np.stack([central, right, left]) - g[idx][None, :]), axis=0)
    assert np.max(err) <= 1e-4 * scale, (name, np.max(err) / scale)


def test_tap_derivatives():
    for m, s in ((15, 1.5), (11, 1.0), (8, 2.0)):
        t, dt = rag.psf_taps_grad(m, s)
        t2, dt2 = oracle.psf_taps_derivative(m, s)
        np.testing.assert_allclose(t, t2, rtol=1e-14)
        np.testing.assert_allclose(dt, dt2, rtol=1e-12, atol=1e-15)
        h = 1e-6
        fd = (rag.psf_taps_grad(m, s + h)[0] - rag.psf_taps_grad(m, s - h)[0]) / (2 * h)
        np.testing.assert_allclose(dt, fd, atol=1e-8)
        assert np.allclose(np.outer(t, t), oracle.gaussian_kernel_2d(m, m, s), atol=1e-15)
    t, dt = rag.lsf_taps_grad(1.2, 1.25)
    np.testing.assert_allclose(t, oracle.lsf_kernel(1.2, 1.25), rtol=1e-14)
    fd = (rag.lsf_taps_grad(1.2 + 1e-6, 1.25)[0] - rag.lsf_taps_grad(1.2 - 1e-6, 1.25)[0]) / 2e-6
    np.testing.assert_allclose(dt, fd, atol=1e-8)


@pytest.mark.parametrize("m", [3, 4, 7, 15])
def test_psf_adjoint_taps(m):
    """<W, PSF_t(x)> = <PSF_adj(t)(W), x> with the oracle's 'same' convolution."""
    rng = np.random.default_rng(m)
    t = rng.random(m)
    x = rng.standard_normal((9, 11, 3))
    W = rng.standard_normal((9, 11, 3))
    ta = rag._psf_adjoint_taps(t)
    lhs = np.sum(W * oracle.apply_psf(x, np.outer(t, t), method="direct"))
    rhs = np.sum(oracle.apply_psf(W, np.outer(ta, ta), method="direct") * x)
    assert abs(lhs - rhs) <= 1e-10 * max(1.0, abs(lhs))


def test_lsf_adjoint_crop():
    """out[t] = sum_j k[j] in[t+crop-j]: the adjoint is reversed taps with K-1-crop."""
    rng = np.random.default_rng(5)
    K, crop, L = 9, 3, 40
    k = rng.random(K)
    x = rng.standard_normal((4, L))
    W = rng.standard_normal((4, L))

    def conv(a, taps, c):
        out = np.zeros_like(a)
        for j in range(len(taps)):
            d = c - j
            lo, hi = max(0, -d), min(L, L - d)
            out[:, lo:hi] += taps[j] * a[:, lo + d:hi + d]
        return out

    lhs = np.sum(W * conv(x, k, crop))
    rhs = np.sum(conv(W, k[::-1], K - 1 - crop) * x)
    assert abs(lhs - rhs) <= 1e-10 * max(1.0, abs(lhs))
