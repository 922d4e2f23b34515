"""The adjoint kernel and DatacubeFunction against the oracle's analytic gradients
(which tests/test_oracle_grads.py pins to finite differences)."""

import numpy as np
import pytest

import oracle
from helpers import to_dev, workload

pytestmark = pytest.mark.gpu

# float32 kernels vs float64 oracle: normwise over particles, and per particle where
# the oracle gradient exceeds 1e-2 of the largest
GRAD_NORM_RTOL = 1e-4
GRAD_ELEM_RTOL = 1e-3


def _compare(name, got, want):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    scale = np.max(np.abs(want))
    assert scale > 0, name
    err = np.abs(got - want)
    assert np.max(err) <= GRAD_NORM_RTOL * scale, (name, np.max(err) / scale)
    big = np.abs(want) > 1e-2 * scale
    assert np.max(err[big] / np.abs(want[big])) <= GRAD_ELEM_RTOL, name


@pytest.fixture(scope="module")
def grad_case():
    import torch

    from rubix_gb300.api import IFURenderer
    from rubix_gb300.autograd import render_cube

    w = workload("small", n=2000)
    p = w.particles
    L = w.wave_t.size
    rng = np.random.default_rng(7)
    W = rng.standard_normal((w.sbin, w.sbin, L)).astype(np.float32)
    r = IFURenderer.from_workload(w, psf=False, lsf=False)
    mass = to_dev(p.mass).requires_grad_()
    met = to_dev(p.metallicity).requires_grad_()
    age = to_dev(p.age).requires_grad_()
    vel = to_dev(p.velocity).requires_grad_()
    sp = torch.tensor(w.psf_sigma, dtype=torch.float64, device="cuda", requires_grad=True)
    sl = torch.tensor(w.lsf_sigma, dtype=torch.float64, device="cuda", requires_grad=True)
    cube = render_cube(r, to_dev(p.coords), vel, mass, met, age, sp, sl, w.psf_size, w.wave_res)
    loss = (cube.double() * to_dev(W).double()).sum()
    loss.backward()
    torch.cuda.synchronize()
    got = {"mass": mass.grad.cpu().numpy(), "metallicity": met.grad.cpu().numpy(),
           "age": age.grad.cpu().numpy(), "vel": vel.grad.cpu().numpy(),
           "sigma_psf": float(sp.grad), "sigma_lsf": float(sl.grad),
           "cube": cube.detach().cpu().numpy()}
    return w, W, got


def test_forward_cube_matches_oracle(grad_case):
    from helpers import assert_cube_close, oracle_stages

    w, _, got = grad_case
    ref = oracle_stages("small", n=2000)
    assert_cube_close(got["cube"], ref["final"], what="differentiable forward")


def test_particle_gradients(grad_case):
    w, W, got = grad_case
    p = w.particles
    L = w.wave_t.size
    mask, f = oracle.filter_particles(p.coords, w.edges, mass=p.mass, metallicity=p.metallicity,
                                      age=p.age)
    idx = oracle.square_spaxel_assignment(p.coords, w.edges).astype(np.int64)
    nseg = w.sbin * w.sbin
    K = oracle.gaussian_kernel_2d(w.psf_size, w.psf_size, w.psf_sigma)
    # symmetric taps, odd sizes: PSF and LSF are self-adjoint
    h = oracle.apply_lsf(oracle.apply_psf(W.astype(np.float64), K), w.lsf_sigma,
                         w.wave_res).reshape(nseg, L)
    keep = mask & (idx >= 0) & (idx < nseg)
    rows = np.zeros((p.n, L))
    rows[keep] = h[idx[keep]]
    want = oracle.particle_grads(f["mass"], f["metallicity"], f["age"], p.velocity[:, 2],
                                 w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z, w.wave_t,
                                 rows)
    want = [np.where(keep, x, 0.0) for x in want]
    _compare("dL/dmass", got["mass"], want[0])
    _compare("dL/dmetallicity", got["metallicity"], want[1])
    _compare("dL/dage", got["age"], want[2])
    _compare("dL/dv_los", got["vel"][:, 2], want[3])
    assert np.all(got["vel"][:, :2] == 0)
    assert np.all(got["mass"][~keep] == 0)


def test_width_gradients(grad_case):
    w, W, got = grad_case
    ref = oracle.render_cube(*(getattr(w.particles, k) for k in
                               ("coords", "velocity", "mass", "metallicity", "age")),
                             w.edges, w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux,
                             w.ssp.wavelength, w.dist_z, w.wave_t)
    raw = ref["cube"]
    Wd = W.astype(np.float64)
    t, dt = oracle.psf_taps_derivative(w.psf_size, w.psf_sigma)
    lsf_cube = oracle.apply_lsf(raw, w.lsf_sigma, w.wave_res)
    dK = np.outer(dt, t) + np.outer(t, dt)
    want_psf = np.sum(Wd * oracle.apply_psf(lsf_cube, dK))
    # dL/dsigma_lsf by central differences of the oracle chain (smooth in sigma)
    K = oracle.gaussian_kernel_2d(w.psf_size, w.psf_size, w.psf_sigma)
    psf_cube = oracle.apply_psf(raw, K)
    hs = 1e-4 * w.lsf_sigma
    want_lsf = (np.sum(Wd * oracle.apply_lsf(psf_cube, w.lsf_sigma + hs, w.wave_res)) -
                np.sum(Wd * oracle.apply_lsf(psf_cube, w.lsf_sigma - hs, w.wave_res))) / (2 * hs)
    assert abs(got["sigma_psf"] - want_psf) <= 1e-4 * abs(want_psf), (got["sigma_psf"], want_psf)
    assert abs(got["sigma_lsf"] - want_lsf) <= 1e-3 * abs(want_lsf), (got["sigma_lsf"], want_lsf)


def test_backward_deterministic():
    import torch

    from rubix_gb300 import ops

    w = workload("small", n=1500)
    p = w.particles
    ssp_dev = [to_dev(x) for x in (w.ssp.flux, w.ssp.metallicity, w.ssp.age, w.wave_z)]
    idx = ops.spaxel_assign(to_dev(p.coords), to_dev(w.edges))
    nseg = w.sbin * w.sbin
    perm, offs = ops.spaxel_sort(idx, nseg)
    rng = np.random.default_rng(1)
    adj = to_dev(rng.standard_normal((nseg, w.wave_t.size)).astype(np.float32))
    outs = [ops.cube_backward(*ssp_dev, to_dev(w.wave_t), to_dev(p.mass), to_dev(p.metallicity),
                              to_dev(p.age), to_dev(p.velocity), 2, perm, offs, nseg, adj)
            for _ in range(2)]
    torch.cuda.synchronize()
    for a, b in zip(*outs):
        assert torch.equal(a, b)


@pytest.mark.parametrize("m", [1, 4, 11, 15, 16])
def test_device_taps_match_host(m):
    """rubix_gauss_taps (sigma on the device) gives the host taps, derivatives and
    adjoint taps of the PSF and LSF."""
    import torch

    from rubix_gb300 import autograd as ag
    from rubix_gb300 import ops

    for sigma in (0.7, 1.5, 3.0):
        sg = torch.tensor(sigma, dtype=torch.float64, device="cuda")
        t, dt, rt = (x.cpu().numpy() for x in ops.gauss_taps(sg, ag._psf_positions(m),
                                                            reversed_pad=(m % 2 == 0)))
        ht, hdt = ag.psf_taps_grad(m, sigma)
        np.testing.assert_allclose(t, ht, rtol=1e-6, atol=1e-9)
        np.testing.assert_allclose(dt, hdt, rtol=1e-5, atol=1e-8)
        np.testing.assert_allclose(rt, ag._psf_adjoint_taps(ht), rtol=1e-6, atol=1e-9)
    sg = torch.tensor(1.2, dtype=torch.float64, device="cuda")
    t, dt, rt = (x.cpu().numpy() for x in ops.gauss_taps(sg, ag._lsf_positions(1.25)))
    ht, hdt = ag.lsf_taps_grad(1.2, 1.25)
    np.testing.assert_allclose(t, ht, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(dt, hdt, rtol=1e-5, atol=1e-8)
    np.testing.assert_allclose(rt, ht[::-1], rtol=1e-6, atol=1e-9)


def test_sigma_tensors_need_no_readback(grad_case):
    """With CUDA sigma tensors the forward and backward issue no device-to-host copy:
    the same gradients come out when the stream is captured in a CUDA graph (a capture
    fails on any synchronising call)."""
    import torch

    from rubix_gb300.api import IFURenderer
    from rubix_gb300.autograd import render_cube

    w, W, got = grad_case
    p = w.particles
    r = IFURenderer.from_workload(w, psf=False, lsf=False)
    coords = to_dev(p.coords)
    mass = to_dev(p.mass).requires_grad_()
    met, age, vel = to_dev(p.metallicity), to_dev(p.age), to_dev(p.velocity)
    sp = torch.tensor(w.psf_sigma, dtype=torch.float64, device="cuda", requires_grad=True)
    sl = torch.tensor(w.lsf_sigma, dtype=torch.float64, device="cuda", requires_grad=True)
    Wd = to_dev(W).double()
    idx, mask = r.assign(coords)
    perm, offs = r.sort(idx, mask)
    from rubix_gb300.autograd import DatacubeFunction

    def step():
        cube = DatacubeFunction.apply(mass, met, age, vel, sp, sl, r, perm, offs, w.psf_size,
                                      w.wave_res)
        (cube.double() * Wd).sum().backward()

    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        step()  # warm-up outside the capture (allocations, library load)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    for t in (mass, sp, sl):
        t.grad = None
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step()
    g.replay()
    torch.cuda.synchronize()
    np.testing.assert_allclose(mass.grad.cpu().numpy(), got["mass"], rtol=1e-5,
                               atol=1e-6 * float(np.abs(got["mass"]).max()))
    assert abs(float(sp.grad) - got["sigma_psf"]) <= 1e-5 * abs(got["sigma_psf"])
    assert abs(float(sl.grad) - got["sigma_lsf"]) <= 1e-5 * abs(got["sigma_lsf"])
