"""Gradients of the differentiation workload against central finite differences.

Workload ``diff``: 2e5 particles, 50 x 50 spaxels x 3721 wavelengths, SSP grid 221 x 6 x
1221, PSF 15 x 15 sigma 1.5, LSF sigma 1.2 A.  Loss L = sum w (cube - target)^2 with
the target rendered from perturbed parameters (mass x 1.05, age and metallicity +0.1
dex, v_los +20 km/s, sigma_PSF x 1.1) and w = 1 / ((target / 20)^2 + floor), floor =
1e-6 max(target)^2.  Gradients (``render_cube`` with ``log_age=True``): dL/dmass,
dL/dlog10(age), dL/dZ and dL/dv_los of 64 particles -- 32 in spaxels holding more
than 256 particles, whose sums the kernels split into chunks, and 32 others -- and
dL/dsigma_PSF, dL/dsigma_LSF.  rubix has no gradient of its own
(rubix/core/pipeline.py:204-208) and jax.grad cannot run here, so finite differences
are the check.  Central differences, step h = 1e-3 relative (log-age: 1e-3 dex).

Which particles.  A central difference measures the derivative only where the function
is smooth on [theta - h, theta + h].  The bilinear SSP lookup has kinks at the grid
nodes (221 ages: nodes 0.0097 dex apart, so a 1e-3 dex step straddles one for about
one particle in five), and the resampling's in-range mask jumps when a node of the
Doppler-shifted SSP grid crosses an end of the telescope range.  The 64 particles are
drawn (seeded) from those whose intervals cross no age or metallicity node and change
no in-range mask entry; the kinks where a shifted SSP node passes a telescope
wavelength (about two per velocity interval) remain, and set the elementwise bound of
the velocity check below.

Two kinds of differences.
* Differences of the float64 oracle's forward (``particle_objective`` with a smooth
  float64 grid and float64 queries) under the loss adjoint of the GPU cube: the
  derivative of the model itself; the GPU gradients must match them to 1e-3 normwise
  over the 64 particles and elementwise on those above 1e-2 of the largest (v_los:
  1e-2 elementwise, the kinks above; a second check with a kink-free step of 1e-6
  relative holds v_los to 1e-3 elementwise as well).  The widths: differences of the float64 PSF and
  LSF applied to the GPU's accumulated cube, to 1e-3.
* Differences of the float32 GPU forward itself.  For one particle they are taken on
  its own contribution: the cube is a sum of per-particle spectra passed through the
  linear LSF and PSF, so L(theta_p +- h) = L(C + delta+-) with delta+- = c_p(theta_p
  +- h) - c_p(theta_p), c_p the particle rendered alone by the same kernels, and
  L(C + delta+) - L(C + delta-) = sum w (delta+ - delta-)(2 (C - target) + delta+ +
  delta-) in float64 (differencing two full renders would add the float32 rounding of
  the ~1e5 other contributions to each spaxel sum, larger than a 1e-3 change of one
  particle).  The float32 cube of one particle changes by ~1e-4 of its value for a
  1e-3 step in Z or age, so these differences carry ~1e-3 of rounding noise: bound
  5e-3 (mass, linear: 1e-3).  In v the float32 forward is a step function: the Doppler
  factor fl32(exp(v/c)) moves by one ulp (6e-8) per 0.02 km/s, so a 1e-3 relative step
  (0.1 km/s at 100 km/s) spans a few ulps; these differences take a step of 2 km/s
  (about 100 ulps) and are bounded by 5e-2 normwise (the interval then holds tens of
  the kinks above, whose slopes the difference averages).  The widths use two full
  float32 renders: bound 2e-3.
"""

import numpy as np
import pytest

import oracle
from helpers import to_dev, workload

pytestmark = pytest.mark.gpu

H_REL = 1e-3          # central-difference step, relative (log-age: 1e-3 dex)
FD_RTOL = 1e-3        # gradients vs differences of the float64 model
FD_RTOL_V_ELEM = 1e-2  # v elementwise: kinks where shifted SSP nodes pass telescope bins
GPU_FD_RTOL = {"mass": 1e-3, "metallicity": 5e-3, "log_age": 5e-3, "v_los": 5e-2,
               "sigma_psf": 2e-3, "sigma_lsf": 2e-3}
GPU_V_STEP = 2.0      # km/s: v step of the float32-forward differences (see above)
N_DENSE, N_RANDOM = 32, 32


def _errors(got, want):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    scale = np.max(np.abs(want))
    err = np.abs(got - want)
    big = np.abs(want) > 1e-2 * scale
    return float(np.max(err) / scale), float(np.max(err[big] / np.abs(want[big])))


def _steps(x, name, gpu=False):
    x = np.asarray(x, dtype=np.float64)
    if name == "log_age":
        return np.full(x.shape, H_REL)
    if name == "v_los":
        return np.full(x.shape, GPU_V_STEP) if gpu else H_REL * np.maximum(np.abs(x), 1.0)
    return H_REL * np.abs(x)


def smooth_intervals(w, mass, met, log_age, v):
    """True where the central-difference intervals of (Z, log-age, v) cross no SSP grid
    node and change no in-range mask entry of the shifted grid (float32 grid of the
    kernels and float64 grid of the oracle)."""
    zg = w.ssp.metallicity.astype(np.float64)
    ag = w.ssp.age.astype(np.float64)
    ok = np.ones(np.shape(mass), dtype=bool)
    for grid, x in ((zg, np.asarray(met, np.float64)),
                    (np.log10(ag), np.asarray(log_age, np.float64))):
        h = _steps(x, "log_age" if grid is not zg else "metallicity")
        lo, hi = x - 2 * h, x + 2 * h
        ok &= (np.searchsorted(grid, lo, "right") == np.searchsorted(grid, hi, "right"))
        ok &= (lo > grid[0]) & (hi < grid[-1])
    vv = np.asarray(v, np.float64)
    hv = np.maximum(_steps(vv, "v_los"), _steps(vv, "v_los", gpu=True))
    lt0, lt1 = float(w.wave_t.min()), float(w.wave_t.max())
    wz = w.wave_z.astype(np.float32)

    def in_range(shift):
        return [(g >= lt0) & (g <= lt1) for g in
                (oracle.doppler_grid(wz, (vv + shift * hv).astype(np.float32)),
                 oracle.doppler_grid(wz, vv + shift * hv, smooth=True))]

    for lo, hi in zip(in_range(-2.0), in_range(2.0)):
        ok &= np.all(lo == hi, axis=1)
    return ok


@pytest.fixture(scope="module")
def fd_case(rubix_lib):
    return make_fd_case()


def make_fd_case():
    import torch

    from rubix_gb300.api import IFURenderer
    from rubix_gb300.autograd import render_cube

    w = workload("diff", edge_cases=False)
    p = w.particles
    r = IFURenderer.from_workload(w, psf=False, lsf=False)
    dev = torch.device("cuda")
    coords = to_dev(p.coords)
    mass0, met0, vel0 = to_dev(p.mass), to_dev(p.metallicity), to_dev(p.velocity)
    la_np = np.log10(p.age.astype(np.float64)).astype(np.float32)
    la0 = to_dev(la_np)
    f64 = dict(dtype=torch.float64, device=dev)
    sp0, sl0 = float(w.psf_sigma), float(w.lsf_sigma)

    def render(c, v, m, z, la, sp, sl):
        return render_cube(r, c, v, m, z, la, sp, sl, w.psf_size, w.wave_res, log_age=True)

    with torch.no_grad():
        vt = vel0.clone()
        vt[:, 2] += 20.0
        target = render(coords, vt, mass0 * 1.05, met0 * np.float32(10 ** 0.1), la0 + 0.1,
                        torch.tensor(sp0 * 1.1, **f64), torch.tensor(sl0, **f64)).double()
        floor = 1e-6 * float(target.abs().max()) ** 2
        weight = 1.0 / ((target / 20.0) ** 2 + floor)

    leaves = [t.clone().requires_grad_() for t in (mass0, met0, la0, vel0)]
    sp = torch.tensor(sp0, requires_grad=True, **f64)
    sl = torch.tensor(sl0, requires_grad=True, **f64)
    cube = render(coords, leaves[3], leaves[0], leaves[1], leaves[2], sp, sl)
    D = cube.double() - target
    loss = (weight * D * D).sum()
    loss.backward()
    torch.cuda.synchronize()
    grads = {"mass": leaves[0].grad.cpu().numpy(), "metallicity": leaves[1].grad.cpu().numpy(),
             "log_age": leaves[2].grad.cpu().numpy(), "v_los": leaves[3].grad[:, 2].cpu().numpy(),
             "sigma_psf": float(sp.grad), "sigma_lsf": float(sl.grad)}
    D = D.detach()

    # the particles: kept, smooth on their difference intervals, half in chunked spaxels
    idx = oracle.square_spaxel_assignment(p.coords, w.edges)
    keep = oracle.mask_particles_outside_aperture(p.coords, w.edges)
    nseg = w.sbin * w.sbin
    counts = np.bincount(idx[keep], minlength=nseg)
    rng = np.random.default_rng(3)
    cand = rng.choice(np.nonzero(keep)[0], 4096, replace=False)
    cand = cand[smooth_intervals(w, p.mass[cand], p.metallicity[cand], la_np[cand],
                                 p.velocity[cand, 2])]
    dense = cand[counts[idx[cand]] > 256]
    other = cand[counts[idx[cand]] <= 256]
    sel = np.concatenate([dense[:N_DENSE], other[:N_RANDOM]])
    assert sel.size == N_DENSE + N_RANDOM

    def own_cube(i, m, z, la, v):
        """Particle i rendered alone (float32 inputs, shape (1,))."""
        with torch.no_grad():
            vel = vel0[i:i + 1].clone()
            vel[0, 2] = float(v)
            return render(coords[i:i + 1], vel, torch.tensor([m], device=dev),
                          torch.tensor([z], device=dev), torch.tensor([la], device=dev),
                          torch.tensor(sp0, **f64), torch.tensor(sl0, **f64)).double()

    def loss_diff(dp, dm):
        return float((weight * (dp - dm) * (2.0 * D + dp + dm)).sum())

    fd = {k: np.zeros(sel.size) for k in ("mass", "metallicity", "log_age", "v_los")}
    base_vals = {"mass": p.mass, "metallicity": p.metallicity, "log_age": la_np,
                 "v_los": p.velocity[:, 2]}
    for j, i in enumerate(sel):
        x = {k: np.float32(base_vals[k][i]) for k in base_vals}
        c0 = own_cube(i, x["mass"], x["metallicity"], x["log_age"], x["v_los"])
        for k in fd:
            step = float(_steps(x[k], k, gpu=True))
            hi, lo = dict(x), dict(x)
            hi[k] = np.float32(float(x[k]) + step)
            lo[k] = np.float32(float(x[k]) - step)
            cp = own_cube(i, hi["mass"], hi["metallicity"], hi["log_age"], hi["v_los"]) - c0
            cm = own_cube(i, lo["mass"], lo["metallicity"], lo["log_age"], lo["v_los"]) - c0
            fd[k][j] = loss_diff(cp, cm) / (float(hi[k]) - float(lo[k]))

    # the widths through the GPU forward: two full renders each
    def full_loss(sp_v, sl_v):
        with torch.no_grad():
            c = render(coords, vel0, mass0, met0, la0, torch.tensor(sp_v, **f64),
                       torch.tensor(sl_v, **f64)).double()
            d = c - target
            return float((weight * d * d).sum())

    fd_sig = {"sigma_psf": (full_loss(sp0 * (1 + H_REL), sl0) -
                            full_loss(sp0 * (1 - H_REL), sl0)) / (2 * H_REL * sp0),
              "sigma_lsf": (full_loss(sp0, sl0 * (1 + H_REL)) -
                            full_loss(sp0, sl0 * (1 - H_REL))) / (2 * H_REL * sl0)}

    # float64 model: the accumulated cube of the GPU (widths), the loss adjoint at each
    # particle's spaxel (LSF and PSF are self-adjoint: symmetric taps, odd sizes)
    from rubix_gb300 import ops

    with torch.no_grad():
        idx_d, mask_d = r.assign(coords)
        perm, offs = r.sort(idx_d, mask_d)
        A = ops.cube_forward(r.ssp_flux, r.ssp_metallicity, r.ssp_age, r.ssp_wave_z,
                             r.wave_t, mass0, met0, torch.pow(10.0, la0), vel0, 2, perm, offs,
                             nseg)
    A = A.view(w.sbin, w.sbin, -1).cpu().numpy().astype(np.float64)
    g = (2.0 * weight * D).cpu().numpy()
    K = oracle.gaussian_kernel_2d(w.psf_size, w.psf_size, w.psf_sigma)
    adj = oracle.apply_lsf(oracle.apply_psf(g, K), w.lsf_sigma, w.wave_res).reshape(nseg, -1)
    ages = torch.pow(10.0, la0).cpu().numpy()
    return dict(w=w, sel=sel, grads=grads, fd=fd, fd_sig=fd_sig, adj=adj[idx[sel]], ages=ages,
                la=la_np, A=A, target=target.cpu().numpy(), weight=weight.cpu().numpy(),
                loss=float(loss.detach()))


def _oracle_fd(case, name, scale=1.0):
    """Central differences (step ``scale`` x the standard step) of the float64 model of
    each selected particle's term sum_t adj_t c_p[t] (the loss is quadratic in the cube:
    its derivative along one particle is that term's derivative)."""
    w, sel = case["w"], case["sel"]
    p = w.particles
    x = {"mass": p.mass[sel].astype(np.float64), "metallicity": p.metallicity[sel].astype(np.float64),
         "log_age": case["la"][sel].astype(np.float64), "v_los": p.velocity[sel, 2].astype(np.float64)}
    grid = (w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z, w.wave_t, case["adj"])
    h = scale * _steps(x[name], name)

    def f(xx):
        return oracle.particle_objective(xx["mass"], xx["metallicity"], 10.0 ** xx["log_age"],
                                         xx["v_los"], *grid, smooth=True)

    hi, lo = dict(x), dict(x)
    hi[name] = x[name] + h
    lo[name] = x[name] - h
    return (f(hi) - f(lo)) / (2 * h)


@pytest.mark.parametrize("name", ["mass", "metallicity", "log_age", "v_los"])
def test_particle_gradients_vs_model_differences(fd_case, name):
    got = fd_case["grads"][name][fd_case["sel"]]
    norm, elem = _errors(got, _oracle_fd(fd_case, name))
    print(f"dL/d{name} vs central differences of the float64 model (64 particles): "
          f"normwise {norm:.2e}, elementwise {elem:.2e}")
    assert norm <= FD_RTOL
    assert elem <= (FD_RTOL_V_ELEM if name == "v_los" else FD_RTOL)


def test_velocity_gradient_vs_kink_free_differences(fd_case):
    """A step of 1e-6 relative (1e-4 km/s at 100 km/s) moves the shifted SSP nodes by
    ~2e-6 A, so its interval holds no node passing a telescope wavelength: the float64
    model's difference is then the derivative itself."""
    got = fd_case["grads"]["v_los"][fd_case["sel"]]
    norm, elem = _errors(got, _oracle_fd(fd_case, "v_los", scale=1e-3))
    print(f"dL/dv_los vs kink-free central differences (step 1e-6 relative) of the float64 "
          f"model: normwise {norm:.2e}, elementwise {elem:.2e}")
    assert norm <= FD_RTOL and elem <= FD_RTOL


@pytest.mark.parametrize("name", ["mass", "metallicity", "log_age", "v_los"])
def test_particle_gradients_vs_gpu_forward_differences(fd_case, name):
    got = fd_case["grads"][name][fd_case["sel"]]
    norm, elem = _errors(got, fd_case["fd"][name])
    print(f"dL/d{name} vs central differences of the float32 GPU forward (64 particles): "
          f"normwise {norm:.2e}, elementwise {elem:.2e}")
    assert norm <= GPU_FD_RTOL[name]


def _model_width_loss(case, sp, sl):
    w = case["w"]
    K = oracle.gaussian_kernel_2d(w.psf_size, w.psf_size, sp)
    c = oracle.apply_lsf(oracle.apply_psf(case["A"], K), sl, w.wave_res)
    d = c - case["target"]
    return float(np.sum(case["weight"] * d * d))


@pytest.mark.parametrize("name", ["sigma_psf", "sigma_lsf"])
def test_width_gradients_vs_differences(fd_case, name):
    w = fd_case["w"]
    sp0, sl0 = float(w.psf_sigma), float(w.lsf_sigma)
    got, want32 = fd_case["grads"][name], fd_case["fd_sig"][name]
    if name == "sigma_psf":
        want = (_model_width_loss(fd_case, sp0 * (1 + H_REL), sl0) -
                _model_width_loss(fd_case, sp0 * (1 - H_REL), sl0)) / (2 * H_REL * sp0)
    else:
        want = (_model_width_loss(fd_case, sp0, sl0 * (1 + H_REL)) -
                _model_width_loss(fd_case, sp0, sl0 * (1 - H_REL))) / (2 * H_REL * sl0)
    rel, rel32 = abs(got - want) / abs(want), abs(got - want32) / abs(want32)
    print(f"dL/d{name}: {got:.6e}; central differences of the float64 convolutions "
          f"{want:.6e} (rel {rel:.2e}), of the float32 GPU forward {want32:.6e} "
          f"(rel {rel32:.2e}); loss {fd_case['loss']:.4e}")
    assert rel <= FD_RTOL
    assert rel32 <= GPU_FD_RTOL[name]
