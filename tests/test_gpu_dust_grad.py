"""Gradients through the dust column: dL/dA_V of every star from the dusty adjoint,
dL/d(star z) and dL/d(cell extinction) from the A_V adjoint, dL/d(gas mass, H, O)
from the extinction adjoint, and the whole chain through ``render_cube(..., gas=...)``.

rubix differentiates calculate_extinction (rubix/core/dust.py:16-65,
rubix/spectra/dust/dust_extinction.py:169-358) with jax.grad, which cannot run here;
the checks are the oracle's analytic derivative of the transmission and central
differences of the oracle's float64 restatement (``spaxel_av`` and ``gas_extinction``
with ``dtype=np.float64``).  A_V is piecewise linear in a star's z (kinks at the gas
heights) and linear in the cells' extinction, so the differences are exact where no
kink lies inside the step; the stars within 1e-5 kpc of a gas height are left out of
the per-star z check.
"""

import numpy as np
import pytest

import oracle
from helpers import to_dev, workload
from oracle import dust_oracle as do

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-4  # float32 kernels vs float64 references, normwise


def _rel(got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return float(np.max(np.abs(got - want)) / max(np.max(np.abs(want)), 1e-300))


def test_cube_adjoint_av_gradient():
    """rubix_cube_bwd_dust_av's dL/dA_V against the analytic derivative of every
    particle's transmitted spectrum: sum_t a_t c_t T_t (-0.4 ln 10 A(t)/A(V))."""
    import torch

    from rubix_gb300 import dust, ops

    w = workload("small", n=2000)
    p = w.particles
    L = w.wave_t.size
    nseg = w.sbin * w.sbin
    rng = np.random.default_rng(23)
    av = rng.uniform(0.0, 2.5, p.n).astype(np.float32)
    e = dust.extinction_exponent(w.wave_t, "Cardelli89", 3.1)
    idx = oracle.square_spaxel_assignment(p.coords, w.edges).astype(np.int64)
    perm, offs = ops.spaxel_sort(to_dev(idx, torch.int32), nseg)
    adj = rng.standard_normal((nseg, L)).astype(np.float32)
    ssp = [to_dev(x) for x in (w.ssp.flux, w.ssp.metallicity, w.ssp.age, w.wave_z)]
    got = ops.cube_backward(*ssp, to_dev(w.wave_t), to_dev(p.mass), to_dev(p.metallicity),
                            to_dev(p.age), to_dev(p.velocity), 2, perm, offs, nseg,
                            to_dev(adj), dust_av=to_dev(av), dust_exponent=to_dev(e),
                            av_grad=True)
    plain = ops.cube_backward(*ssp, to_dev(w.wave_t), to_dev(p.mass), to_dev(p.metallicity),
                              to_dev(p.age), to_dev(p.velocity), 2, perm, offs, nseg,
                              to_dev(adj), dust_av=to_dev(av), dust_exponent=to_dev(e))
    torch.cuda.synchronize()
    for a, b in zip(got[:4], plain):  # the other gradients are unchanged
        assert torch.equal(a, b)
    wave_um = (np.asarray(w.wave_t, np.float32) / np.float32(1e4)).astype(np.float64)
    ax = do.cardelli89(wave_um, 3.1)
    T = do.extinguish(ax, av).astype(np.float64)
    c = oracle.particle_spectra(p.mass, p.metallicity, p.age, p.velocity[:, 2],
                                w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z, w.wave_t)
    keep = (idx >= 0) & (idx < nseg)
    rows = np.zeros((p.n, L))
    rows[keep] = adj.astype(np.float64)[idx[keep]]
    want = np.sum(rows * c * T * (-0.4 * np.log(10.0) * ax)[None, :], axis=1)
    err = _rel(got[4].cpu().numpy(), want)
    print(f"dL/dA_V (cube adjoint) vs the analytic derivative: normwise {err:.2e}")
    assert err <= GRAD_RTOL


def _av_problem(seed, ng, ns, nseg, q2, ties=False):
    from test_gpu_dust import _av_case

    rng = np.random.Generator(np.random.PCG64(seed))
    nb = int(round(np.sqrt(nseg)))
    pa_limit = (nb + 1) ** 2 if q2 else nseg
    gz, gpa, gext, sz, spa = _av_case(rng, ng, ns, nseg, pa_limit, "ties" if ties else "normal")
    return rng, pa_limit, gz, gpa, gext, sz, spa


@pytest.mark.parametrize("ng,nseg,q2,ties", [(3000, 25, False, False), (4000, 100, True, False),
                                             (3000, 25, False, True), (50, 625, False, False)])
def test_av_adjoint_vs_float64_differences(ng, nseg, q2, ties):
    """dL/dz of every star and dL/d ext of the cells for L = sum_i c_i A_V,i."""
    import torch

    from rubix_gb300 import ops

    rng, pa_limit, gz, gpa, gext, sz, spa = _av_problem(ng * 7 + nseg, ng, 3000, nseg, q2, ties)
    c = rng.standard_normal(sz.size)
    gc = np.zeros((ng, 3), np.float32)
    gc[:, 2] = gz
    sc = np.zeros((sz.size, 3), np.float32)
    sc[:, 2] = sz
    g_z, g_ext = ops.dust_av_backward(to_dev(gc), to_dev(gpa), to_dev(gext), to_dev(sc),
                                      to_dev(spa), nseg, pa_limit,
                                      to_dev(c.astype(np.float32)))
    torch.cuda.synchronize()
    g_z, g_ext = g_z.cpu().numpy(), g_ext.cpu().numpy()

    def av64(gext_v, sz_v):
        return do.spaxel_av(gz, gpa, gext_v, sz_v, spa, nseg, dtype=np.float64)

    # stars: each A_V depends on its own z only; away from the gas heights exact
    h = 1e-6
    s64 = sz.astype(np.float64)
    fd_z = c * (av64(gext, s64 + h) - av64(gext, s64 - h)) / (2 * h)
    far = np.min(np.abs(s64[:, None] - gz.astype(np.float64)[None, :]), axis=1) > 1e-5 \
        if ng > 0 else np.ones(sz.size, bool)
    # a star whose bracket pairs its own cell with another spaxel's cell moved to
    # z * 1e30 has a slope near 1e-30: slopes below 1e-12 of the upstream count as 0
    err_z = float(np.max(np.abs(g_z[far] - fd_z[far]), initial=0.0)
                  / max(np.max(np.abs(fd_z[far]), initial=0.0), 1e-12 * np.max(np.abs(c))))
    # cells: L is linear in the extinction; random directions and single cells
    e64 = gext.astype(np.float64)
    errs = []
    dirs = [rng.standard_normal(ng) for _ in range(4)]
    for j in rng.choice(ng, min(ng, 12), replace=False):
        d = np.zeros(ng)
        d[j] = 1.0
        dirs.append(d)
    eps = 1e-3
    for d in dirs:
        fd = np.dot(c, av64(e64 + eps * d, s64) - av64(e64 - eps * d, s64)) / (2 * eps)
        got = float(np.dot(g_ext.astype(np.float64), d))
        scale = max(abs(fd), np.abs(g_ext).max() * np.abs(d).sum() * 1e-3, 1e-30)
        errs.append(abs(got - fd) / scale)
    print(f"A_V adjoint (ng={ng}, nseg={nseg}, q2={q2}, ties={ties}): dL/dz normwise "
          f"{err_z:.2e} over {int(far.sum())} stars; dL/d ext, {len(dirs)} directions: "
          f"worst {max(errs):.2e}")
    assert err_z <= GRAD_RTOL
    assert max(errs) <= GRAD_RTOL


@pytest.mark.parametrize("model,xco", [("broken power law fit", "Z"),
                                       ("power law slope free", "MW")])
def test_gas_extinction_adjoint_vs_float64_differences(model, xco):
    from rubix_gb300 import dust, ops, synth

    g = synth.make_gas(5000, seed=8)
    params, broken = dust.dust_to_gas_params(model, xco)
    area, scale = 0.137, dust.extinction_scale(3.5)
    rng = np.random.default_rng(3)
    c = rng.standard_normal(g.n)
    gm, gmet = ops.dust_gas_extinction_backward(to_dev(g.mass), to_dev(g.metals), params,
                                                broken, scale, area,
                                                to_dev(c.astype(np.float32)))
    gm, gmet = gm.cpu().numpy(), gmet.cpu().numpy()
    cfg = dict(dust_to_gas_model=model, Xco=xco)
    m64, met64 = g.mass.astype(np.float64), g.metals.astype(np.float64)

    def ext(m, met):
        return do.gas_extinction(m, met, area, cfg, dtype=np.float64)

    rel = 1e-6
    fd_m = c * (ext(m64 * (1 + rel), met64) - ext(m64 * (1 - rel), met64)) / (2 * rel * m64)
    out = {"mass": _rel(gm, fd_m)}
    # away from the break of the broken power law (a kink in 12 + log(O/H))
    g_oh = do.log_oh(met64, dtype=np.float64)
    smooth = np.abs(g_oh - 8.10) > 1e-3
    for col, name in ((4, "O"), (0, "H")):
        up, dn = met64.copy(), met64.copy()
        up[:, col] *= 1 + rel
        dn[:, col] *= 1 - rel
        fd = c * (ext(m64, up) - ext(m64, dn)) / (2 * rel * met64[:, col])
        out[name] = _rel(gmet[smooth, col], fd[smooth])
    assert not np.any(np.delete(gmet, [0, 4], axis=1))
    print(f"gas extinction adjoint ({model}, X_CO {xco}): " +
          ", ".join(f"d/d{k} {v:.2e}" for k, v in out.items()))
    assert max(out.values()) <= GRAD_RTOL


def test_dusty_render_gradients_through_the_column():
    """render_cube(..., gas=...) with the stars' coordinates and the gas masses and
    metals requiring gradients: the directional derivatives of L = sum W cube along
    random directions against central differences of the same float32 GPU forward
    (every star's A_V moves and the weights are positive, so the loss changes coherently,
    far above the float32 rounding)."""
    import torch

    from rubix_gb300.api import IFURenderer
    from rubix_gb300.autograd import render_cube
    from test_gpu_dust import _gas

    w = workload("small", n=3000)
    p = w.particles
    g, _ = _gas(3000, seed=12)
    r = IFURenderer.from_workload(w, device="cuda", dust={"extinction_model": "Cardelli89"})
    rng = np.random.default_rng(5)
    # positive weights: L is a coherent sum, far above the rounding of the float32 cube
    W = to_dev(rng.uniform(0.5, 1.5, (w.sbin, w.sbin, w.wave_t.size)).astype(np.float32)).double()
    base = {"coords": to_dev(p.coords), "gmass": to_dev(g.mass), "gmet": to_dev(g.metals)}
    others = [to_dev(x) for x in (p.velocity, p.mass, p.metallicity, p.age)]
    gcoords = to_dev(g.coords)

    def loss(coords, gmass, gmet):
        cube = render_cube(r, coords, others[0], others[1], others[2], others[3], w.psf_sigma,
                           w.lsf_sigma, w.psf_size, w.wave_res, gas=(gcoords, gmass, gmet))
        return (cube.double() * W).sum()

    leaves = {k: v.clone().requires_grad_() for k, v in base.items()}
    loss(leaves["coords"], leaves["gmass"], leaves["gmet"]).backward()
    grads = {k: v.grad.double() for k, v in leaves.items()}
    assert not grads["coords"][:, :2].any()
    assert not grads["gmet"][:, [1, 2, 3, 5, 6, 7, 8, 9]].any()
    out = {}
    for name, eps in (("coords", 1e-3), ("gmass", 1e-3), ("gmet", 1e-3)):
        d = torch.zeros_like(base[name], dtype=torch.float64)
        if name == "coords":
            d[:, 2] = to_dev(rng.standard_normal(p.n)).double()
            step = eps  # kpc
        else:
            d = base[name].double() * to_dev(rng.uniform(-1, 1, tuple(base[name].shape))).double()
            if name == "gmet":
                d[:, [1, 2, 3, 5, 6, 7, 8, 9]] = 0.0
                # rubix's broken power law jumps by ~2.5 % at its break (12 + log(O/H) =
                # 8.10); a difference across the jump is not a derivative: those cells
                # keep their metals
                goh = do.log_oh(g.metals, dtype=np.float64)
                d[to_dev(np.abs(goh - 8.10) < 1e-2)] = 0.0
            step = eps  # relative
        with torch.no_grad():
            args = dict(base)
            args[name] = (base[name].double() + step * d).float()
            lp = float(loss(args["coords"], args["gmass"], args["gmet"]))
            args[name] = (base[name].double() - step * d).float()
            lm = float(loss(args["coords"], args["gmass"], args["gmet"]))
        fd = (lp - lm) / (2 * step)
        an = float((grads[name] * d).sum())
        out[name] = abs(an - fd) / abs(fd)
    print("dusty render, directional derivatives vs central differences of the GPU forward: "
          + ", ".join(f"{k} {v:.2e}" for k, v in out.items()))
    assert out["gmass"] <= 1e-3 and out["gmet"] <= 1e-3
    assert out["coords"] <= 5e-3  # a few stars cross a gas height (kinks) inside the step
