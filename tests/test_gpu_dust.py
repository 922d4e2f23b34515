"""Dust extinction on the GPU against the oracle: per-cell extinction, the stars' A_V
(rubix's column-density interpolation with its 1e30 placement of other spaxels' cells,
ties, empty spaxels, assignments past the last spaxel), the dusty fused cube, the
materialised-spectra path and the calc_dusty_ifu pipeline."""

import numpy as np
import pytest

import oracle
from helpers import assert_cube_close, to_dev, workload
from oracle import dust_oracle as do

pytestmark = pytest.mark.gpu

AV_RTOL = 2e-6  # float32 sums in another order: relative to max |A_V| of the case


def _assert_av_close(got, ref, what="A_V"):
    scale = max(float(np.max(np.abs(ref))) if ref.size else 0.0, 1e-30)
    err = np.max(np.abs(got.astype(np.float64) - ref)) / scale if ref.size else 0.0
    assert err <= AV_RTOL, f"{what}: max |gpu - oracle| / max|oracle| = {err:.3e}"


@pytest.mark.parametrize("model", ["power law slope free", "broken power law fit"])
@pytest.mark.parametrize("xco", ["MW", "Z"])
def test_gas_extinction_kernel(model, xco):
    from rubix_gb300 import dust, ops, synth

    g = synth.make_gas(20000, seed=3)
    metals = g.metals.copy()
    metals[:5, 4] = [0.0, 1e-6, 0.05, 0.02, 0.004]  # no oxygen, very poor, very rich
    params, broken = dust.dust_to_gas_params(model, xco)
    area = 0.137
    got = ops.dust_gas_extinction(to_dev(g.mass), to_dev(metals), params, broken,
                                  dust.extinction_scale(3.5), area).cpu().numpy()
    ref = do.gas_extinction(g.mass, metals, area, dict(dust_to_gas_model=model, Xco=xco))
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=0)


def _av_case(rng, ng, ns, nseg, pa_limit, z_kind="normal"):
    gz = rng.normal(0.0, 1.0, ng).astype(np.float32)
    sz = rng.normal(0.0, 1.5, ns).astype(np.float32)
    if z_kind == "ties":
        gz = np.round(gz * 2) / 2
        sz = np.round(sz * 2) / 2
        gz[:: 7] = 0.0
        gz[1:: 11] = -0.0
        sz[:: 5] = 0.0
    gpa = rng.integers(0, pa_limit, ng).astype(np.int32)
    spa = rng.integers(0, pa_limit, ns).astype(np.int32)
    gext = rng.uniform(0.0, 0.2, ng).astype(np.float32)
    return gz, gpa, gext, sz, spa


def _gpu_av(gz, gpa, gext, sz, spa, nseg, pa_limit):
    from rubix_gb300 import ops

    gc = np.zeros((gz.size, 3), np.float32)
    gc[:, 2] = gz
    sc = np.zeros((sz.size, 3), np.float32)
    sc[:, 2] = sz
    return ops.dust_av(to_dev(gc), to_dev(gpa), to_dev(gext), to_dev(sc), to_dev(spa), nseg,
                       pa_limit).cpu().numpy()


@pytest.mark.parametrize("ng,nseg,q2,z_kind", [
    (3000, 25, False, "normal"), (3000, 25, False, "ties"), (4000, 100, True, "normal"),
    (4000, 100, True, "ties"), (50, 625, False, "normal"), (2, 4, False, "normal"),
    (1, 4, False, "normal"), (0, 9, False, "normal"), (5000, 1, False, "ties"),
])
def test_dust_av_matches_oracle(ng, nseg, q2, z_kind):
    rng = np.random.Generator(np.random.PCG64(ng * 31 + nseg))
    nb = int(round(np.sqrt(nseg)))
    pa_limit = (nb + 1) ** 2 if q2 else nseg
    gz, gpa, gext, sz, spa = _av_case(rng, ng, 3000, nseg, pa_limit, z_kind)
    got = _gpu_av(gz, gpa, gext, sz, spa, nseg, pa_limit)
    ref = do.spaxel_av(gz, gpa, gext, sz, spa, nseg)
    _assert_av_close(got, ref, f"A_V ng={ng} nseg={nseg} q2={q2} {z_kind}")


def test_dust_av_placement_edge_cases():
    """Cells of other spaxels at exactly z = 0 sit inside a spaxel's own range (0 * 1e30
    = 0); tiny |z| lands at ordinary magnitudes; stars on nodes, below and above all."""
    gz = np.array([-1.0, -0.5, 0.5, 1.0, 0.0, 1e-31, -2e-31, 0.0, 3.0], np.float32)
    gpa = np.array([0, 0, 0, 0, 1, 1, 2, 0, 2], np.int32)
    gext = np.array([0.1, 0.2, 0.3, 0.4, 1.0, 2.0, 3.0, 0.05, 0.7], np.float32)
    sz = np.array([-2.0, -1.0, -0.7, -0.2, 0.0, 0.05, 0.2, 0.5, 0.9, 1.0, 5.0, 0.0, -0.1, 4.0,
                   -5.0], np.float32)
    spa = np.array([0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 2, 3], np.int32)
    got = _gpu_av(gz, gpa, gext, sz, spa, 4, 4)
    ref = do.spaxel_av(gz, gpa, gext, sz, spa, 4)
    _assert_av_close(got, ref, "A_V placement cases")


def test_dust_av_large_spot_check():
    """22 500 spaxels, 400 000 cells, 10^6 stars: the oracle on 25 spaxels."""
    from rubix_gb300 import ops, synth

    w = workload("ifu", n=1_000_000, edge_cases=False)
    g = synth.make_gas(400_000, seed=2)
    nseg = w.sbin * w.sbin
    edges = to_dev(w.edges)
    gpa = ops.spaxel_assign(to_dev(g.coords), edges)
    spa = ops.spaxel_assign(to_dev(w.particles.coords), edges)
    gext = np.random.Generator(np.random.PCG64(7)).uniform(0, 0.05, g.n).astype(np.float32)
    pa_limit = (len(w.edges) - 1) ** 2
    got = ops.dust_av(to_dev(g.coords), gpa, to_dev(gext), to_dev(w.particles.coords), spa,
                      nseg, max(pa_limit, nseg)).cpu().numpy()
    spa_h = spa.cpu().numpy()
    centre = (w.sbin // 2) * w.sbin + w.sbin // 2
    pick = np.unique(np.concatenate([[0, nseg - 1, centre, centre + 1, centre + w.sbin],
                                     np.random.Generator(np.random.PCG64(9)).integers(
                                         0, nseg, 20)]))
    ref = do.spaxel_av(g.coords[:, 2], gpa.cpu().numpy(), gext, w.particles.coords[:, 2],
                       spa_h, nseg, spaxels=pick)
    sel = np.isin(np.minimum(spa_h, nseg - 1), pick)
    assert sel.sum() > 1000
    _assert_av_close(got[sel], ref[sel], "A_V large spot check")
    assert np.all(np.isfinite(got))


def _dust_cfg(w, name):
    from test_gpu_steps import _config

    cfg = _config(w, name)
    cfg["pipeline"]["name"] = "calc_dusty_ifu"
    cfg["data"]["args"]["particle_type"] = ["stars", "gas"]
    cfg["ssp"]["dust"] = {"extinction_model": "Cardelli89", "Rv": 3.1,
                          "dust_grain_density": 3.5}
    return cfg


def _gas(n, seed=4):
    from rubix_gb300 import synth

    g = synth.make_gas(n, seed=seed, median_mass=1e6)
    vel = np.random.Generator(np.random.PCG64(seed)).normal(0, 30, (n, 3)).astype(np.float32)
    return g, vel


def _oracle_dusty(w, g, gvel, model="Cardelli89", Rv=3.1, hmr=5.0):
    """The calc_dusty_ifu chain on the oracle: rotation of both components (each by
    its own inertia tensor), filter, assignment, gas extinction, A_V, transmission."""
    from rubix_gb300 import synth
    from rubix_gb300 import telescope as tel

    gc, _ = oracle.rotate_galaxy(g.coords, gvel, g.mass, hmr, 0.0, 0.0, 0.0)
    gmask, gf = oracle.filter_particles(gc, w.edges, mass=g.mass)
    gpa = oracle.square_spaxel_assignment(gc, w.edges)
    _, size = tel.spatial_bin_edges(synth.WORKLOADS[w.name]["fov"], w.sbin, w.dist_z)
    area = float(np.float32(size) ** 2)
    gext = do.gas_extinction(gf["mass"], g.metals, area)
    nseg = w.sbin * w.sbin
    wave_um = (np.asarray(w.wave_t, np.float32) / np.float32(1e4)).astype(np.float32)
    ax = do.axav(model, wave_um.astype(np.float64), Rv)

    def transmission(star_coords):
        spa = oracle.square_spaxel_assignment(star_coords, w.edges)
        av = do.spaxel_av(gc[:, 2], gpa, gext, star_coords[:, 2], spa, nseg)
        return do.extinguish(ax, av)

    p = w.particles
    return oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                              w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux,
                              w.ssp.wavelength, w.dist_z, w.wave_t, psf_size=w.psf_size,
                              psf_sigma=w.psf_sigma, lsf_sigma=w.lsf_sigma,
                              wave_res=w.wave_res, rotation=(hmr, 0.0, 0.0, 0.0),
                              transmission=transmission)


def _dusty_data(w, g, gvel):
    from rubix_gb300.core import GasData
    from test_gpu_steps import _data

    d = _data(w)
    d.gas = GasData(coords=g.coords.copy(), velocity=gvel.copy(), mass=g.mass.copy(),
                    metals=g.metals.copy())
    return d


def test_dusty_pipeline_matches_oracle():
    from rubix_gb300.core import RubixPipeline

    w = workload("small")
    g, gvel = _gas(4000)
    ref = _oracle_dusty(w, g, gvel)
    out = RubixPipeline(_dust_cfg(w, "small_dust"), _dusty_data(w, g, gvel)).run()
    cube = out.stars.datacube.cpu().numpy()
    assert_cube_close(cube, ref["final"], what="calc_dusty_ifu cube")
    # the dust really acts: the dusty cube is dimmer than the dust-free one
    from test_gpu_steps import _oracle_pipeline

    clean = _oracle_pipeline(w)["final"]
    assert cube.sum() < 0.995 * clean.sum()


def test_dusty_materialised_matches_fused():
    """calculate_extinction on materialised spectra (rows kernel) and the segment sum
    equal the fused dusty kernel."""
    import torch

    from rubix_gb300 import core

    w = workload("small", n=600)
    cfg = _dust_cfg(w, "small600_dust")
    g, gvel = _gas(800, seed=6)
    d = _dusty_data(w, g, gvel)
    for step in (core.get_filter_particles, core.get_spaxel_assignment, core.get_reshape_data,
                 core.get_calculate_spectra, core.get_scale_spectrum_by_mass,
                 core.get_doppler_shift_and_resampling):
        d = step(cfg)(d)
    lazy_spec = d.stars.spectra
    res = torch.as_tensor(np.asarray(lazy_spec)).cuda()
    ext = core.get_extinction(cfg)
    d = ext(d)
    fused = core.get_calculate_datacube(cfg)(d).stars.datacube.cpu().numpy()
    mat_rows = np.asarray(d.stars.spectra)  # lazy with dust, materialised on request
    d.stars.spectra = res.clone()
    d = ext(d)
    assert isinstance(d.stars.spectra, torch.Tensor)
    np.testing.assert_allclose(d.stars.spectra.cpu().numpy(), mat_rows, rtol=2e-6,
                               atol=1e-6 * float(np.abs(mat_rows).max()))
    mat = core.get_calculate_datacube(cfg)(d).stars.datacube.cpu().numpy()
    assert_cube_close(mat, fused.astype(np.float64), what="materialised dusty cube")


def test_dusty_gordon23():
    """The Gordon23 curve through the fused kernel (direct ops call)."""
    import torch

    from rubix_gb300 import dust, ops

    w = workload("small", n=3000)
    p = w.particles
    rng = np.random.Generator(np.random.PCG64(11))
    av = rng.uniform(0.0, 3.0, p.n).astype(np.float32)
    e = dust.extinction_exponent(w.wave_t, "Gordon23", 3.1)
    idx = oracle.square_spaxel_assignment(p.coords, w.edges)
    nseg = w.sbin * w.sbin
    perm, offs = ops.spaxel_sort(to_dev(idx, torch.int32), nseg)
    cube = ops.cube_forward(to_dev(w.ssp.flux), to_dev(w.ssp.metallicity), to_dev(w.ssp.age),
                            to_dev(w.wave_z), to_dev(w.wave_t), to_dev(p.mass),
                            to_dev(p.metallicity), to_dev(p.age), to_dev(p.velocity), 2, perm,
                            offs, nseg, dust_av=to_dev(av), dust_exponent=to_dev(e))
    wave_um = (np.asarray(w.wave_t, np.float32) / np.float32(1e4)).astype(np.float64)
    T = do.extinguish(do.gordon23(wave_um, 3.1), av)
    ref = oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                             w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux,
                             w.ssp.wavelength, w.dist_z, w.wave_t, apply_filter=False,
                             transmission=T)["cube"]
    assert_cube_close(cube.cpu().numpy().reshape(ref.shape), ref, what="Gordon23 dusty cube")


def test_renderer_dust_matches_oracle():
    """IFURenderer.render(gas=...) (the bench's path) against the oracle, no rotation."""
    from rubix_gb300 import synth
    from rubix_gb300 import telescope as tel
    from rubix_gb300.api import IFURenderer

    w = workload("small", n=4000)
    g, _ = _gas(3000, seed=8)
    rnd = IFURenderer.from_workload(w, device="cuda", dust={"extinction_model": "Gordon23",
                                                            "Rv": 2.7})
    p = w.particles
    st = rnd.render(p.coords, p.velocity, p.mass, p.metallicity, p.age,
                    gas=(g.coords, g.mass, g.metals))
    _, size = tel.spatial_bin_edges(synth.WORKLOADS["small"]["fov"], w.sbin, w.dist_z)
    area = float(np.float32(size) ** 2)
    _, gf = oracle.filter_particles(g.coords, w.edges, mass=g.mass)
    gext = do.gas_extinction(gf["mass"], g.metals, area)
    gpa = oracle.square_spaxel_assignment(g.coords, w.edges)
    spa = oracle.square_spaxel_assignment(p.coords, w.edges)
    av = do.spaxel_av(g.coords[:, 2], gpa, gext, p.coords[:, 2], spa, w.sbin * w.sbin)
    wave_um = (np.asarray(w.wave_t, np.float32) / np.float32(1e4)).astype(np.float64)
    T = do.extinguish(do.gordon23(wave_um, 2.7), av)
    ref = oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                             w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux,
                             w.ssp.wavelength, w.dist_z, w.wave_t, psf_size=w.psf_size,
                             psf_sigma=w.psf_sigma, lsf_sigma=w.lsf_sigma,
                             wave_res=w.wave_res, transmission=T)
    assert_cube_close(st.final.cpu().numpy(), ref["final"], what="renderer dusty cube")


def test_dusty_particle_gradients():
    """rubix_cube_bwd_dust against the oracle's analytic gradients with the cube adjoint
    seen through each particle's transmission (A_V held fixed)."""
    import torch

    from rubix_gb300 import dust, ops
    from test_gpu_grad import _compare

    w = workload("small", n=2000)
    p = w.particles
    L = w.wave_t.size
    nseg = w.sbin * w.sbin
    rng = np.random.default_rng(21)
    av = rng.uniform(0.0, 2.5, p.n).astype(np.float32)
    e = dust.extinction_exponent(w.wave_t, "Cardelli89", 3.1)
    idx = oracle.square_spaxel_assignment(p.coords, w.edges).astype(np.int64)
    perm, offs = ops.spaxel_sort(to_dev(idx, torch.int32), nseg)
    adj = rng.standard_normal((nseg, L)).astype(np.float32)
    ssp = [to_dev(x) for x in (w.ssp.flux, w.ssp.metallicity, w.ssp.age, w.wave_z)]
    got = ops.cube_backward(*ssp, to_dev(w.wave_t), to_dev(p.mass), to_dev(p.metallicity),
                            to_dev(p.age), to_dev(p.velocity), 2, perm, offs, nseg,
                            to_dev(adj), dust_av=to_dev(av), dust_exponent=to_dev(e))
    wave_um = (np.asarray(w.wave_t, np.float32) / np.float32(1e4)).astype(np.float64)
    T = do.extinguish(do.cardelli89(wave_um, 3.1), av).astype(np.float64)
    rows = adj.astype(np.float64)[idx] * T
    want = oracle.particle_grads(p.mass, p.metallicity, p.age, p.velocity[:, 2],
                                 w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z, w.wave_t,
                                 rows)
    for name, g, wv in zip(("mass", "metallicity", "age", "v_los"), got, want):
        _compare(f"dusty dL/d{name}", g.cpu().numpy(), wv)


def test_dusty_autograd_render():
    """render_cube(..., gas=...) forward equals the renderer's dusty cube; its mass
    gradient is the transmission-weighted one (cube linear in mass)."""
    import torch

    from rubix_gb300.api import IFURenderer
    from rubix_gb300.autograd import render_cube

    w = workload("small", n=1500)
    p = w.particles
    g, _ = _gas(1500, seed=12)
    r = IFURenderer.from_workload(w, device="cuda", dust={"extinction_model": "Cardelli89"})
    gas = tuple(to_dev(a) for a in (g.coords, g.mass, g.metals))
    mass = to_dev(p.mass).requires_grad_()
    cube = render_cube(r, to_dev(p.coords), to_dev(p.velocity), mass, to_dev(p.metallicity),
                       to_dev(p.age), w.psf_sigma, w.lsf_sigma, w.psf_size, w.wave_res, gas=gas)
    ref = r.render(p.coords, p.velocity, p.mass, p.metallicity, p.age, gas=gas).final
    assert_cube_close(cube.detach().cpu().numpy(), ref.cpu().numpy().astype(np.float64),
                      what="autograd dusty forward")
    cube.sum().backward()
    gm = mass.grad.cpu().numpy()
    # linearity in mass: sum_p m_p dL/dm_p = L for L = sum(cube)
    total = float(cube.detach().double().sum())
    assert abs(float(np.dot(gm.astype(np.float64), p.mass.astype(np.float64))) - total) <= \
        1e-4 * abs(total)
