"""The rubix-compatible step API on the GPU against the oracle, step by step and as a
whole pipeline, plus rubix's known-answer cases run through the CUDA kernels."""

import numpy as np
import pytest

import oracle
from helpers import assert_cube_close, oracle_stages, to_dev, workload

pytestmark = pytest.mark.gpu


def _config(w, name="small_test_ssp"):
    from rubix_gb300.core import register_ssp_template
    from rubix_gb300.core.ssp import SSPGrid

    register_ssp_template(name, SSPGrid(age=w.ssp.age, metallicity=w.ssp.metallicity,
                                        wavelength=w.ssp.wavelength, flux=w.ssp.flux))
    return {
        "pipeline": {"name": "calc_ifu"},
        "logger": {"log_level": "WARNING"},
        "data": {"args": {"particle_type": ["stars"]}},
        "telescope": {"name": "MUSE", "psf": {"name": "gaussian", "size": w.psf_size,
                                              "sigma": w.psf_sigma},
                      "lsf": {"sigma": w.lsf_sigma},
                      # S/N so large that the noise cannot change a float32 value: the
                      # parity comparison is pre-noise
                      "noise": {"signal_to_noise": 1e30, "noise_distribution": "normal"}},
        "cosmology": {"name": "PLANCK15"},
        "galaxy": {"dist_z": w.dist_z, "rotation": {"type": "face-on"}},
        "ssp": {"template": {"name": name}, "method": "linear"},
    }


HALFMASS_RADIUS = 5.0  # kpc, of the synthetic exponential disk (R_d = 3 kpc)


def _data(w):
    from rubix_gb300.core import Galaxy, RubixData, StarsData

    p = w.particles
    return RubixData(galaxy=Galaxy(halfmassrad_stars=HALFMASS_RADIUS),
                     stars=StarsData(coords=p.coords.copy(), velocity=p.velocity.copy(),
                                     mass=p.mass.copy(), metallicity=p.metallicity.copy(),
                                     age=p.age.copy()))


def _oracle_pipeline(w):
    """The oracle's calc_ifu chain with the face-on rotation of the step configs."""
    p = w.particles
    return oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                              w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux,
                              w.ssp.wavelength, w.dist_z, w.wave_t, psf_size=w.psf_size,
                              psf_sigma=w.psf_sigma, lsf_sigma=w.lsf_sigma, wave_res=w.wave_res,
                              rotation=(HALFMASS_RADIUS, 0.0, 0.0, 0.0))


@pytest.mark.parametrize("fuse_lsf", [True, False])
def test_rubix_pipeline_matches_oracle(fuse_lsf):
    """The LSF in the accumulate epilogue (default) or as its own step: both match."""
    from rubix_gb300.core import RubixPipeline

    w = workload("small")
    ref = _oracle_pipeline(w)
    pipe = RubixPipeline(_config(w), _data(w), fuse_lsf=fuse_lsf)
    out = pipe.run()
    cube = out.stars.datacube.cpu().numpy()
    assert cube.shape == (25, 25, 3721)
    assert_cube_close(cube, ref["final"], what="RubixPipeline cube")
    assert np.array_equal(out.stars.pixel_assignment.cpu().numpy().reshape(-1),
                          ref["pixel_assignment"])
    assert np.array_equal(out.stars.mask.cpu().numpy().reshape(-1), ref["mask"])


def test_rubix_pipeline_noise():
    """calc_ifu with S/N = 20: the noise step changes the cube by cube * sigma * z."""
    from rubix_gb300.core import RubixPipeline

    w = workload("small")
    cfg = _config(w)
    ref = _oracle_pipeline(w)["final"]
    cfg["telescope"]["noise"] = {"signal_to_noise": 20, "noise_distribution": "normal"}
    out = RubixPipeline(cfg, _data(w)).run().stars.datacube.cpu().numpy().astype(np.float64)
    sig, med = oracle.noise_sigma(ref, 20.0)
    if med == 0.0:  # an empty spaxel disables rubix's noise (NaN median)
        assert_cube_close(out, ref, what="noise-free cube")
        return
    ok = ref > 1e-3 * np.abs(ref).max()
    z = ((out - ref) / (ref * sig[:, :, None]))[ok]
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01


def test_steps_one_by_one_materialised():
    import torch

    from rubix_gb300 import core

    w = workload("small", n=600)
    cfg = _config(w, "small600")
    p = w.particles
    d = _data(w)
    d = core.get_filter_particles(cfg)(d)
    mask, f = oracle.filter_particles(p.coords, w.edges, mass=p.mass, metallicity=p.metallicity,
                                      age=p.age)
    assert np.array_equal(d.stars.mass.cpu().numpy().reshape(-1), f["mass"])
    assert np.array_equal(d.stars.age.cpu().numpy().reshape(-1), f["age"])
    d = core.get_spaxel_assignment(cfg)(d)
    d = core.get_reshape_data(cfg)(d)
    assert d.stars.mass.shape == (1, p.n) and d.stars.coords.shape == (1, p.n, 3)
    d = core.get_calculate_spectra(cfg)(d)
    lookup = oracle.interp2d_linear(f["metallicity"], f["age"], w.ssp.metallicity, w.ssp.age,
                                    w.ssp.flux)
    got = np.asarray(d.stars.spectra)
    assert got.shape == (1, p.n, w.ssp.wavelength.size)
    assert_cube_close(got[0], lookup, what="lookup spectra")
    d = core.get_scale_spectrum_by_mass(cfg)(d)
    assert_cube_close(np.asarray(d.stars.spectra)[0], lookup * f["mass"][:, None],
                      what="mass-scaled spectra")
    d = core.get_doppler_shift_and_resampling(cfg)(d)
    want = oracle.particle_spectra(f["mass"], f["metallicity"], f["age"], p.velocity[:, 2],
                                   w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z, w.wave_t)
    res = np.asarray(d.stars.spectra)
    assert res.shape == (1, p.n, w.wave_t.size)
    assert_cube_close(res[0], want, what="resampled spectra")
    lazy = core.get_calculate_datacube(cfg)(d).stars.datacube.cpu().numpy()
    ref_cube = oracle.calculate_cube(want, oracle.square_spaxel_assignment(p.coords, w.edges),
                                     w.sbin)
    assert_cube_close(lazy, ref_cube, what="lazy datacube")
    # the same step on materialised spectra (segment-sum path)
    d.stars.spectra = torch.as_tensor(res).cuda()
    mat = core.get_calculate_datacube(cfg)(d).stars.datacube.cpu().numpy()
    assert_cube_close(mat, ref_cube, what="datacube from materialised spectra")


def test_doppler_step_on_given_spectra():
    """doppler_shift_and_resampling applied to spectra the caller supplies."""
    import torch

    from rubix_gb300 import core

    w = workload("small", n=300)
    cfg = _config(w, "small300")
    p = w.particles
    rng = np.random.default_rng(4)
    spec = (rng.random((p.n, w.ssp.wavelength.size)) + 0.1).astype(np.float32)
    d = _data(w)
    d.stars.spectra = torch.as_tensor(spec[None]).cuda()
    d = core.get_doppler_shift_and_resampling(cfg)(d)
    lp = oracle.velocity_doppler_shift32(w.wave_z, p.velocity[:, 2])
    want, _ = oracle.resample_spectra(spec, lp, w.wave_t)
    assert_cube_close(d.stars.spectra.cpu().numpy()[0], want, what="resample_rows")


def test_known_answers_on_gpu():
    import torch

    from rubix_gb300 import ops

    # calculate_cube, rubix tests/test_spectra_ifu.py:231-257
    spectra = to_dev(np.array([[100, 200, 300], [400, 500, 600], [700, 800, 900], [1, 2, 3]],
                              dtype=np.float32))
    perm, offs = ops.spaxel_sort(to_dev(np.array([0, 1, 1, 3], dtype=np.int32)), 4)
    cube = ops.segment_sum_rows(spectra, perm, offs, 4).reshape(2, 2, 3).cpu().numpy()
    assert np.array_equal(cube, [[[100, 200, 300], [1100, 1300, 1500]], [[0, 0, 0], [1, 2, 3]]])
    # resample_spectrum, rubix tests/test_spectra_ifu.py:175-228 (zero velocity)
    F = np.array([[1.0, 2.0, 3.0, 4.0, 5.0], [0, 0, 0, 0, 0]], dtype=np.float32)
    lam = np.array([4000.0, 5000.0, 6000.0, 7000.0, 8000.0], dtype=np.float32)
    lt = np.array([4500.0, 5500.0, 6500.0, 7500.0], dtype=np.float32)
    got = ops.resample_rows(to_dev(F), to_dev(lam), to_dev(np.zeros((2, 3), np.float32)), 2,
                            to_dev(lt)).cpu().numpy()
    np.testing.assert_allclose(got[0], oracle.resample_spectrum(F[0], lam, lt), rtol=1e-5)
    assert (got[1] == 0).all() and not np.isnan(got).any()
    # apply_lsf delta, rubix tests/test_telescope_lsf.py:6-60
    from rubix_gb300 import telescope as tel

    sp = np.zeros((3, 100), dtype=np.float32)
    for i, pos in enumerate([20, 50, 75]):
        sp[i, pos] = 1.0
    out = ops.lsf_forward(to_dev(sp), tel.lsf_taps(2.0, 1.0), 12).cpu().numpy()
    x = np.arange(100)
    for i, pos in enumerate([20, 50, 75]):
        g = np.exp(-0.5 * (x - pos) ** 2 / 4.0)
        np.testing.assert_allclose(out[i], g / g.sum(), atol=1e-5)
    # apply_psf with a 3x3 ones kernel, rubix tests/test_telescope_psf.py:21-54
    c = np.zeros((10, 10, 3), dtype=np.float32)
    c[5, 5, :] = 1.0
    o = ops.psf_forward(to_dev(c), np.ones(3)).cpu().numpy()
    want = oracle.apply_psf(c, np.ones((3, 3)))
    np.testing.assert_allclose(o, want, atol=1e-6)
    torch.cuda.synchronize()


def test_host_stream_matches_render():
    """IFURenderer.host_stream (overlapped upload / compute / download over two slots)
    gives every submitted galaxy the cube of a plain render."""
    import torch

    from rubix_gb300.api import IFURenderer

    ws = [workload("small", n=3000 + 500 * k) for k in range(3)]
    rnd = IFURenderer.from_workload(ws[0], device="cuda")
    hs = rnd.host_stream(2)
    outs = []
    for k in range(5):
        p = ws[k % 3].particles
        h = [torch.from_numpy(a).pin_memory() for a in (p.coords, p.velocity, p.mass,
                                                        p.metallicity, p.age)]
        o = torch.empty((ws[0].sbin, ws[0].sbin, ws[0].wave_t.size)).pin_memory()
        hs.submit(*h, out=o)
        outs.append(o)
    hs.synchronize()
    torch.cuda.synchronize()
    for k in range(5):
        p = ws[k % 3].particles
        ref = rnd.render(p.coords, p.velocity, p.mass, p.metallicity, p.age).final.cpu()
        assert torch.equal(outs[k], ref), f"galaxy {k}"


def test_rubix_pipeline_from_galaxy_file(tmp_path):
    """RubixPipeline(config) without data reads <output_path>/rubix_galaxy.h5
    (get_rubix_data: load, centre) and renders the same cube as the same centred arrays
    passed in directly."""
    import torch

    from rubix_gb300.core import (Galaxy, RubixData, RubixPipeline, StarsData,
                                  create_rubix_file)

    w = workload("small")
    p = w.particles
    center = np.array([0.25, -0.5, 0.1])
    v0 = np.array([12.0, -7.0, 30.0])
    create_rubix_file(
        str(tmp_path / "rubix_galaxy.h5"),
        {"stars": {"coords": p.coords + center, "velocity": p.velocity + v0, "mass": p.mass,
                   "metallicity": p.metallicity, "age": p.age}},
        {"center": center, "halfmassrad_stars": np.float64(HALFMASS_RADIUS),
         "redshift": np.float64(0.0)},
        {"simulation": "synthetic"},
        {"galaxy": {"center": "kpc", "halfmassrad_stars": "kpc", "redshift": ""},
         "stars": {"coords": "kpc", "velocity": "km/s", "mass": "Msun", "metallicity": "",
                   "age": "Gyr"}})
    cfg = _config(w)
    cfg["output_path"] = str(tmp_path)
    got = RubixPipeline(cfg).run().stars.datacube
    # the file holds float64; prepare_input gives float32 (rubix's jnp.array) and
    # centres in float32
    coords = (p.coords + center).astype(np.float32)
    vel = (p.velocity + v0).astype(np.float32)
    c32 = center.astype(np.float32)
    near = np.linalg.norm(coords - c32, axis=1) < 10
    direct = RubixData(galaxy=Galaxy(halfmassrad_stars=HALFMASS_RADIUS),
                       stars=StarsData(coords=coords - c32,
                                       velocity=vel - np.median(vel[near], axis=0),
                                       mass=p.mass, metallicity=p.metallicity, age=p.age))
    want = RubixPipeline(cfg, direct).run().stars.datacube
    torch.cuda.synchronize()
    assert torch.equal(got, want)


@pytest.mark.parametrize("n_wave_t", [3721, 256])
def test_render_pads_the_accumulate_stage_for_the_psf(n_wave_t):
    """With a PSF the renderer writes the accumulate stage into rows of L rounded up to a
    multiple of 4 floats (so the PSF stages them by TMA): the stage is a [S, S, L] view
    with that spaxel stride, and the final cube is dense and bit-identical to the PSF of
    a dense copy of the stage (the 4-byte-copy kernel).  A multiple of 4 needs no
    padding."""
    import torch

    from rubix_gb300.api import IFURenderer

    w = workload("small", n=3000, n_wave_t=n_wave_t)
    p = w.particles
    r = IFURenderer.from_workload(w, device="cuda")
    st = r.render(*(to_dev(a) for a in (p.coords, p.velocity, p.mass, p.metallicity, p.age)))
    L = w.wave_t.size
    assert st.cube.shape == (w.sbin, w.sbin, L)
    assert st.cube.stride(1) == (L + 3) // 4 * 4 and st.cube.stride(2) == 1
    assert st.final.is_contiguous()
    dense = st.cube.contiguous()
    again = r.psf(dense)
    torch.cuda.synchronize()
    assert torch.equal(st.final, again)
