"""Host-side logic: telescope grids, bin edges, taps, synthetic data, step-factory
validation and pipeline wiring (no GPU needed)."""

import numpy as np
import pytest

import oracle
from rubix_gb300 import synth
from rubix_gb300 import telescope as tel


def test_muse_grids():
    t = tel.create_telescope("MUSE")
    assert t.sbin == 25
    assert t.wave_seq.dtype == np.float32 and t.wave_seq.size == 3721
    assert np.array_equal(t.wave_seq, oracle.calculate_wave_seq([4700.15, 9351.4], 1.25))
    with pytest.raises(ValueError, match="Telescope NOPE not found in config"):
        tel.create_telescope("NOPE")


@pytest.mark.parametrize("fov,z", [(5.0, 0.1), (30.0, 0.1), (60.0, 0.05), (3.0, 0.3)])
def test_spatial_bin_edges_match_oracle(fov, z):
    sbin = int(np.floor(fov / 0.2))
    got, size = tel.spatial_bin_edges(fov, sbin, z)
    want, wsize = oracle.calculate_spatial_bin_edges(fov, sbin, oracle.angular_scale(z))
    assert got.dtype == np.float32
    assert np.array_equal(got, want) and size == wsize
    assert len(got) - 1 in (sbin, sbin + 1)


@pytest.mark.parametrize("m,sigma", [(3, 2.0), (11, 1.0), (15, 1.5), (4, 0.8)])
def test_psf_taps_are_exact_factors(m, sigma):
    g = tel.gaussian_taps_1d(m, sigma)
    np.testing.assert_allclose(np.outer(g, g), oracle.gaussian_kernel_2d(m, m, sigma),
                               rtol=1e-14, atol=1e-17)


def test_lsf_taps_match_oracle_and_length_check():
    from rubix_gb300.core.lsf import lsf_taps_checked

    np.testing.assert_allclose(tel.lsf_taps(1.2, 1.25), oracle.lsf_kernel(1.2, 1.25), rtol=1e-15)
    assert lsf_taps_checked(1.2, 1.25).size == 25
    bad = [r for r in (0.1, 0.3, 0.7, 1.1, 6.38, 114.36) if tel.lsf_taps(1.0, r).size != 25]
    for r in bad:
        with pytest.raises(ValueError, match="does not preserve"):
            lsf_taps_checked(1.0, r)


def test_synthetic_workload_is_deterministic():
    a = synth.make_workload("small", n=500)
    b = synth.make_workload("small", n=500)
    for k in ("coords", "velocity", "mass", "metallicity", "age"):
        assert np.array_equal(getattr(a.particles, k), getattr(b.particles, k))
    assert np.array_equal(a.ssp.flux, b.ssp.flux)
    assert (a.ssp.flux > 0).all()
    assert a.particles.n == 500 + 14  # appended edge cases


PSF_ERRORS = [  # rubix tests/test_core_psf.py:6-43
    ({"telescope": {}}, "PSF configuration not found in telescope configuration"),
    ({"telescope": {"psf": {}}}, "PSF name not found in telescope configuration"),
    ({"telescope": {"psf": {"name": "gaussian"}}}, "PSF size not found in telescope configuration"),
    ({"telescope": {"psf": {"name": "gaussian", "size": 5}}},
     "PSF sigma not found in telescope configuration"),
    ({"telescope": {"psf": {"name": "unknown", "size": 5, "sigma": 1.5}}},
     "Unknown PSF kernel name: unknown"),
]


@pytest.mark.parametrize("config,message", PSF_ERRORS)
def test_convolve_psf_config_errors(config, message):
    from rubix_gb300.core import get_convolve_psf

    with pytest.raises(ValueError) as e:
        get_convolve_psf(config)
    assert str(e.value) == message


def test_convolve_lsf_config_errors():  # rubix tests/test_core_lsf.py:7-18
    from rubix_gb300.core import get_convolve_lsf

    with pytest.raises(ValueError, match="LSF configuration not found"):
        get_convolve_lsf({"telescope": {}})
    with pytest.raises(ValueError, match="LSF sigma size not found"):
        get_convolve_lsf({"telescope": {"lsf": {}}})


def test_ssp_config_errors_and_method():
    from rubix_gb300.core import get_calculate_spectra, get_ssp

    with pytest.raises(ValueError, match="does not contain 'ssp' field"):
        get_ssp({})
    with pytest.raises(ValueError, match="does not contain 'template' field"):
        get_ssp({"ssp": {}})
    with pytest.raises(ValueError, match="does not contain 'name' field"):
        get_ssp({"ssp": {"template": {}}})
    with pytest.raises(ValueError, match="not available"):
        get_ssp({"ssp": {"template": {"name": "NoSuchTemplate"}}})
    with pytest.raises(FileNotFoundError, match="BC03lr.h5 not found"):
        get_ssp({"ssp": {"template": {"name": "BruzualCharlot2003"}}})
    cfg = {"ssp": {"template": {"name": "synthetic", "n_age": 4, "n_met": 3, "n_wave": 50}}}
    with pytest.raises(ValueError, match="method='linear'"):
        get_calculate_spectra(cfg)  # rubix's default method is "cubic"
    cfg["ssp"]["method"] = "linear"
    assert get_calculate_spectra(cfg).__name__ == "calculate_spectra"


def test_step_names_are_rubix_registry_keys():
    from rubix_gb300 import core

    cfg = {"telescope": {"name": "MUSE", "psf": {"name": "gaussian", "size": 5, "sigma": 0.6},
                         "lsf": {"sigma": 0.6}},
           "galaxy": {"dist_z": 0.1}, "cosmology": {"name": "PLANCK15"},
           "ssp": {"template": {"name": "synthetic", "n_age": 4, "n_met": 3, "n_wave": 50},
                   "method": "linear"}}
    names = [core.get_calculate_spectra(cfg).__name__, core.get_scale_spectrum_by_mass(cfg).__name__,
             core.get_doppler_shift_and_resampling(cfg).__name__,
             core.get_calculate_datacube(cfg).__name__, core.get_convolve_psf(cfg).__name__,
             core.get_convolve_lsf(cfg).__name__, core.get_spaxel_assignment(cfg).__name__,
             core.get_filter_particles(cfg).__name__, core.get_reshape_data(cfg).__name__]
    assert names == ["calculate_spectra", "scale_spectrum_by_mass", "doppler_shift_and_resampling",
                     "calculate_datacube", "convolve_psf", "convolve_lsf", "spaxel_assignment",
                     "filter_particles", "reshape_data"]


def test_linear_pipeline_order_and_validation():
    from rubix_gb300.core.config import get_pipeline_config
    from rubix_gb300.pipeline import LinearTransformerPipeline

    cfg = get_pipeline_config("calc_ifu")
    order = list(cfg["Transformers"])

    def make(name):
        def f(trace):
            return trace + [name]
        f.__name__ = name
        return f

    funcs = [make(n) for n in reversed(order)]  # registration order does not matter
    p = LinearTransformerPipeline(cfg, funcs)
    assert p.apply([]) == order
    with pytest.raises(ValueError, match="already present"):
        LinearTransformerPipeline(cfg, funcs + [make(order[0])])
    bad = get_pipeline_config("calc_ifu")
    bad["Transformers"]["filter_particles"]["depends_on"] = None
    with pytest.raises(ValueError, match="only be one starting point"):
        LinearTransformerPipeline(bad, funcs)
    bad = get_pipeline_config("calc_ifu")
    bad["Transformers"]["convolve_lsf"]["depends_on"] = "convolve_psf"
    bad["Transformers"]["apply_noise"]["depends_on"] = "convolve_psf"
    with pytest.raises(ValueError, match="branching is not allowed"):
        LinearTransformerPipeline(bad, funcs)
    with pytest.raises(ValueError, match="Pipeline nope not found"):
        get_pipeline_config("nope")


def test_renderer_and_pipeline_need_cuda_and_data():
    from rubix_gb300.api import IFURenderer
    from rubix_gb300.core import RubixPipeline

    w = synth.make_workload("small", n=10)
    with pytest.raises(ValueError, match="CUDA"):
        IFURenderer.from_workload(w, device="cpu")
    cfg = {"pipeline": {"name": "calc_ifu"}, "telescope": {"name": "MUSE"},
           "ssp": {"template": {"name": "synthetic"}, "method": "linear"}}
    with pytest.raises(ValueError, match="no particle data"):
        RubixPipeline(cfg).run()
    with pytest.raises(FileNotFoundError, match="rubix_galaxy.h5 not found"):
        RubixPipeline(dict(cfg, output_path="/nonexistent_dir")).run()


def test_lsf_fusable_order():
    from rubix_gb300.core.lsf import lsf_fusable

    calc_ifu = ["rotate_galaxy", "filter_particles", "spaxel_assignment", "calculate_spectra",
                "reshape_data", "scale_spectrum_by_mass", "doppler_shift_and_resampling",
                "calculate_datacube", "convolve_psf", "convolve_lsf", "apply_noise"]
    assert lsf_fusable(calc_ifu)
    assert lsf_fusable(["calculate_datacube", "convolve_lsf", "convolve_psf"])
    # a step between them that is not the PSF (noise does not commute with the LSF)
    assert not lsf_fusable(["calculate_datacube", "apply_noise", "convolve_lsf"])
    assert not lsf_fusable(["convolve_lsf", "calculate_datacube"])
    assert not lsf_fusable(["calculate_datacube", "convolve_psf"])


def test_frame_fusion_order():
    from rubix_gb300.core.telescope import frame_fusion

    h = frame_fusion(["rotate_galaxy", "filter_particles", "spaxel_assignment", "x"])
    assert h is not None and h.rotation
    h = frame_fusion(["filter_particles", "spaxel_assignment"])
    assert h is not None and not h.rotation
    # rotation not directly before the filter: only filter + assignment are joined
    h = frame_fusion(["rotate_galaxy", "x", "filter_particles", "spaxel_assignment"])
    assert h is not None and not h.rotation
    assert frame_fusion(["spaxel_assignment", "filter_particles"]) is None
    assert frame_fusion(["filter_particles", "x", "spaxel_assignment"]) is None


def test_device_constants_and_read_only_arrays():
    import torch

    from rubix_gb300 import telescope as tel
    from rubix_gb300.core.data import device_constant, to_device

    cpu = torch.device("cpu")
    a = np.linspace(0.0, 1.0, 7).astype(np.float32)
    t1 = device_constant(a, cpu)
    t2 = device_constant(a.copy(), cpu)  # same contents: the same uploaded tensor
    assert t1 is t2 and torch.equal(t1, torch.from_numpy(a))
    assert device_constant(a + 1, cpu) is not t1
    # the telescope grids are shared read-only arrays; uploads copy them
    t = tel.create_telescope("MUSE")
    assert not t.wave_seq.flags.writeable
    assert tel.create_telescope("MUSE").wave_seq is t.wave_seq
    u = to_device(t.wave_seq, cpu)
    u[0] = -1.0  # a copy: the shared grid is untouched
    assert t.wave_seq[0] != -1.0
    # a bool mask read as uint8 shares its storage (no copy)
    m = torch.tensor([True, False, True])
    assert to_device(m, cpu, torch.uint8).tolist() == [1, 0, 1]


def test_rubix_default_dtypes_of_loaded_arrays():
    from rubix_gb300.core.galaxy_file import _jax_default

    assert _jax_default(np.zeros(3)).dtype == np.float32
    assert _jax_default(np.zeros(3, np.int64)).dtype == np.int32
    assert _jax_default(np.zeros(3, np.float32)).dtype == np.float32
    assert _jax_default(np.zeros(3, bool)).dtype == bool
