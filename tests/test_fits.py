"""FITS I/O: card format and block structure of the writer, round trips, gzip
reading, rubix's store_fits layout and headers, and the pyPipe3D SSP-template loader on
a file in that format (CPU); the GPU layout kernel against the NumPy layout (gpu)."""

import gzip
import os

import numpy as np
import pytest

from rubix_gb300 import fits


def test_card_format():
    c = fits.format_card("SIMPLE", True, "conforms to FITS standard")
    assert len(c) == 80 and c[:10] == "SIMPLE  = " and c[29] == "T"
    c = fits.format_card("BITPIX", -32)
    assert c[10:30] == f"{-32:>20}"
    c = fits.format_card("PIPELINE", "calc_ifu")
    assert c[10:20] == "'calc_ifu'"
    c = fits.format_card("OBJECT", "a'b")
    assert c[10:20] == "'a''b    '"
    c = fits.format_card("X", 1e-30)
    assert float(c[10:30]) == 1e-30 and "." in c[10:30]
    with pytest.raises(ValueError):
        fits.format_card("TOOLONGKEY", 1)


def test_round_trip_and_blocks(tmp_path):
    rng = np.random.default_rng(0)
    a = rng.standard_normal((5, 4, 3)).astype(np.float32)
    b = rng.integers(-1000, 1000, (7, 2)).astype(np.int16)
    h0 = fits.Header([("PIPELINE", "calc_ifu", "name"), ("DIST_Z", 0.1, ""),
                      ("FLAG", False, ""), ("N", 42, "")])
    h1 = fits.Header([("EXTNAME", "DATA", "")])
    p = tmp_path / "t.fits"
    fits.write_fits(str(p), [fits.HDU(h0), fits.HDU(h1, a), fits.HDU(fits.Header(), b)])
    raw = p.read_bytes()
    assert len(raw) % fits.BLOCK == 0
    assert raw[:80].decode().startswith("SIMPLE  =                    T")
    hdus = fits.read_fits(str(p))
    assert len(hdus) == 3
    assert hdus[0].header["PIPELINE"] == "calc_ifu" and hdus[0].header["DIST_Z"] == 0.1
    assert hdus[0].header["FLAG"] is False and hdus[0].header["N"] == 42
    assert hdus[0].header["EXTEND"] is True and hdus[0].data is None
    assert hdus[1].header["XTENSION"] == "IMAGE" and hdus[1].header["NAXIS1"] == 3
    assert hdus[1].header["NAXIS3"] == 5 and hdus[1].header["BITPIX"] == -32
    np.testing.assert_array_equal(hdus[1].data, a)
    np.testing.assert_array_equal(hdus[2].data, b)
    # big-endian on disk
    off = 2 * fits.BLOCK
    assert np.frombuffer(raw, ">f4", count=1, offset=off)[0] == a.reshape(-1)[0]
    # gzip and BSCALE/BZERO
    gz = tmp_path / "t.fits.gz"
    gz.write_bytes(gzip.compress(raw))
    np.testing.assert_array_equal(fits.read_fits(str(gz))[1].data, a)
    hs = fits.Header([("BSCALE", 0.5, ""), ("BZERO", 10.0, "")])
    fits.write_fits(str(p), [fits.HDU(hs, b)])
    np.testing.assert_allclose(fits.read_fits(str(p))[0].data, b * 0.5 + 10.0)


def _cfg():
    return {"pipeline": {"name": "calc_ifu"}, "galaxy": {"dist_z": 0.1,
                                                         "rotation": {"type": "face-on"}},
            "simulation": {"name": "IllustrisTNG"},
            "data": {"load_galaxy_args": {"id": 14}, "args": {"snapshot": 99},
                     "subset": {"use_subset": True}},
            "ssp": {"template": {"name": "BruzualCharlot2003"}},
            "telescope": {"name": "MUSE", "psf": {"name": "gaussian", "size": 5, "sigma": 0.6},
                          "lsf": {"sigma": 0.5},
                          "noise": {"signal_to_noise": 1, "noise_distribution": "normal"}},
            "cosmology": {"name": "PLANCK15"}}


def test_store_and_load_fits_numpy(tmp_path):
    from rubix_gb300.core import RubixData
    from rubix_gb300.core.fits import load_fits, store_fits

    rng = np.random.default_rng(1)
    cube = rng.standard_normal((6, 5, 40)).astype(np.float32)
    d = RubixData()
    d.stars.datacube = cube
    out = store_fits(_cfg(), d, str(tmp_path) + "/out/")
    assert out.endswith("out/IllustrisTNG_id14_snap99_stars_subsetTrue.fits")
    fc = load_fits(out)
    assert fc.data.shape == (40, 5, 6)
    np.testing.assert_array_equal(fc.datacube, cube)
    np.testing.assert_array_equal(fc.data, cube.T)
    h, h0 = fc.header, fc.primary_header
    assert h["EXTNAME"] == "DATA" and h["CTYPE3"] == "AWAV" and h["CUNIT3"] == "Angstrom"
    assert h["CRPIX1"] == 2.5 and h["CRPIX2"] == 2.0 and h["CD3_3"] == 1.25
    assert h["CD1_1"] == pytest.approx(0.2 / 3600) and h["CRVAL3"] == 4700.15
    assert h["OBJECT"] == "IllustrisTNG 14" and h["BUNIT"] == "erg/(s*cm^2*A)"
    assert h0["PIPELINE"] == "calc_ifu" and h0["GALAXYID"] == 14 and h0["SNAPSHOT"] == 99
    assert h0["S_TO_N"] == 1 and h0["PSF_SIZE"] == 5 and h0["COSMO"] == "PLANCK15"
    np.testing.assert_allclose(fc.wave[:3], 4700.15 + 1.25 * np.arange(3))


def _write_pypipe3d(path, ages_tok, z_tok, n_wave, crval=3000.0, cdelt=2.5, crpix=1.0,
                    gz=False):
    """A template in the pyPipe3D layout: one model per row, metallicity major."""
    rng = np.random.default_rng(3)
    n_models = len(ages_tok) * len(z_tok)
    data = rng.uniform(0.5, 2.0, (n_models, n_wave)).astype(np.float32)
    cards = [("CRVAL1", crval, ""), ("CDELT1", cdelt, ""), ("CRPIX1", crpix, "")]
    norms = []
    i = 0
    for z in z_tok:
        for a in ages_tok:
            norm = 0.0 if i == 1 else float(rng.uniform(0.1, 3.0))
            norms.append(norm)
            cards += [(f"NAME{i}", f"spec_ssp_{a}_{z}.spec", ""), (f"NORM{i}", norm, "")]
            i += 1
    p = str(path)
    fits.write_fits(p, [fits.HDU(fits.Header(cards), data)])
    if gz:
        with open(p, "rb") as f:
            raw = f.read()
        with open(p + ".gz", "wb") as f:
            f.write(gzip.compress(raw))
        p += ".gz"
    return p, data, np.array(norms, np.float32)


def test_pypipe3d_loader(tmp_path, monkeypatch):
    from rubix_gb300.core import ssp

    ages_tok = ["0.0631Gyr", "500Myr", "2.0Gyr", "10.0"]
    z_tok = ["z0190", "z0040"]
    p, data, norms = _write_pypipe3d(tmp_path / "m.fits", ages_tok, z_tok, 50, gz=True)
    g = ssp.load_pypipe3d(p)
    np.testing.assert_allclose(g.age, [0.0631, 0.5, 2.0, 10.0], rtol=1e-6)
    np.testing.assert_allclose(g.metallicity, [0.004, 0.019], rtol=1e-6)
    np.testing.assert_allclose(g.wavelength, 3000.0 + 2.5 * np.arange(50))
    m2l = np.float32(1) / np.where(norms != 0, norms, np.float32(1))
    np.testing.assert_allclose(g.flux, (data / m2l[:, None]).reshape(2, 4, 50), rtol=1e-6)
    # the named template from the template directory
    monkeypatch.setenv("RUBIX_GB300_TEMPLATE_PATH", str(tmp_path))
    os.replace(p, tmp_path / "MaStar_CB19.slog_1_5.fits.gz")
    g2 = ssp.get_ssp_template("Mastar_CB19_SLOG_1_5")
    np.testing.assert_array_equal(g2.flux, g.flux)
    with pytest.raises(FileNotFoundError, match="BC03lr.h5 not found"):
        ssp.get_ssp_template("BruzualCharlot2003")


def test_unit_conversion():
    from rubix_gb300.core import ssp

    np.testing.assert_allclose(ssp.convert_units([500.0], "age", "Myr"), [0.5])
    np.testing.assert_allclose(ssp.convert_units([400.0], "wavelength", "nm"), [4000.0])
    with pytest.raises(ValueError, match="cannot convert"):
        ssp.convert_units([1.0], "flux", "Jy")


@pytest.mark.gpu
def test_fits_layout_kernel_matches_numpy(tmp_path):
    import torch

    from rubix_gb300.core import RubixData
    from rubix_gb300.core.fits import cube_fits_bytes, store_fits

    rng = np.random.default_rng(2)
    for shape in ((25, 25, 3721), (33, 7, 45), (1, 1, 1), (70, 40, 33), (65, 3, 129)):
        cube = rng.standard_normal(shape).astype(np.float32)
        got = cube_fits_bytes(torch.from_numpy(cube).cuda())
        assert got == cube_fits_bytes(cube), shape
    # a cube with a padded spaxel stride (the renderer's accumulate stage)
    cube = rng.standard_normal((20, 21, 47)).astype(np.float32)
    padded = torch.zeros((20, 21, 48), device="cuda")
    padded[:, :, :47] = torch.from_numpy(cube).cuda()
    assert cube_fits_bytes(padded[:, :, :47]) == cube_fits_bytes(cube)
    cube = rng.standard_normal((30, 30, 300)).astype(np.float32)
    d = RubixData()
    d.stars.datacube = torch.from_numpy(cube).cuda()
    a = store_fits(_cfg(), d, str(tmp_path) + "/gpu/")
    d.stars.datacube = cube
    b = store_fits(_cfg(), d, str(tmp_path) + "/cpu/")
    assert open(a, "rb").read() == open(b, "rb").read()
