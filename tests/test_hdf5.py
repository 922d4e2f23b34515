"""The HDF5 subset (rubix_gb300.hdf5): a file written by libhdf5, round trips through
the writer, the HDF5 SSP templates (BC03 / FSPS layouts, rubix/spectra/ssp/grid.py:
304-335) and rubix's galaxy file (rubix/galaxy/input_handler/base.py:17-73,
rubix/utils.py:160-200, rubix/core/data.py:490-604)."""

import os

import numpy as np
import pytest

from rubix_gb300 import hdf5

SCIPY_H5 = None
try:
    import scipy

    SCIPY_H5 = os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data",
                            "testhdf5_7.4_GLNX86.mat")
except ImportError:
    pass


@pytest.mark.skipif(SCIPY_H5 is None or not os.path.exists(SCIPY_H5),
                    reason="scipy's MATLAB 7.3 test file is not installed")
def test_reads_a_file_written_by_libhdf5():
    """MATLAB 7.3 files are HDF5 (written by libhdf5) after a 512-byte user block:
    superblock 0, symbol-table root group, a contiguous float64 dataset with a string
    attribute."""
    f = hdf5.File(SCIPY_H5)
    assert f.keys() == ["testdouble"]
    ds = f["testdouble"]
    assert ds.shape == (9, 1) and ds.dtype == np.float64
    np.testing.assert_allclose(ds[()][:, 0], np.linspace(0.0, 2 * np.pi, 9), rtol=0, atol=1e-15)
    assert ds.attrs["MATLAB_class"] == "double"


def test_round_trip_groups_datasets_attributes(tmp_path):
    rng = np.random.default_rng(0)
    big = rng.normal(size=(100, 37)).astype(np.float32)
    tree = {
        "meta": {"snapshot": np.int64(99), "name": "TNG50-1"},
        "galaxy": {"center": (np.array([1.0, 2.0, 3.0]), {"unit": "kpc"}),
                   "redshift": (np.float64(0.1), {"unit": ""})},
        "particles": {"stars": {
            "coords": (rng.normal(size=(1000, 3)).astype(np.float32), {"unit": "kpc"}),
            "mass": (rng.uniform(size=1000), {"unit": "Msun"}),
            "ids": np.arange(1000, dtype=np.int64),
            "flags": np.array([True, False, True]),
            "be": np.arange(5, dtype=">f8"),
            "chunked": hdf5.Chunked(big, (32, 16), gzip=6, shuffle=True,
                                    attrs={"unit": "erg"}),
            "chunked_plain": hdf5.Chunked(big[:7], (4, 37), gzip=None),
            "empty": np.zeros((0, 3), np.float32),
        }},
        "__attrs__": {"version": np.int32(3), "labels": np.array(["a", "bc"])},
    }
    tree["many"] = {f"m{i:03d}": np.arange(i) for i in range(100)}  # several symbol nodes
    p = str(tmp_path / "t.h5")
    hdf5.write_file(p, tree)
    f = hdf5.File(p)
    assert sorted(f.keys()) == ["galaxy", "many", "meta", "particles"]
    assert f.attrs["version"] == 3 and list(f.attrs["labels"]) == ["a", "bc"]
    assert f["meta/snapshot"][()] == 99 and f["meta/name"][()] == "TNG50-1"
    assert f["galaxy"]["center"].attrs == {"unit": "kpc"}
    st = f["particles/stars"]
    for name in ("coords", "mass", "ids"):
        a = tree["particles"]["stars"][name]
        a = a[0] if isinstance(a, tuple) else a
        got = st[name][()]
        assert got.dtype == a.dtype and np.array_equal(got, a), name
    assert np.array_equal(st["flags"][()], [1, 0, 1])
    assert np.array_equal(st["be"][()], np.arange(5.0))
    assert np.array_equal(st["chunked"][()], big) and st["chunked"].attrs["unit"] == "erg"
    assert np.array_equal(st["chunked_plain"][:], big[:7])
    assert st["empty"].shape == (0, 3) and st["empty"][()].shape == (0, 3)
    assert len(f["many"].keys()) == 100 and np.array_equal(f["many/m099"][()], np.arange(99))
    assert "particles/stars/mass" in f and "particles/nothing" not in f
    with pytest.raises(KeyError):
        f["galaxy/center/deeper"]


def test_fixed_length_string_attributes(tmp_path):
    p = str(tmp_path / "s.h5")
    hdf5.write_file(p, {"x": (np.arange(3.0), {"unit": "km/s"})}, vlen_strings=False)
    assert hdf5.File(p)["x"].attrs["unit"] == "km/s"


def test_rejects_non_hdf5(tmp_path):
    p = tmp_path / "n.h5"
    p.write_bytes(b"not an hdf5 file" * 64)
    with pytest.raises(hdf5.HDF5Error, match="not an HDF5 file"):
        hdf5.File(str(p))
    with pytest.raises(ValueError, match="reads only"):
        hdf5.File(str(p), "w")


@pytest.mark.parametrize("template", ["BruzualCharlot2003", "FSPS"])
def test_hdf5_ssp_templates(tmp_path, monkeypatch, template):
    """HDF5SSPGrid.from_file: datasets named by the template's fields, 10**x for the
    in_log fields (FSPS age and metallicity), float32 in the internal units."""
    from rubix_gb300.core import ssp

    rng = np.random.default_rng(5)
    age = np.geomspace(0.1, 13.5, 12)
    met = np.geomspace(1e-4, 0.03, 4)
    wave = np.linspace(3000.0, 9000.0, 50)
    flux = rng.uniform(0.5, 2.0, (4, 12, 50))
    in_log = template == "FSPS"
    tree = {"age": np.log10(age) if in_log else age,
            "metallicity": np.log10(met) if in_log else met,
            "wavelength": wave, "flux": flux}
    name = ssp.SSP_TEMPLATES[template]["file_name"]
    hdf5.write_file(str(tmp_path / name), tree)
    monkeypatch.setenv("RUBIX_GB300_TEMPLATE_PATH", str(tmp_path))
    monkeypatch.delitem(ssp._TEMPLATES, template, raising=False)
    grid = ssp.get_ssp({"ssp": {"template": {"name": template}}})
    assert grid.flux.shape == (4, 12, 50) and grid.flux.dtype == np.float32
    np.testing.assert_allclose(grid.age, age.astype(np.float32), rtol=1e-6)
    np.testing.assert_allclose(grid.metallicity, met.astype(np.float32), rtol=1e-6)
    assert np.array_equal(grid.wavelength, wave.astype(np.float32))
    assert np.array_equal(grid.flux, flux.astype(np.float32))
    ssp._TEMPLATES.pop(template, None)


def _galaxy(n_stars=500, n_gas=300, seed=1):
    rng = np.random.default_rng(seed)
    center = np.array([10.0, -5.0, 2.0])
    stars = {"coords": center + rng.normal(0, 3.0, (n_stars, 3)),
             "velocity": rng.normal(50.0, 100.0, (n_stars, 3)),
             "mass": rng.uniform(1e4, 1e6, n_stars), "metallicity": rng.uniform(1e-4, 0.03, n_stars),
             "age": rng.uniform(0.1, 13.0, n_stars)}
    gas = {"coords": center + rng.normal(0, 4.0, (n_gas, 3)),
           "velocity": rng.normal(-20.0, 80.0, (n_gas, 3)), "mass": rng.uniform(1e4, 1e6, n_gas),
           "metals": rng.uniform(0, 0.01, (n_gas, 10))}
    galaxy = {"center": center, "halfmassrad_stars": np.float64(4.5), "redshift": np.float64(0.1)}
    units = {"galaxy": {"center": "kpc", "halfmassrad_stars": "kpc", "redshift": ""},
             "stars": {"coords": "kpc", "velocity": "km/s", "mass": "Msun",
                       "metallicity": "", "age": "Gyr"},
             "gas": {"coords": "kpc", "velocity": "km/s", "mass": "Msun", "metals": ""}}
    return {"stars": stars, "gas": gas}, galaxy, units


def test_rubix_galaxy_file_round_trip(tmp_path):
    from rubix_gb300.core import create_rubix_file, load_galaxy_data

    particles, galaxy, units = _galaxy()
    path = create_rubix_file(str(tmp_path / "rubix_galaxy.h5"), particles, galaxy,
                             {"simulation": "TNG50-1", "snapshot": 99}, units)
    data, got_units = load_galaxy_data(path)
    assert got_units == units
    assert np.array_equal(data["subhalo_center"], galaxy["center"])
    assert data["subhalo_halfmassrad_stars"] == 4.5 and data["redshift"] == 0.1
    for ptype, fields in particles.items():
        for k, v in fields.items():
            assert np.array_equal(data["particle_data"][ptype][k], v), (ptype, k)
    with pytest.raises(FileNotFoundError):
        load_galaxy_data(str(tmp_path / "missing.h5"))


def test_prepare_input_centres_and_subsets(tmp_path):
    from rubix_gb300.core import create_rubix_file, get_rubix_data

    particles, galaxy, units = _galaxy()
    create_rubix_file(str(tmp_path / "rubix_galaxy.h5"), particles, galaxy, {}, units)
    cfg = {"output_path": str(tmp_path), "data": {"args": {"particle_type": ["stars", "gas"]}},
           "logger": {"log_level": "WARNING"}}
    d = get_rubix_data(cfg)
    c = galaxy["center"].astype(np.float32)
    for ptype in ("stars", "gas"):
        comp = getattr(d, ptype)
        src = {k: v.astype(np.float32) for k, v in particles[ptype].items()}
        # float32 as rubix (jnp.array without 64-bit types); alignment.py:52-60: median
        # velocity of the particles within 10 kpc of the centre
        assert comp.coords.dtype == np.float32 and comp.mass.dtype == np.float32
        near = np.linalg.norm(src["coords"] - c, axis=1) < 10
        assert np.array_equal(comp.coords, src["coords"] - c)
        assert np.array_equal(comp.velocity,
                              src["velocity"] - np.median(src["velocity"][near], 0))
        assert comp.coords_unit == "kpc" and comp.mass_unit == "Msun"
    assert d.galaxy.halfmassrad_stars == 4.5 and d.galaxy.center_unit == "kpc"
    # rubix's subset: np.random.seed(42) choice without replacement over the stars
    # (data.py:559-575); for the gas the stars are already cut to the subset size
    cfg["data"]["subset"] = {"use_subset": True, "subset_size": 100}
    s = get_rubix_data(cfg)
    np.random.seed(42)
    idx = np.random.choice(np.arange(500), size=100, replace=False)
    assert np.array_equal(s.stars.mass, particles["stars"]["mass"].astype(np.float32)[idx])
    np.random.seed(42)
    idx = np.random.choice(np.arange(100), size=100, replace=False)
    assert np.array_equal(s.gas.mass, particles["gas"]["mass"].astype(np.float32)[idx])
    # a centre outside the particles is refused (alignment.py:38-49)
    galaxy["center"] = np.array([1e3, 0.0, 0.0])
    create_rubix_file(str(tmp_path / "rubix_galaxy.h5"), particles, galaxy, {}, units)
    with pytest.raises(ValueError, match="Center is not within the bounds"):
        get_rubix_data(dict(cfg, data={"args": {"particle_type": ["stars"]}}))


def _ohdr(msgs):
    """A version-2 object header ("OHDR", no times, 4-byte chunk size, a zero
    checksum: the reader does not verify checksums) holding (type, body) messages."""
    import struct

    body = b"".join(struct.pack("<BHB", t, len(d), 0) + d for t, d in msgs)
    return b"OHDR" + struct.pack("<BBI", 2, 0x02, len(body)) + body + b"\0\0\0\0"


def test_reads_version2_superblock_and_object_headers(tmp_path):
    """Superblock 2, version-2 object headers, a compact group of link messages, a
    version-2 dataspace, a version-3 attribute and a compact data layout: the layout
    newer HDF5 libraries write (checked against the file format specification)."""
    import struct

    und = 0xFFFFFFFFFFFFFFFF
    data = np.arange(6, dtype="<f4").reshape(2, 3)
    f32 = struct.pack("<BBBBI", 0x11, 0x20, 31, 0, 4) + struct.pack("<HHBBBBI", 0, 32, 23, 8,
                                                                    0, 23, 127)
    space = struct.pack("<BBBB", 2, 2, 0, 1) + struct.pack("<QQ", 2, 3)
    layout = struct.pack("<BBH", 3, 0, data.nbytes) + data.tobytes()  # compact
    sdt = struct.pack("<BBBBI", 0x13, 0, 0, 0, 3)  # fixed string of 3 bytes
    scal = struct.pack("<BBBB", 2, 0, 0, 0)
    attr = (struct.pack("<BBHHHB", 3, 0, 5, len(sdt), len(scal), 0) + b"unit\0" + sdt + scal
            + b"kpc")
    ds = _ohdr([(0x01, space), (0x03, f32), (0x08, layout), (0x0C, attr)])
    sb_size = 8 + 4 + 4 * 8 + 4
    ds_addr = sb_size

    def link(name, addr):
        nb = name.encode()
        return struct.pack("<BBB", 1, 0, len(nb)) + nb + struct.pack("<Q", addr)

    root = _ohdr([(0x06, link("coords", ds_addr))])
    root_addr = ds_addr + len(ds)
    eof = root_addr + len(root)
    sb = (b"\x89HDF\r\n\x1a\n" + struct.pack("<BBBB", 2, 8, 8, 0)
          + struct.pack("<QQQQ", 0, und, eof, root_addr) + b"\0\0\0\0")
    p = tmp_path / "v2.h5"
    p.write_bytes(sb + ds + root)
    f = hdf5.File(str(p))
    assert f.keys() == ["coords"]
    assert f["coords"].shape == (2, 3)
    assert np.array_equal(f["coords"][()], data)
    assert f["coords"].attrs == {"unit": "kpc"}
