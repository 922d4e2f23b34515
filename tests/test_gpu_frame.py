"""The fused rotate_galaxy + filter_particles + spaxel_assignment pass
(rubix_orient_filter_assign) against the separate launches it replaces (bit-identical),
and whole pipelines with and without the fusion."""

import numpy as np
import pytest

from helpers import to_dev, workload

pytestmark = pytest.mark.gpu


def _same_bits(a, b):
    """Bitwise equality of float32 tensors (NaN rows included)."""
    import torch

    return a.shape == b.shape and torch.equal(a.view(torch.int32), b.view(torch.int32))


def _rotation():
    rng = np.random.default_rng(7)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    return q


def _particles(n=20011):
    rng = np.random.default_rng(3)
    coords = rng.normal(0.0, 4.0, (n, 3)).astype(np.float32)
    vel = rng.normal(0.0, 100.0, (n, 3)).astype(np.float32)
    mass = rng.uniform(1.0, 2.0, n).astype(np.float32)
    met = rng.uniform(0.0, 0.02, n).astype(np.float32)
    wide = rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32)
    return coords, vel, mass, met, wide


@pytest.mark.parametrize("rotate", [True, False])
def test_fused_pass_equals_separate_launches(rotate):
    import torch

    from rubix_gb300 import ops

    coords, vel, mass, met, wide = _particles()
    edges = np.linspace(-6.0, 6.0, 26).astype(np.float32)
    # particles exactly on edges (interior, outer) and NaN coordinates
    coords[:26, 0] = edges
    coords[26:52, 1] = edges
    coords[60, 0] = np.nan
    M = _rotation() if rotate else None
    c, v, e = to_dev(coords), to_dev(vel), to_dev(edges)
    fields = [to_dev(mass), to_dev(met), to_dev(wide)]
    co, vo, outs, mask, idx = ops.orient_filter_assign(c, v, M, e, fields)

    if rotate:
        rc = ops.rotate_vectors(c, M)
        rv = ops.rotate_vectors(v, M)
        assert _same_bits(co, rc) and _same_bits(vo, rv)
    else:
        assert co is None and vo is None
        rc = c
    ref_mask = ops.aperture_mask(rc, e)
    ref_idx = ops.spaxel_assign(rc, e)
    assert torch.equal(mask, ref_mask)
    assert torch.equal(idx, ref_idx)
    for f, o in zip(fields, outs):
        ref = ops.mask_zero_(f.clone(), ref_mask)
        assert _same_bits(o, ref)
    # inputs untouched; some particles inside and some outside
    assert torch.equal(fields[0], to_dev(mass))
    m = mask.cpu().numpy()
    assert 0 < m.sum() < m.size
    # no mask and no fields: assignment (and turn) only
    co2, vo2, outs2, mask2, idx2 = ops.orient_filter_assign(c, v, M, e, (), mask=False)
    assert mask2 is None and outs2 == [] and torch.equal(idx2, idx)


def test_fused_pass_in_place():
    import torch

    from rubix_gb300 import ops

    coords, vel, mass, _, _ = _particles(4097)
    edges = np.linspace(-6.0, 6.0, 26).astype(np.float32)
    M = _rotation()
    c, v, e = to_dev(coords), to_dev(vel), to_dev(edges)
    ref_c, ref_v = ops.rotate_vectors(c, M), ops.rotate_vectors(v, M)
    co, vo, _, _, idx = ops.orient_filter_assign(c, v, M, e, (), out_coords=c, out_velocity=v)
    assert co.data_ptr() == c.data_ptr() and _same_bits(c, ref_c) and _same_bits(v, ref_v)
    assert torch.equal(idx, ops.spaxel_assign(ref_c, e))


def test_pipeline_with_and_without_frame_fusion():
    import torch

    from rubix_gb300.core import RubixPipeline
    from test_gpu_steps import _config, _data

    w = workload("small")
    cfg = _config(w)
    cfg["galaxy"]["rotation"] = {"alpha": 30.0, "beta": 20.0, "gamma": 10.0}
    a = RubixPipeline(cfg, _data(w), fuse_frame=True).run().stars
    b = RubixPipeline(cfg, _data(w), fuse_frame=False).run().stars
    torch.cuda.synchronize()
    for name in ("coords", "velocity", "mass", "metallicity", "age", "mask",
                 "pixel_assignment", "datacube"):
        x, y = getattr(a, name), getattr(b, name)
        assert x.shape == y.shape and x.dtype == y.dtype, name
        assert torch.equal(x, y), name


def test_dusty_pipeline_with_and_without_frame_fusion():
    """Stars and gas both turned, filtered (gas metals kept) and assigned."""
    import torch

    from rubix_gb300.core import RubixPipeline
    from test_gpu_dust import _dust_cfg, _dusty_data, _gas

    w = workload("small")
    g, gvel = _gas(4000)
    cfg = _dust_cfg(w, "small_dust_frame")
    a = RubixPipeline(cfg, _dusty_data(w, g, gvel), fuse_frame=True).run()
    b = RubixPipeline(cfg, _dusty_data(w, g, gvel), fuse_frame=False).run()
    torch.cuda.synchronize()
    for comp in ("stars", "gas"):
        ca, cb = getattr(a, comp), getattr(b, comp)
        for name in ("coords", "velocity", "mass", "metals", "mask", "pixel_assignment"):
            x, y = getattr(ca, name, None), getattr(cb, name, None)
            if x is None and y is None:
                continue
            x, y = torch.as_tensor(x), torch.as_tensor(y)
            assert x.shape == y.shape and torch.equal(x.cpu(), y.cpu()), (comp, name)
    assert torch.equal(a.stars.datacube, b.stars.datacube)
