"""The oracle and the kernels against the committed golden fixtures
(tests/golden/make_golden.py)."""

import os

import numpy as np
import pytest

import oracle
from helpers import assert_cube_close, to_dev

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "small_n300_L64.npz")


def _golden():
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(GOLDEN), "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod, np.load(GOLDEN)


def test_oracle_reproduces_golden():
    mod, g = _golden()
    w, out = mod.stages()
    assert np.array_equal(out["pixel_assignment"], g["pixel_assignment"])
    assert np.array_equal(out["mask"], g["mask"])
    np.testing.assert_allclose(out["cube"], g["cube"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(out["final"].astype(np.float32), g["final"], rtol=0, atol=0)


@pytest.mark.gpu
def test_kernels_match_golden():
    import torch

    from rubix_gb300.api import IFURenderer

    mod, g = _golden()
    from rubix_gb300 import synth

    w = synth.make_workload("small", n=mod.N, n_wave_t=mod.NT)
    p = w.particles
    r = IFURenderer.from_workload(w)
    st = r.render(to_dev(p.coords), to_dev(p.velocity), to_dev(p.mass), to_dev(p.metallicity),
                  to_dev(p.age))
    torch.cuda.synchronize()
    assert np.array_equal(st.pixel_assignment.cpu().numpy(), g["pixel_assignment"])
    assert_cube_close(st.final.cpu().numpy(), g["final"].astype(np.float64), what="golden final")
    raw = r.accumulate(to_dev(p.mass), to_dev(p.metallicity), to_dev(p.age), to_dev(p.velocity),
                       st.perm, st.seg_offsets)
    assert_cube_close(raw.cpu().numpy(), g["cube"], what="golden raw cube")
