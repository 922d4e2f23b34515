"""bench.py's host-side helpers (no GPU): the profile-derived per-launch figures, the
algorithmic FLOP count, the workload description and the argument defaults."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_profile_figures_scale_with_the_particle_count():
    # profiles/cube_fwd_ifu.txt: captured at 1e6 particles, fixed + per-particle parts
    assert bench.traffic_per_launch(1_000_000) == pytest.approx(390.28e6)
    assert bench.instructions_per_launch(1_000_000) == pytest.approx(3001.9e6)
    # the 2e5-particle capture lies on the same line
    assert bench.instructions_per_launch(200_000) == pytest.approx(708.5e6, rel=1e-3)
    assert bench.traffic_per_launch(200_000) == pytest.approx(305.13e6, rel=2e-3)


def test_large_grid_profile_reproduces_its_first_capture():
    # profiles/cube_fwd_large.txt: keys from the 2e6 capture; the 1e6 capture lies on the line
    assert bench.traffic_per_launch(1_000_000, "large") == pytest.approx(1417.92e6, rel=1e-4)
    assert bench.instructions_per_launch(1_000_000, "large") == pytest.approx(3392.6e6, rel=1e-4)


def test_profile_figures_need_a_summary_of_the_workload_grid():
    assert bench.traffic_per_launch(1_000_000, "no-such-workload") is None
    assert bench.instructions_per_launch(1_000_000, "no-such-workload") is None


def test_cpu_step_estimate_covers_every_stage():
    from rubix_gb300 import synth

    w = synth.make_workload("small", n=2000, edge_cases=False)
    t, parts = bench.cpu_step_estimate(w, None, 256, n_sort=1000, n_planes=4, n_rows=16)
    assert set(parts) == {"assign_sort_s", "spectra_and_sum_s", "psf_s", "lsf_s"}
    assert t == pytest.approx(sum(parts.values())) and all(v > 0 for v in parts.values())


def test_summary_block_reads_nested_figures():
    line = {"value": 2.0, "config": {"workload": "large: 10 particles"},
            "roofline": {"frac": 0.5, "issue": {"frac": 0.7}}, "fwd_bwd": {"fwd_bwd_over_fwd": 2.9}}
    s = bench.summary_block(line)
    assert s["workload"] == "large" and s["accumulate_issue_frac"] == 0.7
    assert s["fwd_bwd_over_fwd"] == 2.9 and s["e2e_value"] is None


def test_workload_description_and_flops():
    from rubix_gb300 import synth

    w = synth.make_workload("small", n=100, edge_cases=False)
    cfg = bench.workload_config(w)
    assert cfg["n_particles"] == 100 and cfg["n_wave"] == w.wave_t.size
    assert "flushed" in cfg["l2"]
    f = bench.flops_per_particle_lambda(w)
    assert 7.4 < f < 7.4 + 11.0 * w.wave_z.size / w.wave_t.size + 1e-9


def test_argument_defaults(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse_args()
    assert (a.gpus, a.steps, a.warmup, a.impl, a.workload) == (1, 10, 3, "ours", "large")
    assert a.warmup >= 3 and a.extras is None and a.dust == 0
