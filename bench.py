#!/usr/bin/env python
"""Benchmark of the particle -> IFU datacube forward path on GB300.

One step = one forward pass over one synthetic galaxy:
aperture mask + spaxel assignment + stable sort by spaxel + fused SSP lookup / mass
scaling / Doppler resampling / accumulation + PSF + LSF, all CUDA kernels of
``librubix_gb300.so``.  Workload (default ``ifu``): 10^6 particles, 150x150 spaxels x
3721 wavelengths, SSP grid 221 ages x 6 metallicities x 1221 wavelengths, PSF 15x15
sigma 1.5 spaxel, LSF sigma 1.2 A.

Metric: particles*lambda/s = (particles rendered x telescope wavelengths) / time.
``value`` is device time (CUDA events, inputs resident in HBM, L2 flushed before every
step); ``e2e`` is the same metric through ``IFURenderer.render`` from pinned host
buffers with the host->device copy of the particles and the device->host copy of the
final cube inside the timed region.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank renders its own galaxy (weak scaling, no collective on the
data path); rank 0 prints one JSON line.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "cube_fwd_ifu.txt")
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="ifu")
    ap.add_argument("--particles", type=int, default=None, help="override particle count")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_per_launch(n_particles):
    """DRAM bytes per rubix_cube_fwd launch from the committed ncu summary, scaled to
    the particle count of this run (the summary states the captured count)."""
    try:
        vals = {}
        with open(TRAFFIC_FILE) as f:
            for line in f:
                if ":" in line and not line.startswith("#"):
                    k, v = line.split(":", 1)
                    vals[k.strip()] = v.strip().split()[0]
        b = float(vals["dram_bytes_per_launch"])
        n_cap = float(vals["captured_particles"])
        fixed = float(vals.get("fixed_bytes", 0.0))
        return fixed + (b - fixed) * n_particles / n_cap
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.idx)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ------------------------------------------------------------------ reference arm
def _oracle_chunk(args):
    """Worker: oracle spectra of one particle chunk, summed per spaxel (float64)."""
    import oracle

    (mass, met, age, vz, idx, ssp_met, ssp_age, ssp_flux, wave_z, wave_t) = args
    lp_sp = oracle.particle_spectra(mass, met, age, vz, ssp_met, ssp_age, ssp_flux, wave_z, wave_t)
    uniq, inv = np.unique(idx, return_inverse=True)
    part = np.zeros((uniq.size, wave_t.size))
    np.add.at(part, inv, lp_sp)
    return uniq, part


def run_oracle_sample(w, n_sample, pool=None, chunk=256):
    """Time the oracle port on the first n_sample particles; returns seconds."""
    import oracle

    p = w.particles
    n_sample = min(n_sample, p.n)
    mask = oracle.mask_particles_outside_aperture(p.coords[:n_sample], w.edges)
    idx = oracle.square_spaxel_assignment(p.coords[:n_sample], w.edges)
    sel = np.nonzero(mask)[0]
    jobs = []
    for s in range(0, sel.size, chunk):
        j = sel[s:s + chunk]
        jobs.append((p.mass[j], p.metallicity[j], p.age[j], p.velocity[j, 2], idx[j],
                     w.ssp.metallicity, w.ssp.age, w.ssp.flux, w.wave_z, w.wave_t))
    t0 = time.perf_counter()
    res = pool.map(_oracle_chunk, jobs) if pool is not None else [_oracle_chunk(j) for j in jobs]
    cube_rows = {}
    for uniq, part in res:
        for u, row in zip(uniq, part):
            cube_rows[u] = cube_rows.get(u, 0.0) + row
    return time.perf_counter() - t0, n_sample


def reference_arm(args):
    world, rank, _ = dist_info()
    if rank != 0:
        return 0
    import multiprocessing as mp

    from rubix_gb300 import synth

    w = synth.make_workload(args.workload, n=args.particles, edge_cases=False)
    L = w.wave_t.size
    cores = os.cpu_count() or 1
    n_sample = 8192 * cores // 4
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            run_oracle_sample(w, min(n_sample, 4096), pool)
        times = []
        for _ in range(args.steps):
            dt, ns = run_oracle_sample(w, n_sample, pool)
            times.append(dt)
    value = n_sample * L * len(times) / sum(times)
    unit = "particle*lambda/s"
    line = {
        "impl": "reference", "metric": "particles*lambda/s, particle->IFU datacube forward",
        "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(w),
        "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "kind": "port",
                         "sample": f"{n_sample} particles x {L} wavelengths per step "
                                   "(float64 NumPy restatement, spawn process pool)"},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's JAX pipeline is not installable here; this arm times the "
                "NumPy restatement of its algorithm (oracle/) on the host cores",
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(w):
    p = w.particles
    return {
        "workload": f"{w.name}: {p.n} particles, {w.sbin}x{w.sbin}x{w.wave_t.size} cube, "
                    f"SSP {w.ssp.age.size} ages x {w.ssp.metallicity.size} Z x "
                    f"{w.ssp.wavelength.size} wavelengths, PSF {w.psf_size}x{w.psf_size} "
                    f"sigma {w.psf_sigma}, LSF sigma {w.lsf_sigma} A",
        "n_particles": p.n, "n_spaxels": w.sbin * w.sbin, "n_wave": int(w.wave_t.size),
        "ssp": [int(w.ssp.metallicity.size), int(w.ssp.age.size), int(w.ssp.wavelength.size)],
        "l2": "flushed before every timed step (512 MiB device write)",
        "path": "mask+assign+sort -> fused accumulate with LSF epilogue -> PSF (LSF and PSF commute)",
    }


# ------------------------------------------------------------------ our arm
def main():
    args = parse_args()
    if args.impl == "reference":
        return reference_arm(args)

    world, rank, local = dist_info()
    import torch
    import torch.distributed as dist

    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)

    from rubix_gb300 import _build, ops, synth
    from rubix_gb300 import dist as rdist
    from rubix_gb300.api import IFURenderer

    _build.build()
    # every rank renders its own galaxy (independent seeds): weak scaling, no exchange
    w = synth.make_workload(args.workload, n=args.particles, edge_cases=False,
                            seed=rdist.rank_seed(synth.WORKLOADS[args.workload]["seed"], rank))
    p = w.particles
    N, L = p.n, int(w.wave_t.size)
    S2 = w.sbin * w.sbin
    rnd = IFURenderer.from_workload(w, device=dev)
    d_in = [torch.from_numpy(a).to(dev) for a in (p.coords, p.velocity, p.mass, p.metallicity, p.age)]
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def barrier():
        if world > 1:
            dist.barrier()

    def step_device(ev=None):
        idx, mask = rnd.assign(d_in[0])
        perm, offs = rnd.sort(idx, mask)
        if ev is not None:
            ev[0].record()
        cube = rnd.accumulate(d_in[2], d_in[3], d_in[4], d_in[1], perm, offs, with_lsf=True)
        if ev is not None:
            ev[1].record()
        return rnd.psf(cube)

    for _ in range(max(3, args.warmup)):
        step_device()
    torch.cuda.synchronize()

    sampler = ClockSampler(torch.cuda.current_device() if world == 1 else local)
    n_launch0 = ops.LAUNCHES["count"]
    step_ms, cube_ms = [], []
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        step_device((c0, c1))
        e1.record()
        torch.cuda.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        cube_ms.append(c0.elapsed_time(c1))
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    launches = ops.LAUNCHES["count"] - n_launch0

    total_ms = rdist.max_over_ranks(sum(step_ms))
    value = world * N * L * args.steps / (total_ms * 1e-3)

    # ---------------- e2e through the public renderer from pinned host buffers
    e2e = None
    if not args.no_e2e:
        h_in = [torch.from_numpy(a).pin_memory() for a in (p.coords, p.velocity, p.mass, p.metallicity, p.age)]
        h_out = torch.empty((w.sbin, w.sbin, L), dtype=torch.float32).pin_memory()
        h2d = sum(x.numel() * x.element_size() for x in h_in)
        d2h = h_out.numel() * h_out.element_size()

        def step_e2e():
            st = rnd.render(h_in[0], h_in[1], h_in[2], h_in[3], h_in[4])
            h_out.copy_(st.final, non_blocking=True)

        for _ in range(2):
            step_e2e()
        torch.cuda.synchronize()
        barrier()
        e2e_ms = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            step_e2e()
            e1.record()
            torch.cuda.synchronize()
            e2e_ms.append(e0.elapsed_time(e1))
        te_ms = rdist.max_over_ranks(sum(e2e_ms))
        e2e = {"value": world * N * L * args.steps / (te_ms * 1e-3),
               "unit": "particle*lambda/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": statistics.mean(e2e_ms)}

    # ---------------- roofline of the dominant kernel (rubix_cube_fwd)
    peak, peak_kind = hbm_peak()
    flux_bytes = w.ssp.flux.size * 4
    alg_bytes = 20 * N + flux_bytes + S2 * L * 4   # particle fields + perm, SSP flux, cube write
    cube_avg_s = statistics.mean(cube_ms) * 1e-3
    achieved = alg_bytes / cube_avg_s / 1e9
    traffic = traffic_per_launch(N)
    roofline = {"kernel": "rubix_cube_fwd (fused lookup/mass/Doppler/resample/accumulate)",
                "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": traffic, "algorithmic_bytes": alg_bytes,
                "ms_per_launch": statistics.mean(cube_ms),
                "share_of_step": statistics.mean(cube_ms) / statistics.mean(step_ms)}

    # ---------------- CPU baseline (rank 0, N=1): oracle port, one core, bounded sample
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        n_sample = 1024
        run_oracle_sample(w, 128)
        dt, ns = run_oracle_sample(w, n_sample)
        cpu = {"value": ns * L / dt, "unit": "particle*lambda/s", "cores": 1, "kind": "port",
               "sample": f"first {ns} particles of the workload x {L} wavelengths, float64 "
                         "NumPy restatement (oracle/), single process"}

    if rank == 0:
        line = {
            "metric": "particles*lambda/s, particle->IFU datacube forward",
            "value": value, "unit": "particle*lambda/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": statistics.mean(step_ms),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded exponential disk; synthetic SSP grid)",
            "config": workload_config(w), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches, "clocks": clocks, "wall_s_timed": wall,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
