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
step); ``e2e`` is the same metric host to host through the public renderer
(``IFURenderer.host_stream``): K steps back to back, each uploading its particles from
pinned host memory and downloading its final cube into pinned host memory inside the
timed region, the copies of one step overlapping the compute of the next.  The
latency of one isolated step (``IFURenderer.render`` plus the download, nothing
overlapped) is reported beside it.

``roofline`` relates the dominant kernel to HBM (its algorithmic bytes), to the FP32
FMA rate (its algorithmic FLOPs; measured peak) and to instruction issue (its ncu
instruction count, the resource it is bound by).  At N = 1 the line also carries the
extra measurements (``--extras`` selects them): forward+backward, the plain PyTorch
GPU path, the dusty step, the FITS layout, the noise pass, a galaxy-file load, the
RubixPipeline step API and a ragged batch of 256 galaxies.

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
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="large")
    ap.add_argument("--particles", type=int, default=None, help="override particle count")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the fwd+bwd, plain-GPU-path and ragged-batch measurements")
    ap.add_argument("--extras", default=None, metavar="NAMES",
                    help="comma-separated subset of the extra measurements (fwd_bwd, "
                         "plain_gpu, plain_gpu_fwd_bwd, dusty, fits_layout, noise, "
                         "galaxy_file, pipeline_api, ragged); default all")
    ap.add_argument("--ssp-wave", type=int, default=None, metavar="N",
                    help="synthetic SSP grid with N wavelengths (e.g. 5994, FSPS-sized)")
    ap.add_argument("--dust", type=int, default=0, metavar="N_GAS",
                    help="measure the dusty step (calc_dusty_ifu) with N_GAS gas cells as "
                         "the main line (device time; no e2e)")
    return ap.parse_args()


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def fma_probe(dev, iters: int = 4096):
    """(FMAs launched, out tensor): one launch of the FP32 FMA-rate probe
    (bench_fma_probe.cu, built by rubix_gb300._build.build_probe into its own library)
    on the current stream."""
    import ctypes

    import torch

    from rubix_gb300 import _build

    lib = ctypes.CDLL(_build.build_probe())
    lib.rubix_probe_fma_blocks.restype = ctypes.c_int
    lib.rubix_probe_fma.restype = ctypes.c_int
    lib.rubix_probe_fma.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
    blocks = lib.rubix_probe_fma_blocks()
    if blocks <= 0:
        raise RuntimeError("rubix_probe_fma_blocks failed")
    out = torch.empty(blocks * 256, dtype=torch.float32, device=dev)
    rc = lib.rubix_probe_fma(ctypes.c_void_p(out.data_ptr()), int(iters),
                             ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    if rc != 0:
        raise RuntimeError(f"rubix_probe_fma returned {rc}")
    return blocks * 256 * int(iters) * 128, out


def fp32_peak_tflops(dev, reps=5):
    """FP32 FMA rate of this GPU from the FMA-chain probe (best of reps)."""
    import torch

    best = 0.0
    for i in range(reps + 2):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        n_fma, _ = fma_probe(dev)
        e1.record()
        torch.cuda.synchronize()
        if i >= 2:
            best = max(best, 2.0 * n_fma / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def flops_per_particle_lambda(w):
    """Algorithmic FP32 operations of kernel (b) per (particle, telescope wavelength):
    the evaluation does 7 (x - lambda'_k, the interpolation FMA, T' FMA, accumulation
    FMA) plus the bin width shared by a batch (about 0.4); the row build does 11 per SSP
    entry (four-corner mix 7, lambda' 1, slope 3) over the n_e entries that span the
    telescope range, spread over the L wavelengths."""
    t0, t1 = float(w.wave_t[0]), float(w.wave_t[-1])
    n_e = int(np.count_nonzero((w.wave_z >= t0) & (w.wave_z <= t1))) + 2
    return 7.4 + 11.0 * n_e / float(w.wave_t.size)


def profile_file(workload):
    """The committed ncu summary of the main kernel on this workload's spaxel grid."""
    return os.path.join(ROOT, "profiles", f"cube_fwd_{workload}.txt")


def _profile_per_launch(n_particles, total_key, fixed_key, workload="ifu"):
    """A per-launch count of the main kernel from the committed ncu summary of the
    workload (fixed part + per-particle part), scaled to the particle count of this run;
    None when no summary exists for the workload's grid."""
    try:
        vals = {}
        with open(profile_file(workload)) as f:
            for line in f:
                if ":" in line and not line.startswith("#"):
                    k, v = line.split(":", 1)
                    vals[k.strip()] = v.strip().split()[0]
        b = float(vals[total_key])
        n_cap = float(vals["captured_particles"])
        fixed = float(vals.get(fixed_key, 0.0))
        return fixed + (b - fixed) * n_particles / n_cap
    except Exception:
        return None


def traffic_per_launch(n_particles, workload="ifu"):
    """DRAM bytes per rubix_cube_fwd main-kernel launch (ncu, scaled to the run)."""
    return _profile_per_launch(n_particles, "dram_bytes_per_launch", "fixed_bytes", workload)


def instructions_per_launch(n_particles, workload="ifu"):
    """Warp instructions per main-kernel launch (ncu smsp__inst_executed.sum, scaled)."""
    return _profile_per_launch(n_particles, "warp_instructions_per_launch",
                               "fixed_warp_instructions", workload)


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


# ------------------------------------------------------------------ CPU legs (oracle port)
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
    """Time the oracle port's per-particle spectra and per-spaxel sums on the first
    n_sample particles (on `pool` when given); returns (seconds, particles kept)."""
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
    return time.perf_counter() - t0, int(sel.size)


def cpu_step_estimate(w, pool, n_sample, n_sort=2_000_000, n_planes=32, n_rows=512):
    """One forward step of the workload on the host with the oracle port, estimated from
    bounded samples of each stage, each scaled to the whole workload:
      * aperture mask + spaxel assignment + stable sort of the first n_sort particles
        (single process), scaled by N / n_sort;
      * per-particle spectra + per-spaxel sums of n_sample particles on `pool`, scaled by
        the workload's kept particles / the sample's;
      * the PSF (FFT 'same' convolution per wavelength plane) of n_planes planes of the
        full spatial field, scaled by L / n_planes;
      * the LSF of n_rows spaxel spectra, scaled by spaxels / n_rows.
    Returns (seconds per step, {stage: seconds})."""
    import oracle

    p = w.particles
    N, L, S = p.n, int(w.wave_t.size), int(w.sbin)
    ns = min(n_sort, N)
    t0 = time.perf_counter()
    m = oracle.mask_particles_outside_aperture(p.coords[:ns], w.edges)
    idx = oracle.square_spaxel_assignment(p.coords[:ns], w.edges)
    np.argsort(np.where(m, idx, S * S), kind="stable")
    t_sort = (time.perf_counter() - t0) * N / ns
    kept_frac = float(np.mean(m)) if ns else 1.0
    dt, kept = run_oracle_sample(w, n_sample, pool)
    t_part = dt * (kept_frac * N) / max(kept, 1)
    rng = np.random.default_rng(0)
    slab = rng.random((S, S, n_planes))
    K = oracle.gaussian_kernel_2d(w.psf_size, w.psf_size, w.psf_sigma)
    t0 = time.perf_counter()
    oracle.apply_psf(slab, K, method="fft")
    t_psf = (time.perf_counter() - t0) * L / n_planes
    rows = rng.random((min(n_rows, S * S), L))
    t0 = time.perf_counter()
    oracle.apply_lsf(rows, w.lsf_sigma, w.wave_res)
    t_lsf = (time.perf_counter() - t0) * S * S / rows.shape[0]
    parts = {"assign_sort_s": t_sort, "spectra_and_sum_s": t_part, "psf_s": t_psf,
             "lsf_s": t_lsf}
    return sum(parts.values()), parts


def cpu_sample_text(w, n_sample, cores):
    return (f"estimated {w.name} forward step from bounded samples, each scaled to the "
            f"workload: mask + assignment + stable sort of min(N, 2e6) particles (1 "
            f"process), spectra + per-spaxel sums of {n_sample} particles ({cores} spawn "
            f"processes, float64 NumPy restatement, oracle/), PSF of 32 wavelength planes "
            f"and LSF of 512 spaxel spectra (1 process, float64)")


def reference_arm(args):
    world, rank, _ = dist_info()
    if rank != 0:
        return 0
    import multiprocessing as mp

    from rubix_gb300 import synth

    w = synth.make_workload(args.workload, n=args.particles, edge_cases=False)
    N, L = w.particles.n, w.wave_t.size
    cores = os.cpu_count() or 1
    n_sample = 2048 * cores
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            run_oracle_sample(w, min(n_sample, 1024), pool)
        times, parts = [], None
        for _ in range(args.steps):
            t, parts = cpu_step_estimate(w, pool, n_sample)
            times.append(t)
    value = N * L * len(times) / sum(times)
    unit = "particle*lambda/s"
    line = {
        "impl": "reference", "metric": "particles*lambda/s, particle->IFU datacube forward",
        "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(w),
        "cpu_baseline": {"value": value, "unit": unit, "cores": cores, "kind": "port",
                         "sample": cpu_sample_text(w, n_sample, cores), "stages_s": parts},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's JAX pipeline is not installable here; this arm times the "
                "NumPy restatement of its algorithm (oracle/) on the host cores; the "
                "reference design itself materialises N x L spectra (rubix/core/ifu.py:"
                "278-283), %.0f GB for this workload" % (4.0 * N * L / 1e9),
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
        "path": "mask+assign+sort -> fused accumulate with LSF epilogue -> PSF (LSF and PSF commute)"
                + (f" -> noise at S/N {w.noise_s2n}" if w.noise_s2n else ""),
    }



# ------------------------------------------------------------------ extra measurements
def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time_steps(fn, steps, warmup, flush=None):
    """Mean ms of fn() over `steps` timed calls after `warmup` untimed ones."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        e0, e1 = _events()
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return statistics.mean(ms)


def _diff_setup(dev):
    """Differentiation workload: 2e5 particles, 50x50x3721 cube; target rendered from
    perturbed parameters (mass x1.05, age and Z +0.1 dex, v_los +20 km/s, PSF sigma
    x1.1); loss = sum w (cube - target)^2 with w = 1/((target/20)^2 + floor)."""
    import torch

    from rubix_gb300 import synth
    from rubix_gb300.api import IFURenderer
    from rubix_gb300.autograd import render_cube

    w = synth.make_workload("diff", edge_cases=False)
    p = w.particles
    r = IFURenderer.from_workload(w, device=dev, psf=False, lsf=False)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    coords = t(p.coords)
    base = {"mass": t(p.mass), "metallicity": t(p.metallicity), "age": t(p.age),
            "velocity": t(p.velocity)}
    with torch.no_grad():
        vel_t = base["velocity"].clone()
        vel_t[:, 2] += 20.0
        target = render_cube(r, coords, vel_t, base["mass"] * 1.05,
                             base["metallicity"] * 10 ** 0.1, base["age"] * 10 ** 0.1,
                             w.psf_sigma * 1.1, w.lsf_sigma, w.psf_size, w.wave_res)
        floor = 1e-6 * float(target.abs().max()) ** 2
        weight = 1.0 / ((target / 20.0) ** 2 + floor)
    return w, r, coords, base, target.contiguous(), weight.contiguous()


def fwd_bwd_bench(dev, steps, warmup, flush):
    """Forward + backward of the differentiation workload through DatacubeFunction."""
    import torch

    from rubix_gb300.autograd import render_cube

    w, r, coords, base, target, weight = _diff_setup(dev)
    N, L = w.particles.n, int(w.wave_t.size)
    leaves = {k: v.clone().requires_grad_() for k, v in base.items()}
    sp = torch.tensor(w.psf_sigma, dtype=torch.float64, device=dev, requires_grad=True)
    sl = torch.tensor(w.lsf_sigma, dtype=torch.float64, device=dev, requires_grad=True)

    def fwd():
        with torch.no_grad():
            return render_cube(r, coords, leaves["velocity"], leaves["mass"],
                               leaves["metallicity"], leaves["age"], sp, sl, w.psf_size,
                               w.wave_res)

    def fwd_bwd():
        for v in list(leaves.values()) + [sp, sl]:
            v.grad = None
        cube = render_cube(r, coords, leaves["velocity"], leaves["mass"], leaves["metallicity"],
                           leaves["age"], sp, sl, w.psf_size, w.wave_res)
        d = cube - target
        (weight * d * d).sum().backward()

    f_ms = _time_steps(fwd, steps, warmup, flush)
    fb_ms = _time_steps(fwd_bwd, steps, warmup, flush)
    return {"metric": "particles*lambda/s, forward+backward (loss gradients w.r.t. mass, "
                      "metallicity, age, v_los, sigma_psf, sigma_lsf)",
            "value": N * L / (fb_ms * 1e-3), "unit": "particle*lambda/s",
            "ms_per_step": fb_ms, "fwd_ms_per_step": f_ms, "fwd_bwd_over_fwd": fb_ms / f_ms,
            "workload": f"diff: {N} particles, {w.sbin}x{w.sbin}x{L} cube, SSP "
                        f"{w.ssp.age.size}x{w.ssp.metallicity.size}x{w.ssp.wavelength.size}, "
                        f"PSF {w.psf_size}x{w.psf_size} sigma {w.psf_sigma}, LSF sigma "
                        f"{w.lsf_sigma} A; loss = inverse-variance weighted L2 to a target "
                        "rendered from perturbed parameters"}


def dusty_bench(dev, w, d_in, steps, warmup, flush, n_gas=500_000):
    """The main step with calc_dusty_ifu's dust extinction: 5e5 gas cells -> per-cell
    extinction -> A_V of every star (rubix's column interpolation) -> dusty accumulate
    (+LSF), PSF, noise.  Also times the A_V passes and the dusty accumulate alone."""
    import torch

    from rubix_gb300 import ops, synth
    from rubix_gb300.api import IFURenderer

    g = synth.make_gas(n_gas, seed=2)
    rnd = IFURenderer.from_workload(w, device=dev, dust={"extinction_model": "Cardelli89",
                                                         "Rv": 3.1})
    gas = tuple(torch.from_numpy(a).to(dev) for a in (g.coords, g.mass, g.metals))
    N, L = w.particles.n, int(w.wave_t.size)
    state = {}

    def av_only():
        idx, mask = rnd.assign(d_in[0])
        state["sorted"] = rnd.sort(idx, mask)
        state["av"] = rnd.dust_av(d_in[0], idx, *gas)

    def step():
        idx, mask = rnd.assign(d_in[0])
        perm, offs = rnd.sort(idx, mask)
        av = rnd.dust_av(d_in[0], idx, *gas)
        cube = rnd.accumulate(d_in[2], d_in[3], d_in[4], d_in[1], perm, offs, with_lsf=True,
                              dust_av=av)
        return rnd.noise_(rnd.psf(cube))

    n0 = ops.LAUNCHES["count"]
    step()
    launches = ops.LAUNCHES["count"] - n0
    ms = _time_steps(step, steps, warmup, flush)
    av_ms = _time_steps(av_only, steps, warmup, flush)
    perm, offs = state["sorted"]
    acc_ms = _time_steps(lambda: rnd.accumulate(d_in[2], d_in[3], d_in[4], d_in[1], perm, offs,
                                                with_lsf=True, dust_av=state["av"]),
                         steps, warmup, flush)
    return {"metric": "particles*lambda/s, particle->IFU datacube forward with dust "
                      "extinction (calc_dusty_ifu)",
            "value": N * L / (ms * 1e-3), "unit": "particle*lambda/s", "ms_per_step": ms,
            "assign_sort_av_ms": av_ms, "dusty_accumulate_ms": acc_ms,
            "gpu_launches_per_step": launches,
            "workload": f"{w.name} stars ({N}) + {n_gas} gas cells (exponential disk, h_z 0.15 "
                        "kpc, log-normal masses, 12+log(O/H) 7.9-9.2), Cardelli89 R_V 3.1, "
                        "broken power-law dust-to-gas ratio (X_CO = Z)"}


def pipeline_bench(dev, w, steps, warmup, flush):
    """The same forward through rubix's step API (RubixPipeline.run: rotate_galaxy,
    filter_particles, spaxel_assignment, reshape_data, the lazy spectra steps,
    calculate_datacube, convolve_psf, convolve_lsf, apply_noise) with device-resident
    inputs; the rotation reads the 3x3 inertia tensor back for the host
    eigen-decomposition."""
    import torch

    from rubix_gb300.core import (Galaxy, RubixData, RubixPipeline, StarsData,
                                  register_ssp_template, register_telescope)
    from rubix_gb300.core.ssp import SSPGrid
    from rubix_gb300 import synth

    register_ssp_template("bench_ssp", SSPGrid(age=w.ssp.age, metallicity=w.ssp.metallicity,
                                               wavelength=w.ssp.wavelength, flux=w.ssp.flux))
    fov = synth.WORKLOADS[w.name]["fov"]
    register_telescope("bench_ifu", dict(fov=fov, spatial_res=synth.SPATIAL_RES,
                                         wave_range=list(synth.WAVE_RANGE),
                                         wave_res=synth.WAVE_RES, lsf_fwhm=2.51,
                                         signal_to_noise=None, aperture_type="square",
                                         pixel_type="square"))
    cfg = {"pipeline": {"name": "calc_ifu"}, "logger": {"log_level": "WARNING"},
           "data": {"args": {"particle_type": ["stars"]}},
           "telescope": {"name": "bench_ifu",
                         "psf": {"name": "gaussian", "size": w.psf_size, "sigma": w.psf_sigma},
                         "lsf": {"sigma": w.lsf_sigma},
                         "noise": {"signal_to_noise": 1e30, "noise_distribution": "normal"}},
           "cosmology": {"name": "PLANCK15"},
           "galaxy": {"dist_z": w.dist_z, "rotation": {"type": "face-on"}},
           "ssp": {"template": {"name": "bench_ssp"}, "method": "linear"}}
    p = w.particles
    dev_in = [torch.from_numpy(a).to(dev) for a in (p.coords, p.velocity, p.mass,
                                                     p.metallicity, p.age)]

    def run():
        data = RubixData(galaxy=Galaxy(halfmassrad_stars=5.0),
                         stars=StarsData(coords=dev_in[0], velocity=dev_in[1], mass=dev_in[2],
                                         metallicity=dev_in[3], age=dev_in[4]))
        return RubixPipeline(cfg, data).run().stars.datacube

    ms = _time_steps(run, steps, warmup, flush)
    N, L = p.n, int(w.wave_t.size)
    return {"metric": "particles*lambda/s, particle->IFU datacube forward through "
                      "RubixPipeline(config, data).run()",
            "value": N * L / (ms * 1e-3), "unit": "particle*lambda/s", "ms_per_step": ms,
            "path": "rotate_galaxy (face-on), filter_particles, spaxel_assignment (the "
                    "three in one pass), reshape_data, calculate_spectra, "
                    "scale_spectrum_by_mass, doppler_shift_and_resampling, "
                    "calculate_datacube (with the LSF in its epilogue), convolve_psf, "
                    "convolve_lsf (applied in the epilogue), apply_noise (S/N 1e30: the noise "
                    "kernels run, the cube is unchanged in float32); the pipeline is built "
                    "inside the timed region"}


def galaxy_file_bench(dev, w, steps):
    """rubix's galaxy file of the workload's particles (rubix_galaxy.h5, written once,
    untimed) read back through get_rubix_data (HDF5 read, centring, median velocity)
    and uploaded to the device; host wall time per load."""
    import shutil
    import tempfile
    import time

    import torch

    from rubix_gb300.core import create_rubix_file, get_rubix_data

    p = w.particles
    tmp = tempfile.mkdtemp(prefix="rubix_galaxy_")
    try:
        path = create_rubix_file(
            os.path.join(tmp, "rubix_galaxy.h5"),
            {"stars": {"coords": p.coords, "velocity": p.velocity, "mass": p.mass,
                       "metallicity": p.metallicity, "age": p.age}},
            {"center": np.zeros(3), "halfmassrad_stars": np.float64(5.0),
             "redshift": np.float64(w.dist_z)}, {"simulation": "synthetic"},
            {"galaxy": {"center": "kpc", "halfmassrad_stars": "kpc", "redshift": ""},
             "stars": {"coords": "kpc", "velocity": "km/s", "mass": "Msun",
                       "metallicity": "", "age": "Gyr"}})
        nbytes = os.path.getsize(path)
        cfg = {"output_path": tmp, "data": {"args": {"particle_type": ["stars"]}},
               "logger": {"log_level": "WARNING"}}
        ts = []
        for _ in range(steps + 1):
            t0 = time.perf_counter()
            d = get_rubix_data(cfg)
            st = d.stars
            on_dev = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)
                      for a in (st.coords, st.velocity, st.mass, st.metallicity, st.age)]
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
            del on_dev
        ms = statistics.median(ts[1:]) * 1e3
        return {"what": "get_rubix_data(config) on a rubix_galaxy.h5 of the workload "
                        "(rubix_gb300.hdf5 reader, centring) + upload of the five arrays",
                "file_bytes": nbytes, "ms": ms, "mb_per_s": nbytes / (ms * 1e-3) / 1e6,
                "particles": p.n}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def noise_bench(dev, cube, steps, warmup, flush):
    """apply_noise (S/N 20, normal draws) on a copy of the final cube: the flux image,
    the median select and the noise pass; the noise kernel's algorithmic bytes are 2 C
    (read + write of the cube)."""
    from rubix_gb300 import ops

    work = cube.clone()
    flux = ops.flux_image(work)
    med = ops.noise_median(flux)
    if float(med) == 0.0:
        # rubix's median is NaN (-> 0, no noise) when a spaxel is empty; time the pass
        # with the median of the non-empty spaxels instead
        med = flux[flux > 0].median().reshape(())
    kernel_ms = _time_steps(lambda: ops.apply_noise_(work, 20.0, "normal", 1, flux=flux,
                                                     median=med), steps, warmup, flush)
    step_ms = _time_steps(lambda: ops.apply_noise_(work, 20.0, "normal", 1), steps, warmup,
                          flush)
    nbytes = 2 * cube.numel() * 4
    peak, kind = hbm_peak()
    return {"kernel": "rubix_apply_noise", "ms": kernel_ms,
            "ms_with_flux_image_and_median": step_ms,
            "achieved_gbs": nbytes / (kernel_ms * 1e-3) / 1e9, "peak_gbs": peak,
            "frac": nbytes / (kernel_ms * 1e-3) / 1e9 / peak, "peak_source": kind,
            "bytes": nbytes}


def fits_bench(dev, cube, steps, warmup, flush):
    """FITS layout of the final cube (transpose to [lambda][x][y] + big-endian) on the
    GPU: algorithmic bytes 2 C per launch (read + write), against the HBM peak."""
    from rubix_gb300 import ops

    out = ops.fits_cube_layout(cube)
    ms = _time_steps(lambda: ops.fits_cube_layout(cube, out=out), steps, warmup, flush)
    nbytes = 2 * cube.numel() * 4
    peak, kind = hbm_peak()
    return {"kernel": "rubix_fits_cube_layout", "ms": ms, "achieved_gbs": nbytes / ms / 1e6,
            "peak_gbs": peak, "frac": nbytes / ms / 1e6 / peak, "peak_source": kind,
            "bytes": nbytes}


# The plain GPU path: the same algorithm written with stock torch operations (gathers,
# searchsorted, index_add_, conv2d, conv1d) on the same GPU, materialising the
# per-particle spectra like the reference's step functions do.
def plain_cube(ssp, zg, ag, wave_z, wave_t, mass, Z, A, v, idx, keep, nseg, psf_t, lsf_t,
               chunk=65536):
    import torch
    import torch.nn.functional as F

    c_kms = 299792.458
    L = wave_t.numel()
    nZ, nA, nW = ssp.shape
    dlt = torch.diff(wave_t, prepend=wave_t[:1])
    lo_t, hi_t = wave_t.min(), wave_t.max()
    cube = torch.zeros((nseg, L), dtype=torch.float32, device=ssp.device)
    sel = torch.nonzero(keep, as_tuple=True)[0]
    for s in range(0, sel.numel(), chunk):
        j = sel[s:s + chunk]
        z, a, m, vv = Z[j], A[j], mass[j], v[j]
        iz = torch.clamp(torch.searchsorted(zg, z, right=True), 1, nZ - 1)
        ia = torch.clamp(torch.searchsorted(ag, a, right=True), 1, nA - 1)
        tz = ((z - zg[iz - 1]) / (zg[iz] - zg[iz - 1]))[:, None]
        ta = ((a - ag[ia - 1]) / (ag[ia] - ag[ia - 1]))[:, None]
        G = ((1 - tz) * (1 - ta) * ssp[iz - 1, ia - 1] + tz * (1 - ta) * ssp[iz, ia - 1]
             + (1 - tz) * ta * ssp[iz - 1, ia] + tz * ta * ssp[iz, ia])
        out = (z < zg[0]) | (z > zg[-1]) | (a < ag[0]) | (a > ag[-1])
        G = torch.where(out[:, None], torch.zeros_like(G), G) * m[:, None]
        lp = wave_z[None, :] * torch.exp(vv / c_kms)[:, None]
        inr = (lp >= lo_t) & (lp <= hi_t)
        T = (G * torch.diff(lp, dim=1, prepend=lp[:, :1]) * inr).sum(1)
        q = wave_t[None, :].expand(lp.shape[0], L).contiguous()
        k = torch.clamp(torch.searchsorted(lp, q, right=True), 1, nW - 1)
        x0, x1 = torch.gather(lp, 1, k - 1), torch.gather(lp, 1, k)
        f0, f1 = torch.gather(G, 1, k - 1), torch.gather(G, 1, k)
        I = f0 + (q - x0) / (x1 - x0) * (f1 - f0)
        I = torch.where(q < lp[:, :1], G[:, :1], torch.where(q > lp[:, -1:], G[:, -1:], I))
        Tp = (I * dlt[None, :]).sum(1)
        sc = torch.nan_to_num(T / Tp, nan=0.0)
        cube.index_add_(0, idx[j].long(), I * sc[:, None])
    S = int(round(nseg ** 0.5))
    m = psf_t.numel()
    k2 = (psf_t[:, None] * psf_t[None, :]).flip(0, 1)[None, None]
    planes = cube.view(S, S, L).permute(2, 0, 1).unsqueeze(1)
    planes = F.conv2d(planes, k2, padding=(m - 1) // 2)
    cube = planes.squeeze(1).permute(1, 2, 0).reshape(nseg, 1, L)
    K = lsf_t.numel()
    cube = F.conv1d(cube, lsf_t.flip(0)[None, None], padding=(K - 1) // 2)
    return cube.view(S, S, L)


def plain_bench(dev, w, rnd, d_in, ours_cube, steps, warmup, flush):
    import torch

    from rubix_gb300 import telescope as tel

    p = w.particles
    N, L = p.n, int(w.wave_t.size)
    idx, mask = rnd.assign(d_in[0])
    keep = mask.bool()
    psf_t = torch.tensor(tel.gaussian_taps_1d(w.psf_size, w.psf_sigma), dtype=torch.float32,
                         device=dev)
    lsf_t = torch.tensor(tel.lsf_taps(w.lsf_sigma, w.wave_res), dtype=torch.float32, device=dev)

    def fwd():
        with torch.no_grad():
            return plain_cube(rnd.ssp_flux, rnd.ssp_metallicity, rnd.ssp_age, rnd.ssp_wave_z,
                              rnd.wave_t, d_in[2], d_in[3], d_in[4], d_in[1][:, 2], idx, keep,
                              w.sbin * w.sbin, psf_t, lsf_t)

    ms = _time_steps(fwd, max(1, min(steps, 3)), 1, flush)
    cube = fwd()
    rel = float((cube - ours_cube).abs().max() / ours_cube.abs().max())
    return {"metric": "particles*lambda/s, particle->IFU datacube forward, plain GPU path",
            "value": N * L / (ms * 1e-3), "unit": "particle*lambda/s", "ms_per_step": ms,
            "max_rel_diff_vs_ours": rel,
            "path": "torch eager: searchsorted + gathers (bilinear lookup), exp Doppler, "
                    "searchsorted + gathers (interp), index_add_ (spaxel sum), conv2d (PSF), "
                    "conv1d (LSF); per-particle spectra materialised in chunks of 65536"}


def plain_fwd_bwd_bench(dev, steps, warmup):
    """fwd+bwd of the differentiation workload through torch autograd of plain_cube."""
    import torch

    from rubix_gb300 import telescope as tel
    from rubix_gb300.autograd import lsf_taps_grad, psf_taps_grad

    w, r, coords, base, target, weight = _diff_setup(dev)
    N, L = w.particles.n, int(w.wave_t.size)
    idx, mask = r.assign(coords)
    keep = mask.bool()
    x = np.arange(-((w.psf_size - 1) / 2), ((w.psf_size - 1) / 2) + 1)
    xl = np.arange(-12 * w.wave_res, 12 * w.wave_res + w.wave_res, w.wave_res,
                   dtype=np.float32).astype(np.float64)
    xt = torch.tensor(x, dtype=torch.float32, device=dev)
    xlt = torch.tensor(xl, dtype=torch.float32, device=dev)
    leaves = {k: v.clone().requires_grad_() for k, v in base.items()}
    sp = torch.tensor(w.psf_sigma, dtype=torch.float32, device=dev, requires_grad=True)
    sl = torch.tensor(w.lsf_sigma, dtype=torch.float32, device=dev, requires_grad=True)

    def fwd_bwd():
        for v in list(leaves.values()) + [sp, sl]:
            v.grad = None
        e = torch.exp(-xt ** 2 / (2 * sp ** 2))
        pt = e / e.sum()
        g = torch.exp(-0.5 * xlt ** 2 / sl ** 2)
        lt = g / g.sum()
        cube = plain_cube(r.ssp_flux, r.ssp_metallicity, r.ssp_age, r.ssp_wave_z, r.wave_t,
                          leaves["mass"], leaves["metallicity"], leaves["age"],
                          leaves["velocity"][:, 2], idx, keep, w.sbin * w.sbin, pt, lt,
                          chunk=1 << 30)
        d = cube - target
        (weight * d * d).sum().backward()

    ms = _time_steps(fwd_bwd, max(1, min(steps, 3)), 1)
    return {"metric": "particles*lambda/s, forward+backward, plain GPU path (torch autograd)",
            "value": N * L / (ms * 1e-3), "unit": "particle*lambda/s", "ms_per_step": ms}


def plain_assign(coords, edges, S):
    """rubix's square_spaxel_assignment and aperture mask in stock torch operations
    (searchsorted digitize, clip, flatten; inclusive aperture; ids >= S^2 dropped)."""
    import torch

    nb = edges.numel() - 1
    x, y = coords[:, 0].contiguous(), coords[:, 1].contiguous()
    ix = torch.clamp(torch.searchsorted(edges, x, right=True) - 1, 0, nb - 1)
    iy = torch.clamp(torch.searchsorted(edges, y, right=True) - 1, 0, nb - 1)
    idx = ix + nb * iy
    keep = ((x >= edges[0]) & (x <= edges[-1]) & (y >= edges[0]) & (y <= edges[-1])
            & (idx < S * S))
    return idx, keep


def _plain_taps(psf_sigma, psf_size, lsf_sigma, wave_res, dev):
    """Normalised PSF and LSF taps as differentiable torch functions of the sigmas."""
    import torch

    x = torch.tensor(np.arange(-((psf_size - 1) / 2), ((psf_size - 1) / 2) + 1),
                     dtype=torch.float32, device=dev)
    xl = torch.tensor(np.arange(-12 * wave_res, 12 * wave_res + wave_res, wave_res,
                                dtype=np.float32), dtype=torch.float32, device=dev)
    e = torch.exp(-x ** 2 / (2 * psf_sigma ** 2))
    gl = torch.exp(-0.5 * xl ** 2 / lsf_sigma ** 2)
    return e / e.sum(), gl / gl.sum()


def plain_galaxy_forward(r, c, v, m, z, a, edges, S, psf_sigma, psf_size, lsf_sigma,
                         wave_res):
    """One galaxy through the plain GPU path (stock torch operations, no kernel of
    this package)."""
    import torch

    idx, keep = plain_assign(c, edges, S)
    pt, lt = _plain_taps(torch.tensor(psf_sigma, device=c.device),
                         psf_size, torch.tensor(lsf_sigma, device=c.device), wave_res,
                         c.device)
    return plain_cube(r.ssp_flux, r.ssp_metallicity, r.ssp_age, r.ssp_wave_z, r.wave_t, m, z,
                      a, v[:, 2], idx, keep, S * S, pt, lt)


def plain_galaxy_forward_backward(r, c, v, m, z, a, edges, S, psf_sigma, psf_size, lsf_sigma,
                                  wave_res, target, weight, chunk=65536):
    """Loss sum(weight (cube - target)^2) of one galaxy and its gradients (mass,
    metallicity, age, v_los, sigma_PSF, sigma_LSF) through torch autograd of the plain
    path.  The cube is linear in the particles and the convolutions, so the backward
    recomputes it chunk by chunk against the cube adjoint (the whole galaxy's autograd
    graph would not fit in memory for 10^6 particles)."""
    import torch

    idx, keep = plain_assign(c, edges, S)
    leaves = [t.detach().clone().requires_grad_() for t in (m, z, a, v[:, 2])]
    sp = torch.tensor(float(psf_sigma), device=c.device, requires_grad=True)
    sl = torch.tensor(float(lsf_sigma), device=c.device, requires_grad=True)
    grid = (r.ssp_flux, r.ssp_metallicity, r.ssp_age, r.ssp_wave_z, r.wave_t)
    with torch.no_grad():
        pt, lt = _plain_taps(sp, psf_size, sl, wave_res, c.device)
        cube = plain_cube(*grid, *leaves, idx, keep, S * S, pt, lt)
        d = cube - target
        loss = (weight * d * d).sum()
        g = 2.0 * weight * d
    for s in range(0, c.shape[0], chunk):
        e = min(c.shape[0], s + chunk)
        pt, lt = _plain_taps(sp, psf_size, sl, wave_res, c.device)
        part = plain_cube(*grid, *(x[s:e] for x in leaves), idx[s:e], keep[s:e], S * S, pt, lt)
        (part * g).sum().backward()
    return loss, [x.grad for x in leaves], sp.grad, sl.grad


def ragged_bench(dev, steps, warmup):
    """256 galaxies (particle counts log-uniform 1e3-1e6, spaxel grids 16^2-64^2, PSF sigma
    0.8-2.0) rendered as one ragged batch (one launch per kernel; fwd+bwd replayed from a
    CUDA graph; work items autotuned), against two per-galaxy loops: the plain GPU path
    (stock torch operations, the loop a user of the reference's design would write on a
    GPU) and this package's own single-galaxy launches."""
    import torch

    from rubix_gb300 import autotune, ragged, synth
    from rubix_gb300 import telescope as tel
    from rubix_gb300.api import IFURenderer

    counts, sbins, sig, sizes = ragged.synthetic_batch_spec()
    ssp = synth.make_ssp(221, 6, 1221, seed=2)
    wave_t = tel.calculate_wave_seq(synth.WAVE_RANGE, synth.WAVE_RES)
    edges = [ragged.galaxy_edges(int(s), synth.DIST_Z) for s in sbins]
    gals = [synth.make_galaxy(int(n), seed=1000 + g) for g, n in enumerate(counts)]
    cat = [np.concatenate([getattr(p, k) for p in gals]) for k in
           ("coords", "velocity", "mass", "metallicity", "age")]
    del gals
    r = IFURenderer(ssp.age, ssp.metallicity, ssp.wavelength, ssp.flux, wave_t, edges[0],
                    int(sbins[0]), synth.DIST_Z, device=dev)
    b = ragged.RaggedBatch(r, counts, sbins, edges, sig, sizes, synth.LSF_SIGMA, synth.WAVE_RES)
    d = [torch.from_numpy(a).to(dev) for a in cat]
    args = (d[0], d[1], d[2], d[3], d[4])
    n_gal = b.n_gal
    tune = autotune.autotune(lambda: b.render(*args), key=("ragged", n_gal, int(counts.sum())),
                             device=dev.index or 0, candidates=((256, 64), (128, 64), (64, 16)),
                             repeats=1)
    fwd_ms = _time_steps(lambda: b.render(*args), steps, warmup)
    loop_fwd_ms = _time_steps(lambda: ragged.render_per_galaxy(b, *args), steps, 1)
    d_edges = [torch.from_numpy(e).to(dev) for e in edges]

    def galaxy(g):
        p0, p1 = int(b.t.poff[g]), int(b.t.poff[g + 1])
        return [x[p0:p1] for x in args]

    def plain_loop():
        with torch.no_grad():
            for g in range(n_gal):
                plain_galaxy_forward(r, *galaxy(g), d_edges[g], int(sbins[g]), float(sig[g]),
                                     int(sizes[g]), synth.LSF_SIGMA, synth.WAVE_RES)

    plain_fwd_ms = _time_steps(plain_loop, 1, 0)
    with torch.no_grad():
        c0 = b.render(*args)
        target = (c0 * 1.05).contiguous()
        weight = 1.0 / ((target / 20.0) ** 2 + 1e-6 * float(target.abs().max()) ** 2)
        del c0
    graph, _ = b.capture(b.forward_backward, *args, target, weight, False, warmup=1)
    fb_ms = _time_steps(graph.replay, steps, 1)
    del graph
    torch.cuda.empty_cache()
    loop_fb_ms = _time_steps(
        lambda: ragged.forward_backward_per_galaxy(b, *args, target, weight), 1, 1)

    # forward + backward of the plain path on a subset (every 16th galaxy), against a
    # ragged batch of the same subset replayed from its own CUDA graph
    sub = np.arange(0, n_gal, 16)
    sub_b = ragged.RaggedBatch(r, counts[sub], sbins[sub], [edges[g] for g in sub], sig[sub],
                               sizes[sub], synth.LSF_SIGMA, synth.WAVE_RES)
    sub_args = tuple(torch.cat([galaxy(g)[k] for g in sub]) for k in range(5))
    sub_t = torch.cat([target[int(b.t.seg_base[g]):int(b.t.seg_base[g + 1])] for g in sub])
    sub_w = torch.cat([weight[int(b.t.seg_base[g]):int(b.t.seg_base[g + 1])] for g in sub])

    def plain_sub_fb():
        for g in sub:
            s0, s1 = int(b.t.seg_base[g]), int(b.t.seg_base[g + 1])
            S = int(sbins[g])
            plain_galaxy_forward_backward(
                r, *galaxy(g), d_edges[g], S, float(sig[g]), int(sizes[g]), synth.LSF_SIGMA,
                synth.WAVE_RES, target[s0:s1].view(S, S, -1), weight[s0:s1].view(S, S, -1))

    plain_sub_fb_ms = _time_steps(plain_sub_fb, 1, 1)
    g_sub, _ = sub_b.capture(sub_b.forward_backward, *sub_args, sub_t, sub_w, False, warmup=1)
    sub_fb_ms = _time_steps(g_sub.replay, steps, 1)
    del g_sub
    torch.cuda.empty_cache()
    autotune.set_tuning(dev.index or 0, None)
    return {"metric": "ragged mocks/s (galaxies rendered per second)",
            "fwd_value": n_gal / (fwd_ms * 1e-3), "fwd_bwd_value": n_gal / (fb_ms * 1e-3),
            "unit": "galaxies/s", "fwd_ms": fwd_ms, "fwd_bwd_ms": fb_ms,
            "plain_gpu_loop_fwd_ms": plain_fwd_ms,
            "speedup_fwd_vs_plain_gpu_loop": plain_fwd_ms / fwd_ms,
            "subset_fwd_bwd": {
                "galaxies": int(sub.size), "particles": int(counts[sub].sum()),
                "plain_gpu_loop_ms": plain_sub_fb_ms, "ragged_graph_ms": sub_fb_ms,
                "speedup_vs_plain_gpu_loop": plain_sub_fb_ms / sub_fb_ms,
                "plain_path": "torch autograd of the plain path, per galaxy, the backward "
                              "recomputed per chunk of 65536 particles"},
            "per_galaxy_loop_fwd_ms": loop_fwd_ms, "per_galaxy_loop_fwd_bwd_ms": loop_fb_ms,
            "speedup_fwd": loop_fwd_ms / fwd_ms, "speedup_fwd_bwd": loop_fb_ms / fb_ms,
            "autotune": {"best_chunk_big_item": list(tune["best"]),
                         "times_ms": {f"{c[0]}/{c[1]}": t for c, t in tune["times_ms"].items()}},
            "batch": f"{n_gal} galaxies, {int(counts.sum())} particles, "
                     f"{b.n_segments} spaxels x {b.L} wavelengths, PSF sigma 0.8-2.0 "
                     f"(kernels up to {b.m}x{b.m}), LSF sigma {synth.LSF_SIGMA} A"}


def ifu_bench(dev, steps, warmup, flush):
    """The 10^6-particle IFU workload (150 x 150 x 3721 cube): the same forward step as
    the main line (device time, inputs resident, L2 flushed) and the fused accumulate
    launch inside it."""
    import torch

    from rubix_gb300 import synth
    from rubix_gb300.api import IFURenderer

    w = synth.make_workload("ifu", edge_cases=False)
    p = w.particles
    rnd = IFURenderer.from_workload(w, device=dev)
    d_in = [torch.from_numpy(a).to(dev) for a in (p.coords, p.velocity, p.mass, p.metallicity,
                                                   p.age)]
    acc = []

    def step():
        idx, mask = rnd.assign(d_in[0])
        perm, offs = rnd.sort(idx, mask)
        e0, e1 = _events()
        e0.record()
        cube = rnd.accumulate(d_in[2], d_in[3], d_in[4], d_in[1], perm, offs, with_lsf=True)
        e1.record()
        acc.append((e0, e1))
        return rnd.noise_(rnd.psf(cube))

    ms = _time_steps(step, steps, warmup, flush)
    torch.cuda.synchronize()
    acc_ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in acc[-steps:])
    N, L = p.n, int(w.wave_t.size)
    return {"metric": "particles*lambda/s, particle->IFU datacube forward",
            "value": N * L / (ms * 1e-3), "unit": "particle*lambda/s", "ms_per_step": ms,
            "accumulate_ms": acc_ms, "workload": workload_config(w)["workload"]}


def summary_block(line):
    """The headline figures of the line in one short object, printed last (so that the
    end of the line, which log tails keep, carries them)."""
    def get(*keys):
        d = line
        for k in keys:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d

    return {
        "workload": (get("config", "workload") or "").split(":")[0],
        "value": get("value"), "ms_per_step": get("ms_per_step"),
        "e2e_value": get("e2e", "value"), "e2e_ms_per_step": get("e2e", "ms_per_step"),
        "accumulate_ms": get("roofline", "ms_per_launch"),
        "accumulate_hbm_frac": get("roofline", "frac"),
        "accumulate_issue_frac": get("roofline", "issue", "frac"),
        "step_hbm_frac": get("roofline", "step", "frac"),
        "cpu_baseline_value": get("cpu_baseline", "value"),
        "ifu_ms_per_step": get("ifu", "ms_per_step"),
        "fwd_bwd_over_fwd": get("fwd_bwd", "fwd_bwd_over_fwd"),
        "ours_over_plain_gpu": get("plain_gpu", "ours_over_plain"),
        "fwd_bwd_ours_over_plain_gpu": get("plain_gpu_fwd_bwd", "ours_over_plain"),
        "ragged_fwd_vs_plain_gpu_loop": get("ragged", "speedup_fwd_vs_plain_gpu_loop"),
        "ragged_fwd_bwd_vs_plain_gpu_loop": get("ragged", "subset_fwd_bwd",
                                                "speedup_vs_plain_gpu_loop"),
        "ragged_fwd_vs_own_kernel_loop": get("ragged", "speedup_fwd"),
        "ragged_fwd_bwd_vs_own_kernel_loop": get("ragged", "speedup_fwd_bwd"),
        "psf_ms": get("psf", "ms"),
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
                            seed=rdist.rank_seed(synth.WORKLOADS[args.workload]["seed"], rank),
                            n_wave_ssp=args.ssp_wave)
    p = w.particles
    N, L = p.n, int(w.wave_t.size)
    S2 = w.sbin * w.sbin
    dusty = args.dust > 0
    rnd = IFURenderer.from_workload(w, device=dev, dust={"extinction_model": "Cardelli89",
                                                         "Rv": 3.1} if dusty else None)
    d_in = [torch.from_numpy(a).to(dev) for a in (p.coords, p.velocity, p.mass, p.metallicity, p.age)]
    gas = None
    if dusty:
        g = synth.make_gas(args.dust, seed=rdist.rank_seed(2, rank))
        gas = tuple(torch.from_numpy(a).to(dev) for a in (g.coords, g.mass, g.metals))
        args.no_e2e = True
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def barrier():
        if world > 1:
            dist.barrier()

    def step_device(ev=None):
        idx, mask = rnd.assign(d_in[0])
        perm, offs = rnd.sort(idx, mask)
        av = rnd.dust_av(d_in[0], idx, *gas) if dusty else None
        if ev is not None:
            ev[0].record()
        cube = rnd.accumulate(d_in[2], d_in[3], d_in[4], d_in[1], perm, offs, with_lsf=True,
                              dust_av=av)
        if ev is not None:
            ev[1].record()
        return rnd.noise_(rnd.psf(cube))

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

        # single render, host to host, nothing overlapped: the latency of one step
        for _ in range(2):
            step_e2e()
        torch.cuda.synchronize()
        barrier()
        lat_ms = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            step_e2e()
            e1.record()
            torch.cuda.synchronize()
            lat_ms.append(e0.elapsed_time(e1))

        # K renders back to back through IFURenderer.host_stream: every step uploads its
        # particles from pinned memory and downloads its cube into a pinned buffer; the
        # copies of one step overlap the compute of the next (two device slots)
        hs = rnd.host_stream(2)
        h_outs = [h_out, torch.empty_like(h_out).pin_memory()]
        for k in range(2):
            hs.submit(*h_in, out=h_outs[k % 2])
        hs.synchronize()
        torch.cuda.synchronize()
        barrier()
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for k in range(args.steps):
            hs.submit(*h_in, out=h_outs[k % 2])
        hs.synchronize()
        e1.record()
        torch.cuda.synchronize()
        te_ms = rdist.max_over_ranks(e0.elapsed_time(e1))
        e2e = {"value": world * N * L * args.steps / (te_ms * 1e-3),
               "unit": "particle*lambda/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": te_ms / args.steps,
               "pipelining": "IFURenderer.host_stream: upload/compute/download on three "
                             "streams, two device slots, K steps back to back",
               "single_step_latency_ms": statistics.mean(lat_ms),
               "single_step_value": world * N * L / (statistics.mean(lat_ms) * 1e-3)}

    # ---------------- roofline of the dominant kernel (rubix_cube_fwd)
    peak, peak_kind = hbm_peak()
    flux_bytes = w.ssp.flux.size * 4
    alg_bytes = 20 * N + flux_bytes + S2 * L * 4   # particle fields + perm, SSP flux, cube write
    cube_avg_s = statistics.mean(cube_ms) * 1e-3
    achieved = alg_bytes / cube_avg_s / 1e9
    traffic = traffic_per_launch(N, w.name)
    fpl = flops_per_particle_lambda(w)
    fp32_peak = fp32_peak_tflops(dev)
    fp32_achieved = fpl * N * L / cube_avg_s / 1e12
    compute = {"fp32_peak_tflops": fp32_peak, "peak_source": "measured FMA-chain probe "
               "(bench_fma_probe.cu)", "achieved_tflops": fp32_achieved,
               "frac": fp32_achieved / fp32_peak if fp32_peak else None,
               "flops_per_particle_lambda": fpl}
    # instruction issue, the resource the main kernel is bound by: warp instructions per
    # launch (ncu count, scaled to N) over the launch time, against one instruction per
    # cycle per scheduler (4 per SM) at the SM clock sampled during the timed region
    insts = instructions_per_launch(N, w.name) if not dusty else None  # dust-free kernel
    issue = None
    if insts:
        sm_mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz") or 2070.0
        n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
        peak_issue = n_sm * 4 * sm_mhz * 1e6
        issue = {"warp_instructions_per_launch": insts, "achieved_per_s": insts / cube_avg_s,
                 "peak_per_s": peak_issue, "frac": insts / cube_avg_s / peak_issue,
                 "source": f"smsp__inst_executed.sum of profiles/cube_fwd_{w.name}.txt scaled to "
                           f"{N} particles; peak = {n_sm} SMs x 4 schedulers x 1 warp "
                           f"instruction per cycle at {sm_mhz:.0f} MHz"}
    roofline = {"kernel": "rubix_cube_fwd (fused lookup/mass/Doppler/resample/accumulate)",
                "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": traffic, "algorithmic_bytes": alg_bytes, "issue": issue,
                "ms_per_launch": statistics.mean(cube_ms),
                "share_of_step": statistics.mean(cube_ms) / statistics.mean(step_ms),
                "fp32": compute}
    # the whole step against the path's algorithmic traffic 24 N + |T| + 5 C (particle
    # fields read once, SSP flux once, cube written by the accumulate, PSF read + write,
    # LSF read + write)
    step_bytes = 24 * N + flux_bytes + 5 * S2 * L * 4
    step_gbs = step_bytes / (statistics.mean(step_ms) * 1e-3) / 1e9
    roofline["step"] = {"algorithmic_bytes": step_bytes, "achieved": step_gbs, "peak": peak,
                        "unit": "GB/s", "frac": step_gbs / peak,
                        "ms_per_step": statistics.mean(step_ms)}

    # ---------------- CPU baseline (rank 0, N=1): oracle port on the host cores, an
    # estimated step from bounded samples of every stage
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import multiprocessing as mp

        cores = os.cpu_count() or 1
        n_sample = 2048 * cores
        with mp.get_context("spawn").Pool(cores) as pool:
            run_oracle_sample(w, 512, pool)
            t_cpu, parts = cpu_step_estimate(w, pool, n_sample)
        cpu = {"value": N * L / t_cpu, "unit": "particle*lambda/s", "cores": cores,
               "kind": "port", "sample": cpu_sample_text(w, n_sample, cores),
               "ms_per_step": 1e3 * t_cpu, "stages_s": parts,
               "reference_design": "rubix materialises the N x L resampled spectra "
                                   "(rubix/core/ifu.py:278-283): %.0f GB for this workload"
                                   % (4.0 * N * L / 1e9)}

    # ---------------- fwd+bwd, plain GPU path and ragged batch (rank 0, N=1)
    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        ours_final = step_device()
        for name, fn in (
                ("ifu", lambda: ifu_bench(dev, args.steps, 3, flush)),
                ("fwd_bwd", lambda: fwd_bwd_bench(dev, min(args.steps, 5), 3, flush)),
                ("plain_gpu", lambda: plain_bench(dev, w, rnd, d_in, ours_final, args.steps,
                                                  args.warmup, flush)),
                ("plain_gpu_fwd_bwd", lambda: plain_fwd_bwd_bench(dev, args.steps, 1)),
                ("dusty", lambda: dusty_bench(dev, w, d_in, args.steps, 3, flush)),
                ("fits_layout", lambda: fits_bench(dev, ours_final, args.steps, 3, flush)),
                ("noise", lambda: noise_bench(dev, ours_final, args.steps, 3, flush)),
                ("galaxy_file", lambda: galaxy_file_bench(dev, w, 3)),
                ("pipeline_api", lambda: pipeline_bench(dev, w, min(args.steps, 5), 3, flush)),
                ("ragged", lambda: ragged_bench(dev, 3, 2))):
            if args.extras is not None and name not in args.extras.split(","):
                continue
            try:
                extras[name] = fn()
            except Exception as exc:  # report and keep the main line
                extras[name] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
            torch.cuda.empty_cache()
        del ours_final
        if "value" in extras.get("plain_gpu", {}):
            extras["plain_gpu"]["ours_over_plain"] = value / extras["plain_gpu"]["value"]
        if "value" in extras.get("plain_gpu_fwd_bwd", {}) and "value" in extras.get("fwd_bwd", {}):
            extras["plain_gpu_fwd_bwd"]["ours_over_plain"] = (
                extras["fwd_bwd"]["value"] / extras["plain_gpu_fwd_bwd"]["value"])

    if rank == 0:
        cfg = workload_config(w)
        if dusty:
            cfg["path"] = cfg["path"].replace("mask+assign+sort", "mask+assign+sort -> A_V "
                                              f"of every star from {args.dust} gas cells")
            cfg["dust"] = "Cardelli89, R_V 3.1, broken power-law dust-to-gas ratio (X_CO = Z)"
        line = {
            "metric": "particles*lambda/s, particle->IFU datacube forward"
                      + (" with dust extinction" if dusty else ""),
            "value": value, "unit": "particle*lambda/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": statistics.mean(step_ms),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded exponential disk; synthetic SSP grid)",
            "config": cfg, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches, "clocks": clocks, "wall_s_timed": wall,
        }
        line.update(extras)
        line["summary"] = summary_block(line)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
