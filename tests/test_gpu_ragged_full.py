"""The 256-galaxy ragged batch at full size (the batch the benchmark times).

256 galaxies with particle counts log-uniform in [1e3, 1e6] (about 4.6e7 particles),
square spaxel grids of 16^2 to 64^2, the shared 3721-bin telescope grid, per-galaxy PSF
sigma uniform in [0.8, 2.0] spaxel, SSP grid 221 x 6 x 1221.  Checked:
* every galaxy's final cube bit-identical to its own single-galaxy launches;
* the accumulated cubes of the three largest galaxies against the float64 oracle on
  sampled spaxels (the two densest and six random non-empty ones of each), and the
  PSF + LSF of the largest galaxy against the oracle's convolutions on a window around
  its densest spaxel (rubix/core/ifu.py:63-341, rubix/telescope/psf/psf.py:33-58,
  rubix/telescope/lsf/lsf.py:29-105);
* forward + backward replayed from a captured CUDA graph bit-identical to the eager run.
"""

import numpy as np
import pytest

import oracle
from helpers import CUBE_RTOL, to_dev

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def full_batch(rubix_lib):
    from rubix_gb300 import ragged, synth
    from rubix_gb300 import telescope as tel
    from rubix_gb300.api import IFURenderer

    counts, sbins, sig, sizes = ragged.synthetic_batch_spec()
    ssp = synth.make_ssp(221, 6, 1221, seed=2)
    wave_t = tel.calculate_wave_seq(synth.WAVE_RANGE, synth.WAVE_RES)
    edges = [ragged.galaxy_edges(int(s), synth.DIST_Z) for s in sbins]
    gals = [synth.make_galaxy(int(n), seed=1000 + g) for g, n in enumerate(counts)]
    r = IFURenderer(ssp.age, ssp.metallicity, ssp.wavelength, ssp.flux, wave_t, edges[0],
                    int(sbins[0]), synth.DIST_Z)
    b = ragged.RaggedBatch(r, counts, sbins, edges, sig, sizes, synth.LSF_SIGMA,
                           synth.WAVE_RES)
    d = [to_dev(np.concatenate([getattr(p, k) for p in gals]))
         for k in ("coords", "velocity", "mass", "metallicity", "age")]
    return dict(b=b, ssp=ssp, wave_t=wave_t, edges=edges, gals=gals, counts=counts,
                sbins=sbins, sig=sig, sizes=sizes, args=tuple(d))


def test_full_batch_equals_single_galaxy_launches(full_batch):
    import torch

    from rubix_gb300 import ragged

    b, args = full_batch["b"], full_batch["args"]
    batched = b.render(*args)
    looped = ragged.render_per_galaxy(b, *args)
    torch.cuda.synchronize()
    bad = [g for g in range(b.n_gal)
           if not torch.equal(b.galaxy_view(batched, g), b.galaxy_view(looped, g))]
    print(f"ragged batch: {b.n_gal} galaxies, {int(full_batch['counts'].sum())} particles, "
          f"{b.n_segments} spaxels; galaxies differing from their own launches: {len(bad)}")
    assert not bad


def test_largest_galaxies_vs_oracle(full_batch):
    from oracle import pool

    b, args = full_batch["b"], full_batch["args"]
    ssp, wave_t = full_batch["ssp"], full_batch["wave_t"]
    L = wave_t.size
    wave_z = oracle.cosmological_doppler_shift(0.1, ssp.wavelength)
    idx, keep = b.assign(args[0])
    perm, offs = b.sort(idx, keep)
    raw = b.accumulate(args[2], args[3], args[4], args[1], perm, offs, with_lsf=False)
    rng = np.random.default_rng(11)
    groups, rows = [], []
    for g in np.argsort(-full_batch["counts"], kind="stable")[:3]:
        p, e, S = full_batch["gals"][g], full_batch["edges"][g], int(full_batch["sbins"][g])
        li = oracle.square_spaxel_assignment(p.coords, e)
        # flat ids use len(edges) - 1 columns, which can exceed S; ids >= S^2 are dropped
        inside = oracle.mask_particles_outside_aperture(p.coords, e) & (li < S * S)
        c = np.bincount(li[inside], minlength=S * S)
        dense = np.argsort(-c, kind="stable")[:2]
        rest = np.setdiff1d(np.nonzero(c)[0], dense)
        for s in np.concatenate([dense, rng.choice(rest, 6, replace=False)]):
            j = np.nonzero(inside & (li == s))[0]
            groups.append((p.mass[j], p.metallicity[j], p.age[j], p.velocity[j, 2]))
            rows.append(int(b.t.seg_base[g]) + int(s))
    want = pool.spaxel_spectra(groups, ssp.metallicity, ssp.age, ssp.flux, wave_z, wave_t)
    got = raw.view(-1, L)[to_dev(np.asarray(rows, dtype=np.int64))].cpu().numpy()
    norm, elem = oracle.cube_rel_error(got, want)
    per = max(float(np.abs(a - w).max() / np.abs(w).max()) for a, w in zip(got, want))
    print(f"ragged, 3 largest galaxies, {len(rows)} spaxels "
          f"({sum(len(x[0]) for x in groups)} particles): normwise {norm:.2e}, elementwise "
          f"{elem:.2e}, worst per-spaxel normwise {per:.2e}")
    assert norm <= CUBE_RTOL and elem <= CUBE_RTOL and per <= CUBE_RTOL

    # PSF + LSF of the largest galaxy around its densest spaxel
    g = int(np.argmax(full_batch["counts"]))
    S, m, sg = int(full_batch["sbins"][g]), int(full_batch["sizes"][g]), float(full_batch["sig"][g])
    final = b.galaxy_view(b.psf(b.lsf(raw)), g)
    h = (m - 1) // 2
    cy, cx = divmod(rows[0] - int(b.t.seg_base[g]), S)
    y0, x0 = max(cy - 2 * h, 0), max(cx - 2 * h, 0)
    y1, x1 = min(cy + 2 * h + 1, S), min(cx + 2 * h + 1, S)
    win = b.galaxy_view(raw, g)[y0:y1, x0:x1].cpu().numpy().astype(np.float64)
    ref = oracle.apply_lsf(oracle.apply_psf(win, oracle.gaussian_kernel_2d(m, m, sg)), 1.2, 1.25)
    # compare where the window's cut edges (not the galaxy's own edges) are out of reach
    ys = slice(0 if y0 == 0 else h, (y1 - y0) if y1 == S else (y1 - y0) - h)
    xs = slice(0 if x0 == 0 else h, (x1 - x0) if x1 == S else (x1 - x0) - h)
    norm, elem = oracle.cube_rel_error(final[y0:y1, x0:x1].cpu().numpy()[ys, xs], ref[ys, xs])
    print(f"ragged, largest galaxy PSF {m}x{m} sigma {sg:.3f} + LSF window: normwise "
          f"{norm:.2e}, elementwise {elem:.2e}")
    assert norm <= CUBE_RTOL and elem <= CUBE_RTOL


def test_full_batch_graph_replay_equals_eager(full_batch):
    import torch

    b, args = full_batch["b"], full_batch["args"]
    with torch.no_grad():
        c0 = b.render(*args)
        target = (c0 * 1.05).contiguous()
        weight = 1.0 / ((target / 20.0) ** 2 + 1e-6 * float(target.abs().max()) ** 2)
        del c0
    eager = b.forward_backward(*args, target, weight)
    eager = (eager[0].clone(), [x.clone() for x in eager[1]], eager[2].clone(),
             eager[3].clone(), eager[4].clone())
    graph, out = b.capture(b.forward_backward, *args, target, weight, warmup=1)
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(out[4], eager[4])
    for a, c in zip(out[1], eager[1]):
        assert torch.equal(a, c)
    assert torch.equal(out[2], eager[2]) and torch.equal(out[3], eager[3])
    assert torch.equal(out[0], eager[0])
