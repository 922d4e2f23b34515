"""Regenerates the golden fixtures of this directory from the oracle.

    python tests/golden/make_golden.py

small_n300_L64.npz: the calc_ifu chain (filter -> assignment -> lookup -> mass ->
Doppler/resample -> cube -> PSF -> LSF) of the oracle on the first 300 particles of the
"small" workload (plus its 14 edge-case particles) and the first 64 telescope
wavelengths.  The inputs are regenerated by rubix_gb300.synth (seeded); the file keeps
the oracle's outputs (the raw cube in float64, the final cube rounded to float32) so
that kernels and oracle are checked against fixed numbers.
These are oracle outputs, not outputs of the reference (which cannot run here).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from rubix_gb300 import synth  # noqa: E402

N, NT = 300, 64


def stages():
    w = synth.make_workload("small", n=N, n_wave_t=NT)
    p = w.particles
    out = oracle.render_cube(p.coords, p.velocity, p.mass, p.metallicity, p.age, w.edges,
                             w.sbin, w.ssp.metallicity, w.ssp.age, w.ssp.flux,
                             w.ssp.wavelength, w.dist_z, w.wave_t, psf_size=w.psf_size,
                             psf_sigma=w.psf_sigma, lsf_sigma=w.lsf_sigma, wave_res=w.wave_res)
    return w, out


if __name__ == "__main__":
    w, out = stages()
    path = os.path.join(HERE, "small_n300_L64.npz")
    np.savez_compressed(path, pixel_assignment=out["pixel_assignment"].astype(np.int32),
                        mask=out["mask"], cube=out["cube"],
                        final=out["final"].astype(np.float32))
    print(path, os.path.getsize(path), "bytes")
