"""Seeded synthetic inputs with the shapes and distributions of the benchmark workloads.

No simulation snapshots or SSP template files are available, so every workload is
generated from a fixed ``numpy.random.Generator(PCG64(seed))``:

* SSP grid: ages log-spaced in [0.1, 13.5] Gyr, metallicities log-spaced in
  [1e-4, 0.05], wavelengths uniform in [3000, 10000] A; flux = smooth power-law
  continuum whose slope and level change with age and metallicity, times seeded
  Gaussian absorption lines; strictly positive float32, layout [Z, age, lambda].
* Stellar disk: exponential radial profile (scale length R_d), exponential vertical
  profile (h_z), flat rotation curve plus Gaussian line-of-sight dispersion,
  inclined about the x axis so rotation projects onto the line of sight (z).
  Optional Plummer bulge.  Ages log-uniform 0.1-13.5 Gyr, metallicity log-uniform
  1e-4-0.05, masses log-normal (median 1e5 Msun).
* Edge cases appended on request: particles exactly on interior and outer spaxel
  edges, outside the field of view, ages/metallicities on grid nodes and outside
  the grid, zero mass.
* Gas disk (for dust extinction): exponential in R and z, log-normal masses, metal
  mass fractions with 12 + log(O/H) spread around solar.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import telescope as tel


@dataclass
class SSPData:
    age: np.ndarray          # [n_age] Gyr
    metallicity: np.ndarray  # [n_met]
    wavelength: np.ndarray   # [n_wave] Angstrom (rest frame)
    flux: np.ndarray         # [n_met, n_age, n_wave]


@dataclass
class ParticleData:
    coords: np.ndarray    # [n, 3] kpc
    velocity: np.ndarray  # [n, 3] km/s
    mass: np.ndarray      # [n] Msun
    metallicity: np.ndarray
    age: np.ndarray       # Gyr

    @property
    def n(self) -> int:
        return int(self.mass.shape[0])


def make_ssp(n_age: int, n_met: int, n_wave: int, seed: int = 0, n_lines: int = 48) -> SSPData:
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    age = np.geomspace(0.1, 13.5, n_age).astype(np.float32)
    met = np.geomspace(1e-4, 0.05, n_met).astype(np.float32)
    wave = np.linspace(3000.0, 10000.0, n_wave).astype(np.float32)
    la = np.log10(age.astype(np.float64) / 0.1) / np.log10(135.0)          # 0..1
    lz = np.log10(met.astype(np.float64) / 1e-4) / np.log10(500.0)          # 0..1
    x = wave.astype(np.float64) / 5500.0
    slope = -2.5 + 3.0 * la[None, :, None] + 0.5 * lz[:, None, None]
    level = 1e-3 * (age.astype(np.float64)[None, :, None] ** -0.8) * (1.0 + 0.3 * lz[:, None, None])
    cont = level * x[None, None, :] ** slope
    centers = rng.uniform(3000.0, 10000.0, n_lines)
    widths = rng.uniform(2.0, 8.0, n_lines)
    depth0 = rng.uniform(0.05, 0.45, n_lines)
    absorb = np.ones((n_met, n_age, n_wave))
    for c, w, d in zip(centers, widths, depth0):
        depth = d * (0.3 + 0.7 * la[None, :, None]) * (0.5 + 0.5 * lz[:, None, None])
        absorb *= 1.0 - depth * np.exp(-0.5 * ((wave[None, None, :] - c) / w) ** 2)
    flux = (cont * absorb).astype(np.float32)
    return SSPData(age=age, metallicity=met, wavelength=wave, flux=flux)


def make_galaxy(n: int, seed: int = 0, R_d: float = 3.0, h_z: float = 0.3, v_rot: float = 200.0,
                sigma_los: float = 50.0, inclination_deg: float = 60.0, bulge_frac: float = 0.0,
                bulge_a: float = 1.0, bulge_sigma: float = 120.0) -> ParticleData:
    rng = np.random.Generator(np.random.PCG64(seed))
    nb = int(round(n * bulge_frac))
    nd = n - nb
    # disk (disk frame: z is the rotation axis)
    R = rng.gamma(2.0, R_d, nd)
    phi = rng.uniform(0.0, 2.0 * np.pi, nd)
    zz = rng.laplace(0.0, h_z, nd)
    pos = np.stack([R * np.cos(phi), R * np.sin(phi), zz], axis=1)
    vel = np.stack([-v_rot * np.sin(phi), v_rot * np.cos(phi), np.zeros(nd)], axis=1)
    if nb > 0:
        u = rng.uniform(1e-6, 1.0, nb)
        r = bulge_a / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        r = np.minimum(r, 50.0 * bulge_a)
        d = rng.normal(size=(nb, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        pos = np.concatenate([pos, r[:, None] * d])
        vel = np.concatenate([vel, rng.normal(0.0, bulge_sigma, (nb, 3))])
    inc = np.deg2rad(inclination_deg)
    rot = np.array([[1, 0, 0], [0, np.cos(inc), -np.sin(inc)], [0, np.sin(inc), np.cos(inc)]])
    pos = pos @ rot.T
    vel = vel @ rot.T
    vel[:, 2] += rng.normal(0.0, sigma_los, n)
    age = np.exp(rng.uniform(np.log(0.1), np.log(13.5), n))
    met = np.exp(rng.uniform(np.log(1e-4), np.log(0.05), n))
    mass = 1e5 * np.exp(rng.normal(0.0, 0.5, n))
    perm = rng.permutation(n)
    return ParticleData(coords=pos[perm].astype(np.float32), velocity=vel[perm].astype(np.float32),
                        mass=mass[perm].astype(np.float32), metallicity=met[perm].astype(np.float32),
                        age=age[perm].astype(np.float32))


@dataclass
class GasData:
    coords: np.ndarray  # [n, 3] kpc
    mass: np.ndarray    # [n] Msun
    metals: np.ndarray  # [n, 10] mass fractions: H, He, C, N, O, Ne, Mg, Si, Fe, total

    @property
    def n(self) -> int:
        return int(self.mass.shape[0])


def make_gas(n: int, seed: int = 0, R_d: float = 3.0, h_z: float = 0.15,
             inclination_deg: float = 60.0, median_mass: float = 3e4) -> GasData:
    """A gas disk for the dust step: exponential in R (scale R_d) and z (h_z), inclined
    like the stellar disk; log-normal masses; hydrogen mass fraction 0.74 and oxygen
    log-uniform in [1e-3, 2e-2] (12 + log(O/H) between about 7.9 and 9.2)."""
    rng = np.random.Generator(np.random.PCG64(5000 + seed))
    R = rng.gamma(2.0, R_d, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    zz = rng.laplace(0.0, h_z, n)
    pos = np.stack([R * np.cos(phi), R * np.sin(phi), zz], axis=1)
    inc = np.deg2rad(inclination_deg)
    rot = np.array([[1, 0, 0], [0, np.cos(inc), -np.sin(inc)], [0, np.sin(inc), np.cos(inc)]])
    pos = pos @ rot.T
    mass = median_mass * np.exp(rng.normal(0.0, 0.5, n))
    metals = np.zeros((n, 10))
    metals[:, 0] = 0.74
    metals[:, 1] = 0.25
    metals[:, 4] = np.exp(rng.uniform(np.log(1e-3), np.log(2e-2), n))
    metals[:, 2] = 0.2 * metals[:, 4]
    metals[:, 9] = 1.0 - metals[:, 0] - metals[:, 1]
    return GasData(coords=pos.astype(np.float32), mass=mass.astype(np.float32),
                   metals=metals.astype(np.float32))


def append_edge_cases(p: ParticleData, edges: np.ndarray, ssp: SSPData) -> ParticleData:
    """Append particles on spaxel edges, outside the field, on/outside SSP grid nodes."""
    e = np.asarray(edges, dtype=np.float32)
    mid = e[len(e) // 2]
    rows = []
    def add(x, y, z, age, met, mass, vz=0.0):
        rows.append((x, y, z, vz, age, met, mass))
    a0, a1 = float(ssp.age[0]), float(ssp.age[-1])
    z0, z1 = float(ssp.metallicity[0]), float(ssp.metallicity[-1])
    am, zm = float(ssp.age[len(ssp.age) // 2]), float(ssp.metallicity[len(ssp.metallicity) // 2])
    add(mid, mid, 0.0, am, zm, 1e5)                 # exactly on an interior edge (both axes)
    add(e[0], e[0], 0.0, am, zm, 1e5)               # on the lower outer edge
    add(e[-1], e[-1], 0.0, am, zm, 1e5)             # on the upper outer edge
    add(e[1], e[-2], 0.0, am, zm, 1e5)              # on interior edges
    add(e[-1] * 1.5, 0.0, 0.0, am, zm, 1e5)         # outside the field
    add(0.0, e[0] * 2.0, 0.0, am, zm, 1e5)          # outside the field
    add(0.1 * mid, 0.0, 0.0, a0, z0, 1e5)           # on the lowest grid nodes
    add(0.0, 0.1 * mid, 0.0, a1, z1, 1e5)           # on the highest grid nodes
    add(0.0, 0.0, 0.0, am, zm, 1e5, 300.0)          # on interior grid nodes, receding
    add(0.0, 0.0, 0.0, a1 * 1.5, zm, 1e5)           # older than the grid -> zero spectrum
    add(0.0, 0.0, 0.0, am, z1 * 2.0, 1e5)           # more metal-rich than the grid
    add(0.0, 0.0, 0.0, am, z0 * 0.5, 1e5)           # more metal-poor than the grid
    add(0.0, 0.0, 0.0, am, zm, 0.0)                 # zero mass
    add(0.0, 0.0, 0.0, am, zm, 1e5, -900.0)         # large approaching velocity
    r = np.array(rows, dtype=np.float64)
    coords = np.concatenate([p.coords, r[:, 0:3].astype(np.float32)])
    vel_e = np.zeros((len(rows), 3), dtype=np.float32)
    vel_e[:, 2] = r[:, 3]
    return ParticleData(
        coords=coords, velocity=np.concatenate([p.velocity, vel_e]),
        mass=np.concatenate([p.mass, r[:, 6].astype(np.float32)]),
        metallicity=np.concatenate([p.metallicity, r[:, 5].astype(np.float32)]),
        age=np.concatenate([p.age, r[:, 4].astype(np.float32)]),
    )


# Workloads: the plain-forward, differentiation and large configurations.
WORKLOADS = {
    "small": dict(n=10_000, ssp=(20, 6, 1000), fov=5.0, psf_size=11, psf_sigma=1.0, seed=1),
    "ifu": dict(n=1_000_000, ssp=(221, 6, 1221), fov=30.0, psf_size=15, psf_sigma=1.5, seed=2),
    "diff": dict(n=200_000, ssp=(221, 6, 1221), fov=10.0, psf_size=15, psf_sigma=1.5, seed=3),
    "large": dict(n=10_000_000, ssp=(221, 6, 1221), fov=60.0, psf_size=15, psf_sigma=1.5,
                  seed=5, bulge_frac=0.3, noise_s2n=20.0),
}
SPATIAL_RES = 0.2   # arcsec per spaxel (MUSE)
DIST_Z = 0.1
LSF_SIGMA = 1.2     # Angstrom
WAVE_RANGE = (4700.15, 9351.4)
WAVE_RES = 1.25


@dataclass
class Workload:
    name: str
    particles: ParticleData
    ssp: SSPData
    edges: np.ndarray
    sbin: int
    wave_t: np.ndarray
    wave_z: np.ndarray
    psf_size: int
    psf_sigma: float
    lsf_sigma: float
    wave_res: float
    dist_z: float
    noise_s2n: float | None = None  # Gaussian noise at this S/N after PSF and LSF


def make_workload(name: str, n: int | None = None, edge_cases: bool = True,
                  n_wave_t: int | None = None, seed: int | None = None,
                  n_wave_ssp: int | None = None) -> Workload:
    """Build a named workload; ``n`` overrides the particle count, ``n_wave_t`` truncates
    the telescope grid (for fast CPU checks), ``seed`` the particle seed, ``n_wave_ssp``
    the number of SSP wavelengths."""
    cfg = dict(WORKLOADS[name])
    if seed is not None:
        cfg["seed"] = seed
    n_age, n_met, n_wave = cfg["ssp"]
    if n_wave_ssp is not None:
        n_wave = int(n_wave_ssp)
    ssp = make_ssp(n_age, n_met, n_wave, seed=WORKLOADS[name]["seed"])
    sbin = int(np.floor(cfg["fov"] / SPATIAL_RES))
    edges, _ = tel.spatial_bin_edges(cfg["fov"], sbin, DIST_Z)
    gal = make_galaxy(cfg["n"] if n is None else n, seed=cfg["seed"],
                      bulge_frac=cfg.get("bulge_frac", 0.0))
    if edge_cases:
        gal = append_edge_cases(gal, edges, ssp)
    wave_t = tel.calculate_wave_seq(WAVE_RANGE, WAVE_RES)
    if n_wave_t is not None:
        wave_t = wave_t[:n_wave_t]
    return Workload(name=name, particles=gal, ssp=ssp, edges=edges, sbin=sbin, wave_t=wave_t,
                    wave_z=tel.cosmological_doppler_shift(DIST_Z, ssp.wavelength),
                    psf_size=cfg["psf_size"], psf_sigma=cfg["psf_sigma"], lsf_sigma=LSF_SIGMA,
                    wave_res=WAVE_RES, dist_z=DIST_Z, noise_s2n=cfg.get("noise_s2n"))
