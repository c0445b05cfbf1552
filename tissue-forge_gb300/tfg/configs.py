"""Seeded synthetic workloads for the per-step particle path.

Each generator returns a `Workload`: the space description, particle arrays and the
interaction model (potential factory arguments, fluxes, bonds, angles, per-type
dynamics).  No dataset is involved; all inputs are synthetic with fixed seeds
(numpy PCG64, seed = workload index * 1000 + replica).

Workloads (sizes as used by the benchmark and the parity tests):
  cell_sorting   3D periodic box side 20, cutoff 3 (6^3 cells), 4,000 particles, two types
                 50/50, radius 1, mass 1, shifted Morse a=5 r0=1 [0.01, 3] with depth 3 (A-A,
                 B-B) and 0.5 (A-B), overdamped, dt 0.005, 100 steps.
  dpd_droplets   box side 40, cutoff 1 (40^3 cells), two droplets of radius 12 centred at
                 (10,10,10) and (30,30,30) holding 100,000 particles, Maxwell velocities at
                 kT=1, DPD alpha=10 gamma=4.5 sigma=3, one species S (0 in droplet 1, 1 in
                 droplet 2), Fick k=0.5 between same-type pairs, Newtonian, dt 0.01, 1,000 steps.
  bonded_fluid   2,000,000 particles at number density 0.85 (side 133.0, 53^3 cells), LJ 12-6
                 A=B=1 on [0.1, 2.5], linear chains of 16 (random walks of step 1 from uniform
                 starts), harmonic bonds k=100 r0=1, harmonic angles k=20 theta0=pi, 50
                 overdamped relaxation steps then 500 Newtonian steps at dt 0.002.
  ensemble       256 cell_sorting-style simulations, N log-uniform in [500, 50,000], A-B depth
                 U[0.1, 2.0], box side (N/0.5)^(1/3), Gaussian random force std 0.1, 1,000 steps.
  served_stream  Poisson arrivals at 200 requests/s, 60/40 cell_sorting / dpd_droplets-style,
                 N log-uniform in [1,000, 200,000], steps U[100, 5,000].
"""
import math
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import abi


@dataclass
class PotSpec:
    """Arguments of one reference Potential factory call, or ("table") a potential as the
    reference stores it: kind, flags, alpha, r0_plusone, a, b, n, c (tuples) and dpd."""
    kind: str                  # "morse" | "lj" | "harmonic" | "harmonic_angle" | "dpd" | "table"
    args: dict


@dataclass
class Workload:
    name: str
    origin: tuple
    dim: tuple
    cells: tuple
    cutoff: float
    dt: float
    steps: int
    x: np.ndarray                      # (n,3) float32 global positions
    type: np.ndarray                   # (n,) int32
    v: Optional[np.ndarray] = None     # (n,3) float32
    radius: Optional[np.ndarray] = None
    imass: Optional[np.ndarray] = None
    species: Optional[np.ndarray] = None   # (n, nspec)
    nr_species: int = 0
    max_type: int = 1
    dynamics: List[int] = field(default_factory=lambda: [abi.NEWTONIAN])
    mass: List[float] = field(default_factory=lambda: [1.0])
    pots: dict = field(default_factory=dict)        # (ti,tj) -> PotSpec
    fluxes: list = field(default_factory=list)      # (ti, tj, abi.Flux)
    bond_pot: Optional[PotSpec] = None
    angle_pot: Optional[PotSpec] = None
    bonds: Optional[np.ndarray] = None  # (nb,2) int32
    angles: Optional[np.ndarray] = None  # (na,3) int32
    random_force: Optional[tuple] = None  # (mean, std, duration_steps) for every type
    relax_steps: int = 0               # overdamped steps before the timed dynamics
    flags: int = 0
    seed: int = 0x5EED
    nr_fluxsteps: int = 1
    boundaries: list = field(default_factory=list)  # (wall, kind, velocity, restore, radius)
    wall_pots: list = field(default_factory=list)   # (wall or -1, type, PotSpec)
    # bonded potentials by slot, with each bond's and angle's slot (default: bond_pot in
    # slot 0 for every bond, angle_pot in slot 1 for every angle)
    bonded_pots: list = field(default_factory=list)
    bond_slot: Optional[np.ndarray] = None
    angle_slot: Optional[np.ndarray] = None
    type_forces: list = field(default_factory=list)  # (type, mean, std, duration_steps)
    flags_particles: Optional[np.ndarray] = None      # per-particle flags (frozen axes)
    species_reset: Optional[list] = None              # species values after a RESETTING wall
    force_i: Optional[np.ndarray] = None              # (n,3) external force per particle
    max_dist_fraction: float = 0.05                  # particle_max_dist_fraction

    @property
    def n(self):
        return int(self.x.shape[0])

    def desc(self, capacity=0, device=0):
        nb = 0 if self.bonds is None else len(self.bonds)
        na = 0 if self.angles is None else len(self.angles)
        return abi.engine_desc(self.origin, self.dim, self.cells, self.cutoff, self.dt,
                               max_type=self.max_type, nr_species=self.nr_species,
                               particle_max_dist_fraction=self.max_dist_fraction,
                               seed=self.seed, capacity=capacity or self.n,
                               max_bonds=nb, max_angles=na, device=device, flags=self.flags,
                               nr_fluxsteps=self.nr_fluxsteps)


def in_box(x, side):
    """Wrap positions into the periodic box [0, side) and keep them off its upper face:
    space_setpartp (tfSpace.cpp:443-448) rejects a particle whose clamped coordinate
    rounds to cell index cdim, which FP32 can do within a few ulps of the face."""
    x = np.mod(np.asarray(x, np.float64), side)
    return np.minimum(x, side * (1.0 - 1e-6)).astype(np.float32)


def cells_for(side, cutoff):
    """Cells per axis with edge >= cutoff (span 1): floor(side/cutoff), at least 3."""
    return max(3, int(math.floor(side / cutoff)))


def cell_sorting(n=4000, side=20.0, cutoff=3.0, depth_ab=0.5, steps=100, seed=0, random_force=None):
    rng = np.random.default_rng(np.random.PCG64(seed))
    x = in_box(rng.uniform(0.0, side, size=(n, 3)), side)
    t = np.zeros(n, np.int32)
    t[rng.permutation(n)[: n // 2]] = 1
    c = cells_for(side, cutoff)
    w = Workload(
        name="cell_sorting", origin=(0.0, 0.0, 0.0), dim=(side,) * 3, cells=(c, c, c), cutoff=cutoff,
        dt=0.005, steps=steps, x=x, type=t, radius=np.ones(n, np.float32), imass=np.ones(n, np.float32),
        max_type=2, dynamics=[abi.OVERDAMPED, abi.OVERDAMPED], mass=[1.0, 1.0],
        random_force=random_force, seed=seed * 1000 + 1)
    morse = lambda d: PotSpec("morse", dict(d=d, a=5.0, r0=1.0, min=0.01, max=3.0, tol=0.001, shifted=True))
    w.pots[(0, 0)] = morse(3.0)
    w.pots[(1, 1)] = morse(3.0)
    w.pots[(0, 1)] = morse(depth_ab)
    return w


def dpd_droplets(n=100_000, side=40.0, cutoff=1.0, radius=12.0, steps=1000, seed=1):
    rng = np.random.default_rng(np.random.PCG64(1000 + seed))
    centres = np.array([[side / 4.0] * 3, [3.0 * side / 4.0] * 3])
    pts = []
    drop = []
    for d in range(2):
        m = n // 2 if d == 0 else n - n // 2
        got = np.zeros((0, 3))
        while got.shape[0] < m:
            cand = rng.uniform(-radius, radius, size=(2 * m, 3))
            cand = cand[np.einsum("ij,ij->i", cand, cand) <= radius * radius]
            got = np.concatenate([got, cand])
        pts.append(got[:m] + centres[d])
        drop.append(np.full(m, d, np.int32))
    x = in_box(np.concatenate(pts), side)
    droplet = np.concatenate(drop)
    v = rng.normal(0.0, 1.0, size=(n, 3)).astype(np.float32)   # kT = 1, m = 1
    species = droplet.astype(np.float32).reshape(n, 1)          # 0 in droplet 1, 1 in droplet 2
    c = cells_for(side, cutoff)
    w = Workload(
        name="dpd_droplets", origin=(0.0, 0.0, 0.0), dim=(side,) * 3, cells=(c, c, c), cutoff=cutoff,
        dt=0.01, steps=steps, x=x, type=np.zeros(n, np.int32), v=v, radius=np.ones(n, np.float32),
        imass=np.ones(n, np.float32), species=species, nr_species=1, max_type=1,
        dynamics=[abi.NEWTONIAN], mass=[1.0], seed=1000 + seed)
    w.pots[(0, 0)] = PotSpec("dpd", dict(alpha=10.0, gamma=4.5, sigma=3.0, cutoff=cutoff, shifted=False))
    f = abi.Flux()
    f.kind = abi.FLUX_FICK
    f.type_a = 0
    f.type_b = 0
    f.index_a = 0
    f.index_b = 0
    f.coef = 0.5
    f.decay = 0.0
    f.target = 0.0
    f.cutoff = cutoff
    w.fluxes.append((0, 0, f))
    return w


def dpd_droplets_species(n=100_000, side=40.0, cutoff=1.0, radius=12.0, steps=1000, seed=1):
    """The DPD droplets with three species, each diffusing by Fick (the multi-species flux
    path): the droplet marker of dpd_droplets (k 0.5), a second species from a uniform random
    start (k 0.2) and a third from a uniform 0.25 with decay (k 0.1, decay 0.05).  All
    particles have one type, so only symmetric fluxes are used: a flux whose two sides differ
    (secrete, uptake, or two species indices) between particles of one type acts from the
    pair's first particle to its second, and which is first depends on the order of the
    particles in their cell."""
    w = dpd_droplets(n=n, side=side, cutoff=cutoff, radius=radius, steps=steps, seed=seed)
    rng = np.random.default_rng(np.random.PCG64(1500 + seed))
    s = np.zeros((w.n, 3), np.float32)
    s[:, 0] = w.species[:, 0]
    s[:, 1] = rng.uniform(0.0, 1.0, size=w.n).astype(np.float32)
    s[:, 2] = 0.25
    w.species = s
    w.nr_species = 3
    w.name = "dpd_droplets_species"
    w.fluxes = []
    for kind, ia, ib, coef, decay, target in [(abi.FLUX_FICK, 0, 0, 0.5, 0.0, 0.0),
                                              (abi.FLUX_FICK, 1, 1, 0.2, 0.0, 0.0),
                                              (abi.FLUX_FICK, 2, 2, 0.1, 0.05, 0.0)]:
        f = abi.Flux()
        f.kind = kind
        f.type_a = 0
        f.type_b = 0
        f.index_a = ia
        f.index_b = ib
        f.coef = coef
        f.decay = decay
        f.target = target
        f.cutoff = cutoff
        w.fluxes.append((0, 0, f))
    return w


def bonded_fluid(n=2_000_000, density=0.85, cutoff=2.5, chain=16, steps=500, relax_steps=50, seed=2):
    rng = np.random.default_rng(np.random.PCG64(2000 + seed))
    n = (n // chain) * chain
    side = float((n / density) ** (1.0 / 3.0))
    nch = n // chain
    starts = rng.uniform(0.0, side, size=(nch, 3))
    dirs = rng.normal(size=(nch, chain - 1, 3))
    dirs /= np.linalg.norm(dirs, axis=2, keepdims=True)
    walk = np.concatenate([np.zeros((nch, 1, 3)), np.cumsum(dirs, axis=1)], axis=1) + starts[:, None, :]
    x = in_box(walk.reshape(n, 3), side)
    ids = np.arange(n, dtype=np.int32).reshape(nch, chain)
    bonds = np.stack([ids[:, :-1].reshape(-1), ids[:, 1:].reshape(-1)], axis=1).astype(np.int32)
    angles = np.stack([ids[:, :-2].reshape(-1), ids[:, 1:-1].reshape(-1), ids[:, 2:].reshape(-1)],
                      axis=1).astype(np.int32)
    c = cells_for(side, cutoff)
    w = Workload(
        name="bonded_fluid", origin=(0.0, 0.0, 0.0), dim=(side,) * 3, cells=(c, c, c), cutoff=cutoff,
        dt=0.002, steps=steps, x=x, type=np.zeros(n, np.int32), radius=np.ones(n, np.float32),
        imass=np.ones(n, np.float32), max_type=1, dynamics=[abi.NEWTONIAN], mass=[1.0],
        bonds=bonds, angles=angles, relax_steps=relax_steps, seed=2000 + seed)
    w.pots[(0, 0)] = PotSpec("lj", dict(min=0.1, max=cutoff, A=1.0, B=1.0, tol=0.0))
    w.bond_pot = PotSpec("harmonic", dict(k=100.0, r0=1.0, min=-1.0, max=-1.0, tol=0.0))
    w.angle_pot = PotSpec("harmonic_angle", dict(k=20.0, theta0=math.pi, min=-1.0, max=-1.0, tol=0.0))
    return w


def ensemble_sizes(count=256, nmin=500, nmax=50_000, seed=3):
    """Particle counts and A-B depths of the parameter sweep (no particle data)."""
    rng = np.random.default_rng(np.random.PCG64(3000 + seed))
    ns = np.exp(rng.uniform(math.log(nmin), math.log(nmax), size=count)).astype(np.int64)
    depths = rng.uniform(0.1, 2.0, size=count)
    return ns, depths


def ensemble(count=256, nmin=500, nmax=50_000, density=0.5, cutoff=3.0, steps=1000, seed=3, indices=None):
    """Parameter sweep: `count` independent cell_sorting-style simulations (or only those
    listed in `indices`; each simulation depends only on its index and `seed`)."""
    ns, depths = ensemble_sizes(count, nmin, nmax, seed)
    sims = []
    for i in (range(count) if indices is None else indices):
        n = int(ns[i])
        side = float((n / density) ** (1.0 / 3.0))
        w = cell_sorting(n=n, side=side, cutoff=cutoff, depth_ab=float(depths[i]), steps=steps,
                         seed=3000 + 17 * i + seed, random_force=(0.0, 0.1, 1))
        w.name = "ensemble[%d]" % i
        sims.append(w)
    return sims


def served_requests(count=10_000, rate=200.0, seed=4, nmin=1000, nmax=200_000, smin=100, smax=5000):
    """Arrival times and request shapes of the served stream (no particle data)."""
    rng = np.random.default_rng(np.random.PCG64(4000 + seed))
    gaps = rng.exponential(1.0 / rate, size=count)
    t = np.cumsum(gaps)
    kind = np.where(rng.uniform(size=count) < 0.6, 0, 1)
    n = np.exp(rng.uniform(math.log(nmin), math.log(nmax), size=count)).astype(np.int64)
    steps = rng.integers(smin, smax + 1, size=count)
    return [dict(t=float(t[i]), kind=int(kind[i]), n=int(n[i]), steps=int(steps[i]), seed=i)
            for i in range(count)]


def request_workload(req):
    """Materialise one served request: a cell_sorting- or dpd_droplets-style simulation."""
    n = req["n"]
    if req["kind"] == 0:
        side = float((n / 0.5) ** (1.0 / 3.0))
        return cell_sorting(n=n, side=side, steps=req["steps"], seed=50_000 + req["seed"])
    # DPD droplets scaled to n particles: keep the droplet density of the full-size case
    scale = (n / 100_000) ** (1.0 / 3.0)
    side = max(40.0 * scale, 8.0)
    return dpd_droplets(n=n, side=side, radius=12.0 * scale, steps=req["steps"], seed=50_000 + req["seed"])


def verlet(w, skin=0.2):
    """`w` in Verlet mode (TFG_ENGINE_VERLET) on a coarser grid whose cell edge is at least
    (1 + skin) * cutoff: the reference's skin is the slack min(h) - cutoff of the cell grid
    (engine_verlet_update, tfEngine.cpp:231), so a Verlet run needs cells larger than the
    cutoff."""
    import dataclasses
    cells = tuple(max(3, int(math.floor(d / (w.cutoff * (1.0 + skin))))) for d in w.dim)
    return dataclasses.replace(w, cells=cells, flags=w.flags | abi.ENGINE_VERLET,
                               name=w.name + "_verlet")


def lj_fluid(n=2_000_000, density=0.85, cutoff=2.5, temperature=0.5, steps=500, seed=5):
    """Lennard-Jones fluid (the bonded fluid's 12-6 potential, no bonds) started without
    overlaps: a simple cubic lattice at the given density, jittered, with Maxwell
    velocities.  Stable without the reference's displacement clamp, so it also runs in
    Verlet mode."""
    rng = np.random.default_rng(np.random.PCG64(5000 + seed))
    m = int(round((n) ** (1.0 / 3.0)))
    n = m ** 3
    side = float((n / density) ** (1.0 / 3.0))
    a = side / m
    g = (np.arange(m) + 0.5) * a
    x = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(n, 3)
    x = in_box(x + rng.uniform(-0.05 * a, 0.05 * a, size=x.shape), side)
    v = rng.normal(0.0, math.sqrt(temperature), size=(n, 3))
    v -= v.mean(axis=0)
    c = cells_for(side, cutoff)
    w = Workload(
        name="lj_fluid", origin=(0.0, 0.0, 0.0), dim=(side,) * 3, cells=(c, c, c), cutoff=cutoff,
        dt=0.002, steps=steps, x=x, type=np.zeros(n, np.int32), v=v.astype(np.float32),
        radius=np.ones(n, np.float32), imass=np.ones(n, np.float32), max_type=1,
        dynamics=[abi.NEWTONIAN], mass=[1.0], seed=5000 + seed)
    w.pots[(0, 0)] = PotSpec("lj", dict(min=0.1, max=cutoff, A=1.0, B=1.0, tol=0.0))
    return w
