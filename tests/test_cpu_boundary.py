"""Known-answer tests of the oracle's boundary conditions (tfBoundaryConditions.h,
tf_boundary_eval.h): no cell pairs across a non-periodic edge, reflection at FREESLIP and
VELOCITY (NO_SLIP) walls, and wall potentials."""
import numpy as np

import oracle as O
from tfg import Potential, abi


def _one(x, v, walls, dyn=abi.NEWTONIAN, pot=None, wall_pot=None, side=20.0, cells=20, cutoff=1.0, dt=0.005):
    d = abi.engine_desc((0, 0, 0), (side,) * 3, (cells,) * 3, cutoff, dt, max_type=1)
    e = O.OracleEngine(d, O.MODE_NO_DENSITY)
    e.set_type(0, dyn)
    for w, kind, vel in walls:
        e.set_boundary(w, kind, vel)
    if pot is not None:
        e.set_potential(0, 0, pot.ptr)
    if wall_pot is not None:
        e.set_boundary_potential(wall_pot[0], 0, wall_pot[1].ptr)
    e.load(np.array(x, np.float32), v=np.array(v, np.float32))
    return e


def test_no_pairs_across_a_non_periodic_edge():
    lj = Potential.lennard_jones_12_6(0.1, 1.0, 1.0, 1.0)
    x = [[0.3, 5.0, 5.0], [19.8, 5.0, 5.0]]
    e = _one(x, np.zeros((2, 3)), [], pot=lj)
    e.record_pairs(True)
    e.force_only()
    assert len(e.pairs()) == 1                      # periodic by default
    e = _one(x, np.zeros((2, 3)), [(0, abi.BOUNDARY_FREESLIP, (0, 0, 0)), (1, abi.BOUNDARY_FREESLIP, (0, 0, 0))],
             pot=lj)
    e.record_pairs(True)
    e.force_only()
    assert len(e.pairs()) == 0


def test_freeslip_reflects_normal_velocity():
    walls = [(w, abi.BOUNDARY_FREESLIP, (0, 0, 0)) for w in (0, 1)]
    e = _one([[0.002, 5.5, 5.5]], [[-1.0, 0.5, 0.0]], walls)
    e.step(1)
    d = e.download()
    # x = 0.002 - 0.005 = -0.003 -> reflected to 0.003 in cell 0, v_x flipped
    assert abs(d["x"][0][0] - np.float32(0.003)) < 1e-6
    assert np.allclose(d["v"][0], [1.0, 0.5, 0.0])
    assert d["cell"][0] == 5 * 20 + 5   # still in the x = 0 column


def test_no_slip_wall_reverses_velocity():
    walls = [(w, abi.BOUNDARY_NO_SLIP, (0, 0, 0)) for w in (4, 5)]
    e = _one([[5.5, 5.5, 19.999]], [[0.3, -0.2, 1.0]], walls)
    e.step(1)
    d = e.download()
    # z = 19.999 + 0.005 crosses the top: z -> h - (z - h) inside the top cell, v -> -v
    assert d["x"][0][2] < 20.0 and d["x"][0][2] > 19.99
    assert np.allclose(d["v"][0], [-0.3, 0.2, -1.0])


def test_wall_potential_force():
    lj = Potential.lennard_jones_12_6(0.1, 2.0, 1.0, 1.0)
    walls = [(w, abi.BOUNDARY_POTENTIAL, (0, 0, 0)) for w in (0, 1)]
    r = 0.8
    e = _one([[r, 5.5, 5.5]], [[0.0, 0.0, 0.0]], walls, dyn=abi.OVERDAMPED, wall_pot=(0, lj), cutoff=2.0, cells=10)
    e.force_only()
    f = e.download()["f"][0]
    ee, fr = lj.eval(r)
    # part.f -= f * dx with dx = +r for the low wall
    assert abs(f[0] - (-fr * r)) <= 1e-5 * max(1.0, abs(fr * r))
    assert f[1] == 0 and f[2] == 0


def resetting_box():
    """A periodic box whose x walls are PERIODIC | RESETTING: particles carry one species at
    1.0 and drift at constant velocity; those crossing the x boundary take the reset value
    0.25 (apply_boundary_particle_crossing, tfBoundaryConditions.cpp:676-735), those crossing
    the plain periodic y boundary keep theirs."""
    from tfg.configs import Workload
    n = 40
    rng = np.random.default_rng(3)
    x = np.zeros((n, 3), np.float32)
    v = np.zeros((n, 3), np.float32)
    x[:20, 0] = rng.uniform(9.90, 9.98, 20)        # about to cross x = 10 in +x
    x[:20, 1:] = rng.uniform(1.0, 9.0, (20, 2))
    v[:20, 0] = 1.0
    x[20:30, 0] = rng.uniform(0.02, 0.08, 10)      # about to cross x = 0 in -x
    x[20:30, 1:] = rng.uniform(1.0, 9.0, (10, 2))
    v[20:30, 0] = -1.0
    x[30:, 1] = rng.uniform(9.90, 9.98, 10)        # about to cross y = 10 in +y (not resetting)
    x[30:, [0, 2]] = rng.uniform(1.0, 9.0, (10, 2))
    v[30:, 1] = 1.0
    w = Workload(name="resetting_box", origin=(0.0, 0.0, 0.0), dim=(10.0,) * 3, cells=(3, 3, 3), cutoff=1.0,
                 dt=0.01, steps=20, x=x, type=np.zeros(n, np.int32), v=v, radius=np.ones(n, np.float32),
                 imass=np.ones(n, np.float32), species=np.ones((n, 1), np.float32), nr_species=1, max_type=1,
                 dynamics=[abi.NEWTONIAN], mass=[1.0], flags=abi.ENGINE_NO_DENSITY)
    kind = abi.BOUNDARY_PERIODIC | abi.BOUNDARY_RESETTING
    w.boundaries = [(0, kind, (0, 0, 0), 1.0, 0.0), (1, kind, (0, 0, 0), 1.0, 0.0)]
    w.species_reset = [0.25]
    return w


def test_resetting_boundary_resets_species_of_crossers_only():
    from helpers import make_oracle
    w = resetting_box()
    e = make_oracle(w)
    e.step(20)
    d = e.download()
    assert np.all(d["x"][:20, 0] < 1.0) and np.all(d["x"][20:30, 0] > 9.0)   # wrapped in x
    assert np.all(d["species"][:30, 0] == np.float32(0.25))
    assert np.all(d["x"][30:, 1] < 1.0)                                        # wrapped in y
    assert np.all(d["species"][30:, 0] == 1.0)


def test_resetting_needs_both_walls_periodic():
    """A RESETTING wall facing a non-periodic one: check_periodicy makes both exactly
    PERIODIC (tfBoundaryConditions.cpp:192-216), which drops RESETTING: nothing resets."""
    from helpers import make_oracle
    w = resetting_box()
    w.boundaries = [(0, abi.BOUNDARY_PERIODIC | abi.BOUNDARY_RESETTING, (0, 0, 0), 1.0, 0.0),
                    (1, abi.BOUNDARY_FREESLIP, (0, 0, 0), 1.0, 0.0)]
    e = make_oracle(w)
    e.step(20)
    assert np.all(e.download()["species"][:, 0] == 1.0)
