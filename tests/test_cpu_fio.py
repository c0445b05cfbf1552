"""FIO (JSON) import and export (tfFIO.cpp, tfSimulator.cpp:940-1020, tfUniverse.cpp:413-678):
lossless round trips of the workloads, identical oracle runs of a model and of its imported
copy, and the import of a file in the reference writer's layout."""
import json
import os

import numpy as np

import oracle as O
from helpers import small_bonded, small_cell_sorting, small_dpd
from tfg import abi, configs, fio
from tfg.engine import setup_model
from tfg.potentials import Potential

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _with_walls(w):
    w.boundaries = [(4, abi.BOUNDARY_FREESLIP, (0.0, 0.0, 0.0), 1.0, 0.0),
                    (5, abi.BOUNDARY_VELOCITY, (0.5, 0.0, 0.0), 0.8, 0.0)]
    w.wall_pots = [(4, 1, configs.PotSpec("lj", dict(min=0.1, max=1.0, A=0.01, B=0.02, tol=0.0)))]
    w.random_force = (0.0, 0.3, 1)
    return w


CASES = {
    "cell_sorting": lambda: _with_walls(small_cell_sorting()),
    "dpd": lambda: small_dpd(n=1500, side=9.0),
    "bonded": lambda: small_bonded(n=16 * 120),
}


def _table(spec):
    p = Potential.from_spec(spec)
    st = p.ptr.contents
    c = np.ctypeslib.as_array(st.c, shape=((st.n + 1) * abi.POTENTIAL_CHUNK,)).copy() if st.c else None
    return st.kind, st.flags, tuple(st.alpha), st.n, c, (st.dpd_alpha, st.dpd_gamma, st.dpd_sigma)


def test_round_trip_is_lossless():
    for name, make in CASES.items():
        w = make()
        w2 = fio.load(json.dumps(fio.from_workload(w)))
        assert w2.n == w.n and w2.max_type == w.max_type and tuple(w2.cells) == tuple(w.cells), name
        assert np.array_equal(w2.x, w.x) and np.array_equal(w2.type, w.type), name
        assert np.array_equal(w2.radius, w.radius) and np.array_equal(w2.imass, w.imass), name
        if w.v is not None:
            assert np.array_equal(w2.v, w.v), name
        if w.nr_species:
            assert np.array_equal(w2.species, w.species), name
        assert set(w2.pots) == set(w.pots), name
        for k in w.pots:
            a, b = _table(w.pots[k]), _table(w2.pots[k])
            assert a[:4] == b[:4] and a[5] == b[5], name
            assert (a[4] is None and b[4] is None) or np.array_equal(a[4], b[4]), name
        if w.bonds is not None:
            assert np.array_equal(w2.bonds, w.bonds) and np.array_equal(w2.angles, w.angles)
        assert [b[:2] for b in w2.boundaries if b[1] != abi.BOUNDARY_PERIODIC] == [b[:2] for b in w.boundaries]


def test_imported_model_runs_bitexact():
    """The oracle runs a model and its FIO copy to the same bits."""
    for name, make in CASES.items():
        w = make()
        w2 = fio.load(json.dumps(fio.from_workload(w)))
        a = O.OracleEngine(w.desc(), 0, 1)
        a._k = setup_model(a, w)
        b = O.OracleEngine(w2.desc(), 0, 1)
        b._k = setup_model(b, w2)
        a.step(5)
        b.step(5)
        da, db = a.download(), b.download()
        for k in ("x", "v", "f"):
            assert np.array_equal(da[k].view(np.uint32), db[k].view(np.uint32)), (name, k)


def test_reference_style_file():
    """A file in the reference writer's layout (six-decimal floats, built-in types first, a
    destroyed particle's id missing; tests/golden/make_fio_fixture.py)."""
    w = fio.load(os.path.join(GOLDEN, "fio_reference_style.json"))
    assert w.n == 48 and w.max_type == 4
    assert w.dynamics[2] == abi.OVERDAMPED and w.mass[3] == 2.0
    assert sorted(w.pots) == [(2, 2), (2, 3), (3, 3)]
    assert np.array_equal(w.type[:4], [2, 3, 2, 3])
    assert np.allclose(w.imass[:2], [1.0, 0.5])
    # ids 0..48 without 17: bonds and angles refer to the compacted ids
    assert w.bonds.tolist() == [[0, 1], [1, 2], [2, 3]] and w.angles.tolist() == [[0, 1, 2]]
    assert list(w.bond_slot) == [0, 0, 0] and list(w.angle_slot) == [1]
    assert w.type_forces == [(3, 0.0, 0.5, 1)]
    kinds = {b[0]: b[1] for b in w.boundaries}
    assert kinds[4] == kinds[5] == abi.BOUNDARY_FREESLIP and kinds[0] == abi.BOUNDARY_PERIODIC
    assert sorted((wall, t) for wall, t, _ in w.wall_pots) == [(4, 2), (5, 2)]
    # six decimals: the Morse table read back is the factory's to within 5e-7
    ref = _table(configs.PotSpec("morse", dict(d=1.0, a=3.0, r0=1.0, min=0.2, max=3.0, tol=0.01, shifted=True)))
    got = _table(w.pots[(2, 2)])
    assert got[3] == ref[3] and np.max(np.abs(got[4] - ref[4])) <= 5e-7
    # and the model runs
    e = O.OracleEngine(w.desc(), 0, 1)
    e._k = setup_model(e, w)
    e.step(3)
    r = e.reductions()
    assert np.isfinite(r.epot) and r.steps == 3
