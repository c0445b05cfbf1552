"""Writes fio_reference_style.json: a small model in the FIO layout the reference's writer
produces (FIO::toFile), for the importer's tests.

Nothing here runs the reference (it cannot be built here).  The file follows the writer's
code: every float is std::to_string of the value, i.e. six decimals (tf_io.cpp:30-33); the
built-in types "Particle" (id 0) and "Cluster" (id 1) come first in particleTypes
(tfUniverse.cpp:616-619); particle ids have a gap where a particle was destroyed;
potentials are indexed by position in particleTypes (tfUniverse.cpp:621-645); and a
boundaryCondition has a "velocity" child only for velocity kinds
(tfBoundaryConditions.cpp:752-754).  The tables are those of the library's Potential
factories.

Usage: python tests/golden/make_fio_fixture.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "tissue-forge_gb300"))

from tfg import abi  # noqa: E402
from tfg.potentials import Potential  # noqa: E402

T, V = "IOType", "IOValue"


def f(x):
    return {T: "float", V: "%f" % float(np.float32(x))}


def i(x, t="int"):
    return {T: t, V: str(int(x))}


def s(x):
    return {T: "string", V: x}


def node(t, **ch):
    d = {T: t, V: ""}
    d.update(ch)
    return d


def vec(items):
    d = node("vector")
    for k, it in enumerate(items):
        d[str(k)] = it
    return d


def v3(a, conv=f):
    return node("Vector3", x=conv(a[0]), y=conv(a[1]), z=conv(a[2]))


def pot(p, name):
    st = p.ptr.contents
    nc = (st.n + 1) * abi.POTENTIAL_CHUNK
    return node("Potential", kind=i(st.kind, "unsigned_int"), flags=i(st.flags, "unsigned_int"), name=s(name),
                a=f(st.a), b=f(st.b), alpha=vec([f(st.alpha[k]) for k in range(4)]), n=i(st.n),
                c=vec([f(st.c[k]) for k in range(nc)]), r0_plusone=f(st.r0_plusone), mu=f(0.0),
                offset=vec([f(0.0)] * 3))


def main():
    rng = np.random.default_rng(123)
    side, cells, cutoff = 12.0, 4, 3.0
    # two user types A (id 2) and B (id 3); 48 particles, id 17 destroyed
    ids = [k for k in range(49) if k != 17]
    x = rng.uniform(0.5, side - 0.5, size=(len(ids), 3))
    v = rng.normal(0.0, 0.3, size=(len(ids), 3))
    typ = [2 if k % 2 == 0 else 3 for k in range(len(ids))]
    mass = [1.0 if t == 2 else 2.0 for t in typ]
    morse_aa = Potential.morse(1.0, 3.0, 1.0, 0.2, 3.0, 0.01, True)
    morse_ab = Potential.morse(0.3, 3.0, 1.0, 0.2, 3.0, 0.01, True)
    bond = Potential.harmonic(20.0, 1.2, -1.0, -1.0, 0.0)
    angle = Potential.harmonic_angle(5.0, np.pi, -1.0, -1.0, 0.0)
    wall = Potential.lennard_jones_12_6(0.2, 1.5, 0.01, 0.02, 0.0)

    parts = []
    for k, pid in enumerate(ids):
        parts.append(node("Particle", force=v3((0, 0, 0)), force_i=v3((0, 0, 0)), number_density=f(0.0),
                          velocity=v3(v[k]), position=v3(x[k]), creation_time=f(0.0),
                          persistent_force=v3((0, 0, 0)), radius=f(0.5 if typ[k] == 2 else 0.6), mass=f(mass[k]),
                          q=f(0.0), p0=v3((0, 0, 0)), v0=v3((0, 0, 0)), id=i(pid), vid=i(0), typeId=i(typ[k]),
                          clusterId=i(-1), flags=i(0, "unsigned_short")))
    ptypes = []
    for tid, name, tmass, dyn in ((0, "Particle", 1.0, 0), (1, "Cluster", 1.0, 0), (2, "A", 1.0, 1), (3, "B", 2.0, 1)):
        ptypes.append(node("ParticleType", id=i(tid), type_flags=i(0, "unsigned_int"),
                           particle_flags=i(2 if tid == 1 else 0, "unsigned_int"), mass=f(tmass), charge=f(0.0),
                           radius=f(1.0), kinetic_energy=f(0.0), potential_energy=f(0.0), target_energy=f(0.0),
                           minimum_radius=f(0.0), eps=f(1.0), rmin=f(1.0), dynamics=i(dyn, "unsigned_int"),
                           name=s(name), name2=s(name)))
    bonds = [(0, 1), (1, 2), (2, 3)]
    angles = [(0, 1, 2)]
    # the wall potential acts on type A at the bottom and top walls
    walls = {}
    for wname, wid in (("top", 5), ("bottom", 4), ("left", 0), ("right", 1), ("front", 2), ("back", 3)):
        kind = abi.BOUNDARY_FREESLIP if wname in ("top", "bottom") else abi.BOUNDARY_PERIODIC
        bc = node("boundaryCondition", kind=i(kind), id=i(wid), restore=f(1.0), name=s(wname),
                  normal=v3((0, 0, 0)), radius=f(0.0))
        if wname in ("top", "bottom"):
            bc["potentialIndices"] = vec([i(2, "unsigned_int")])
            bc["potentials"] = vec([pot(wall, "wall")])
        walls[wname] = bc
    sim = node("Simulator", dim=v3((side, side, side)), cutoff=f(cutoff), cells=v3((cells,) * 3, i),
               integrator=i(0), dt=f(0.002), time=i(0), boundary_conditions=node("boundaryConditions", **walls),
               max_distance=f(0.05 * side / cells), seed=i(4321, "unsigned_int"), nr_fluxsteps=i(1, "unsigned_int"))
    uni = node("Universe", name=s("fixture"), particles=vec(parts),
               bonds=vec([node("Bond", flags=i(1, "unsigned_int"), i=i(ids[a]), j=i(ids[b]), id=i(k),
                               creation_time=f(0.0), half_life=f(0.0), dissociation_energy=f(-1.0),
                               potential_energy=f(0.0)) for k, (a, b) in enumerate(bonds)]),
               bondPotentials=vec([pot(bond, "bond")]), bondPotentialIdx=vec([vec([i(0, "unsigned_int"),
                                                                                   i(1, "unsigned_int"),
                                                                                   i(2, "unsigned_int")])]),
               angles=vec([node("Angle", flags=i(1, "unsigned_int"), i=i(ids[a]), j=i(ids[b]), k=i(ids[c]),
                                id=i(0), creation_time=f(0.0), half_life=f(0.0), dissociation_energy=f(-1.0),
                                potential_energy=f(0.0)) for (a, b, c) in angles]),
               anglePotentials=vec([pot(angle, "angle")]), anglePotentialIdx=vec([vec([i(0, "unsigned_int")])]),
               temperature=f(0.0), kineticEnergy=f(0.0), particleTypes=vec(ptypes),
               potentials=vec([pot(morse_aa, "aa"), pot(morse_ab, "ab"), pot(morse_aa, "bb")]),
               potentialTypeA=vec([i(2, "unsigned_int"), i(2, "unsigned_int"), i(3, "unsigned_int")]),
               potentialTypeB=vec([i(2, "unsigned_int"), i(3, "unsigned_int"), i(3, "unsigned_int")]),
               forces=vec([node("GaussianForce", type=i(1), stateVectorIndex=i(-1), std=f(0.5), mean=f(0.0),
                                durration_steps=i(1))]),
               forceType=vec([i(3, "unsigned_int")]))
    root = node("Root", MetaData=node("MetaData", versionMajor=i(0), versionMinor=i(2), versionPatch=i(0)),
                Simulator=sim, Universe=uni)
    with open(os.path.join(HERE, "fio_reference_style.json"), "w") as fh:
        json.dump(root, fh, separators=(",", ":"))


if __name__ == "__main__":
    main()
