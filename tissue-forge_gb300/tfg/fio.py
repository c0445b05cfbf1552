"""Tissue Forge FIO (JSON) files in and out of the per-step particle path.

The reference saves a simulation with FIO::toFile (source/io/tfFIO.cpp:206-316) as a JSON
tree.  Every node is an object {"IOType": type, "IOValue": value, <key>: node, ...}
(io::toFile / io::fromFile of json, tfFIO.cpp:51-101).  Scalars hold std::to_string of the
value (tf_io.cpp:30-33), vectors have children "0".."n-1" (tf_io.h:540-570), and 3-vectors
have children "x", "y", "z" (tf_io.h:213-240).  The root has the children "MetaData"
(tf_io.cpp:283-300), "Simulator" (tfSimulator.cpp:940-960) and "Universe"
(tfUniverse.cpp:413-678).

`to_workload` reads the parts that the particle path consumes into a configs.Workload, which
the engine, the batch and the server take like any other workload:
- Simulator: space, cutoff, cells, dt, seed, displacement limit, flux substeps, boundary
  conditions with their wall potentials;
- Universe: particle types, particles (position, velocity, external force, radius, mass,
  flags, species values), the pair potentials per type pair, bonds and angles with their
  potentials, and Gaussian random forces per type.

Potentials are taken as tables, as the reference stores them (tfPotential.cpp:3282-3340), and
are not rebuilt from factory arguments.  `from_workload` writes the same layout; it writes
floats with nine significant digits, where the reference's writer keeps six decimals.

Clusters, large particles, dihedrals, other force kinds, potentials of kind "combination" and
integrators other than forward Euler are outside the path and are rejected with ValueError.
Flux objects are not part of a saved Universe (the reference re-creates them in its scripts),
so the model's fluxes have to be added to the returned workload by the caller.
"""
import json

import numpy as np

from . import abi
from .configs import PotSpec, Workload

T, V = "IOType", "IOValue"
_WALLS = {"left": 0, "right": 1, "front": 2, "back": 3, "bottom": 4, "top": 5}
_PARTICLE_CLUSTER = 1 << 1          # ParticleFlags (tfParticle.h:68-78)
_POTENTIAL_KIND_COMBINATION = 3     # tfPotential.h:56-61
_FORWARD_EULER = 0                  # EngineIntegrator (tfEngine.h:89-92)


# ---- reading nodes ----

def _children(node):
    return {k: v for k, v in node.items() if k not in (T, V)}


def _f(node):
    """A float as std::stof parses the stored text."""
    return float(np.float32(float(node[V])))


def _i(node):
    return int(float(node[V]))


def _vec(node, conv):
    n = len(_children(node))
    return [conv(node[str(i)]) for i in range(n)]


def _v3(node, conv=_f):
    return tuple(conv(node[k]) for k in ("x", "y", "z"))


def _has(node, key):
    return key in node and isinstance(node[key], dict)


def _in_box(x, dim):
    """Positions wrapped into the periodic box and kept off its upper faces (space_setpartp,
    tfSpace.cpp:443-448, rejects a coordinate that rounds to the upper face)."""
    d = np.asarray(dim, np.float64)
    y = np.mod(np.asarray(x, np.float64), d)
    return np.minimum(y, d * (1.0 - 1e-6)).astype(np.float32)


def read(src):
    """The JSON tree of a FIO file (a path), or of a JSON string."""
    if isinstance(src, (bytes, str)) and str(src).lstrip().startswith("{"):
        return json.loads(src)
    with open(src) as f:
        return json.load(f)


def _potential(node):
    kind = _i(node["kind"])
    flags = _i(node["flags"])
    if kind == _POTENTIAL_KIND_COMBINATION:
        raise ValueError("combined potentials are not supported")
    if kind == abi.POTENTIAL_KIND_DPD:   # DPDPotential (tfDPDPotential.cpp:66-80)
        # fields DPD does not store keep Potential's defaults (tfPotential.cpp:59-81)
        return PotSpec("table", dict(kind=kind, flags=flags, alpha=(0.0,) * 4, r0_plusone=1.0, a=_f(node["a"]),
                                     b=_f(node["b"]), n=1, c=(),
                                     dpd=(_f(node["alpha"]), _f(node["gamma"]), _f(node["sigma"]))))
    alpha = tuple(_vec(node["alpha"], _f))
    n = _i(node["n"])
    c = tuple(_vec(node["c"], _f))
    if len(c) != (n + 1) * abi.POTENTIAL_CHUNK:
        raise ValueError("potential table has %d coefficients, expected %d" % (len(c), (n + 1) * abi.POTENTIAL_CHUNK))
    return PotSpec("table", dict(kind=kind, flags=flags, alpha=alpha, r0_plusone=_f(node["r0_plusone"]),
                                 a=_f(node["a"]), b=_f(node["b"]), n=n, c=c))


def to_workload(tree, name="fio", steps=100):
    """A configs.Workload from a FIO tree (see the module docstring)."""
    sim, uni = tree["Simulator"], tree["Universe"]
    if _has(sim, "integrator") and _i(sim["integrator"]) != _FORWARD_EULER:
        raise ValueError("only the forward Euler integrator is supported")
    dim = _v3(sim["dim"])
    cells = _v3(sim["cells"], _i)
    cutoff = _f(sim["cutoff"])
    dt = _f(sim["dt"])
    seed = _i(sim["seed"]) if _has(sim, "seed") else 0
    nfs = _i(sim["nr_fluxsteps"]) if _has(sim, "nr_fluxsteps") else 1
    frac = 0.05
    if _has(sim, "max_distance") and _f(sim["max_distance"]) >= 0:   # tfSimulator.cpp:661-666
        frac = _f(sim["max_distance"]) / (dim[0] / cells[0])

    # particle types: engine type ids; potentials and forces index this list by position
    ptypes = _vec(uni["particleTypes"], lambda nd: nd) if _has(uni, "particleTypes") else []
    type_ids = [_i(t["id"]) for t in ptypes]
    max_type = max(type_ids) + 1 if type_ids else 1
    dynamics = [abi.NEWTONIAN] * max_type
    mass = [1.0] * max_type
    for t, tid in zip(ptypes, type_ids):
        dynamics[tid] = _i(t["dynamics"])
        mass[tid] = _f(t["mass"])

    parts = _vec(uni["particles"], lambda nd: nd) if _has(uni, "particles") else []
    if any(_i(p["flags"]) & _PARTICLE_CLUSTER for p in parts):
        raise ValueError("clusters are not supported")
    parts.sort(key=lambda p: _i(p["id"]))
    local = {_i(p["id"]): k for k, p in enumerate(parts)}
    n = len(parts)
    x = np.array([_v3(p["position"]) for p in parts], np.float32).reshape(n, 3)
    v = np.array([_v3(p["velocity"]) for p in parts], np.float32).reshape(n, 3)
    fi = np.array([_v3(p["force_i"]) if _has(p, "force_i") else (0.0, 0.0, 0.0) for p in parts],
                  np.float32).reshape(n, 3)
    radius = np.array([_f(p["radius"]) for p in parts], np.float32)
    pmass = np.array([_f(p["mass"]) for p in parts], np.float32)
    imass = np.where(pmass > 0, np.float32(1.0) / np.where(pmass > 0, pmass, 1), 0).astype(np.float32)
    ptype = np.array([_i(p["typeId"]) for p in parts], np.int32)
    pflags = np.array([_i(p["flags"]) for p in parts], np.uint32)
    quant = [(_vec(p["state_vector"]["quantities"], _f) if _has(p, "state_vector") and
              _has(p["state_vector"], "quantities") else []) for p in parts]
    nspec = max((len(q) for q in quant), default=0)
    species = None
    if nspec:
        species = np.zeros((n, nspec), np.float32)
        for k, q in enumerate(quant):
            species[k, :len(q)] = q

    w = Workload(name=name, origin=(0.0, 0.0, 0.0), dim=dim, cells=cells, cutoff=cutoff, dt=dt, steps=steps,
                 x=_in_box(x, dim), type=ptype, v=v, radius=radius,
                 imass=imass, species=species, nr_species=nspec, max_type=max_type, dynamics=dynamics, mass=mass,
                 seed=seed, nr_fluxsteps=nfs, flags_particles=pflags, force_i=fi, max_dist_fraction=frac)

    if _has(uni, "potentials"):
        pots = _vec(uni["potentials"], _potential)
        ia = _vec(uni["potentialTypeA"], _i)
        ib = _vec(uni["potentialTypeB"], _i)
        for spec, a, b in zip(pots, ia, ib):
            w.pots[(type_ids[a], type_ids[b])] = spec

    slot = 0
    for key, pkey, ikey, arity in (("bonds", "bondPotentials", "bondPotentialIdx", 2),
                                   ("angles", "anglePotentials", "anglePotentialIdx", 3)):
        if not _has(uni, key):
            continue
        items = _vec(uni[key], lambda nd: nd)
        ids = np.array([[local[_i(it[c])] for c in "ijk"[:arity]] for it in items], np.int32).reshape(-1, arity)
        slots = np.zeros(len(items), np.int32)
        if _has(uni, pkey):
            for k, (spec, idx) in enumerate(zip(_vec(uni[pkey], _potential), _vec(uni[ikey], lambda nd: _vec(nd, _i)))):
                w.bonded_pots.append(spec)
                slots[idx] = slot + k
            slot = len(w.bonded_pots)
        if key == "bonds":
            w.bonds, w.bond_slot = ids, slots
        else:
            w.angles, w.angle_slot = ids, slots
    if slot > 16:
        raise ValueError("more than 16 bonded potentials")
    if _has(uni, "dihedrals") and len(_children(uni["dihedrals"])):
        raise ValueError("dihedrals are not supported")

    if _has(uni, "forces"):
        ft = _vec(uni["forceType"], _i)
        for f, ti in zip(_vec(uni["forces"], lambda nd: nd), ft):
            if f.get(T) != "GaussianForce":
                raise ValueError("force kind %r is not supported" % f.get(T))
            w.type_forces.append((type_ids[ti], _f(f["mean"]), _f(f["std"]), _i(f["durration_steps"])))

    if _has(sim, "boundary_conditions"):
        bcs = sim["boundary_conditions"]
        for wname, wall in _WALLS.items():
            if not _has(bcs, wname):
                continue
            bc = bcs[wname]
            kind = _i(bc["kind"])
            vel = _v3(bc["velocity"]) if _has(bc, "velocity") else (0.0, 0.0, 0.0)
            restore = _f(bc["restore"]) if _has(bc, "restore") else 1.0
            rad = _f(bc["radius"]) if _has(bc, "radius") else 0.0
            w.boundaries.append((wall, kind, vel, restore, rad))
            if _has(bc, "potentials"):
                for t, spec in zip(_vec(bc["potentialIndices"], _i), _vec(bc["potentials"], _potential)):
                    w.wall_pots.append((wall, t, spec))
    return w


def load(src, name="fio", steps=100):
    """to_workload of a FIO file (a path) or JSON string."""
    return to_workload(read(src), name=name, steps=steps)


# ---- writing nodes ----

def _s(value, type_):
    if type_ in ("float", "double"):
        text = "%.9g" % float(value)
    else:
        text = str(int(value))
    return {T: type_, V: text}


def _node(type_, **children):
    d = {T: type_, V: ""}
    d.update(children)
    return d


def _wvec(items):
    d = _node("vector")
    for k, it in enumerate(items):
        d[str(k)] = it
    return d


def _w3(v, type_="float"):
    return _node("Vector3", x=_s(v[0], type_), y=_s(v[1], type_), z=_s(v[2], type_))


def _wpot(spec, name=""):
    from .potentials import Potential
    p = Potential.from_spec(spec)
    st = p.ptr.contents
    if st.kind == abi.POTENTIAL_KIND_DPD:
        return _node("Potential", kind=_s(st.kind, "unsigned_int"), flags=_s(st.flags, "unsigned_int"),
                     name={T: "string", V: name}, a=_s(st.a, "float"), b=_s(st.b, "float"),
                     alpha=_s(st.dpd_alpha, "float"), gamma=_s(st.dpd_gamma, "float"), sigma=_s(st.dpd_sigma, "float"))
    nc = (st.n + 1) * abi.POTENTIAL_CHUNK
    return _node("Potential", kind=_s(st.kind, "unsigned_int"), flags=_s(st.flags, "unsigned_int"),
                 name={T: "string", V: name}, a=_s(st.a, "float"), b=_s(st.b, "float"),
                 alpha=_wvec([_s(st.alpha[k], "float") for k in range(4)]), n=_s(st.n, "int"),
                 c=_wvec([_s(st.c[k], "float") for k in range(nc)]), r0_plusone=_s(st.r0_plusone, "float"),
                 mu=_s(0.0, "float"), offset=_wvec([_s(0.0, "float") for _ in range(3)]))


def from_workload(w):
    """A FIO tree in the reference's layout for a configs.Workload (no fluxes: see above)."""
    h0 = w.dim[0] / w.cells[0]
    bcs = _node("boundaryConditions")
    walls = {wall: (kind, vel, restore, rad) for (wall, kind, vel, restore, rad) in w.boundaries}
    wpots = {}
    for (wall, t, spec) in w.wall_pots:
        wpots.setdefault(wall, []).append((t, spec))
    for wname, wall in _WALLS.items():
        kind, vel, restore, rad = walls.get(wall, (abi.BOUNDARY_PERIODIC, (0.0, 0.0, 0.0), 1.0, 0.0))
        bc = _node("boundaryCondition", kind=_s(kind, "int"), id=_s(wall, "int"), restore=_s(restore, "float"),
                   name={T: "string", V: wname}, normal=_w3((0.0, 0.0, 0.0)), radius=_s(rad, "float"))
        if kind & abi.BOUNDARY_VELOCITY:
            bc["velocity"] = _w3(vel)
        if wall in wpots:
            bc["potentialIndices"] = _wvec([_s(t, "unsigned_int") for t, _ in wpots[wall]])
            bc["potentials"] = _wvec([_wpot(spec) for _, spec in wpots[wall]])
        bcs[wname] = bc
    sim = _node("Simulator", dim=_w3(w.dim), cutoff=_s(w.cutoff, "float"), cells=_w3(w.cells, "int"),
                integrator=_s(_FORWARD_EULER, "int"), dt=_s(w.dt, "float"), time=_s(0, "int"),
                boundary_conditions=bcs, max_distance=_s(w.max_dist_fraction * h0, "float"),
                seed=_s(w.seed & 0xFFFFFFFF, "unsigned_int"), nr_fluxsteps=_s(w.nr_fluxsteps, "unsigned_int"))

    types = []
    for t in range(w.max_type):
        types.append(_node("ParticleType", id=_s(t, "int"), mass=_s(w.mass[t], "float"),
                           radius=_s(1.0, "float"), dynamics=_s(w.dynamics[t], "unsigned_int"),
                           name={T: "string", V: "type%d" % t}))
    n = w.n
    v = w.v if w.v is not None else np.zeros((n, 3), np.float32)
    fi = w.force_i if w.force_i is not None else np.zeros((n, 3), np.float32)
    radius = w.radius if w.radius is not None else np.ones(n, np.float32)
    imass = w.imass if w.imass is not None else np.ones(n, np.float32)
    flags = w.flags_particles if w.flags_particles is not None else np.zeros(n, np.uint32)
    parts = []
    for k in range(n):
        p = _node("Particle", position=_w3(w.x[k]), velocity=_w3(v[k]), force_i=_w3(fi[k]),
                  radius=_s(radius[k], "float"),
                  mass=_s(1.0 / imass[k] if imass[k] > 0 else 0.0, "float"), id=_s(k, "int"),
                  typeId=_s(w.type[k], "int"), flags=_s(flags[k], "unsigned_int"))
        if w.nr_species:
            p["state_vector"] = _node("StateVector", size=_s(w.nr_species, "unsigned_int"),
                                      quantities=_wvec([_s(q, "float") for q in w.species[k]]))
        parts.append(p)
    uni = _node("Universe", name={T: "string", V: w.name}, particles=_wvec(parts), particleTypes=_wvec(types))
    if w.pots:
        keys = sorted(w.pots)
        uni["potentials"] = _wvec([_wpot(w.pots[k]) for k in keys])
        uni["potentialTypeA"] = _wvec([_s(a, "unsigned_int") for a, _ in keys])
        uni["potentialTypeB"] = _wvec([_s(b, "unsigned_int") for _, b in keys])
    bonded = list(w.bonded_pots)
    bslot, aslot = w.bond_slot, w.angle_slot
    if not bonded and (w.bond_pot is not None or w.angle_pot is not None):
        bonded = [w.bond_pot, w.angle_pot]
        bslot = None if w.bonds is None else np.zeros(len(w.bonds), np.int32)
        aslot = None if w.angles is None else np.ones(len(w.angles), np.int32)
    for key, pkey, ikey, items, slots, cls in (("bonds", "bondPotentials", "bondPotentialIdx", w.bonds, bslot, "Bond"),
                                               ("angles", "anglePotentials", "anglePotentialIdx", w.angles, aslot,
                                                "Angle")):
        if items is None or not len(items):
            continue
        uni[key] = _wvec([_node(cls, flags=_s(1, "unsigned_int"), id=_s(k, "int"),
                                **{c: _s(it[m], "int") for m, c in enumerate("ijk"[:items.shape[1]])})
                          for k, it in enumerate(items)])
        used = sorted(set(int(s) for s in slots))
        uni[pkey] = _wvec([_wpot(bonded[s]) for s in used])
        uni[ikey] = _wvec([_wvec([_s(k, "unsigned_int") for k in np.nonzero(slots == s)[0]]) for s in used])
    forces = list(w.type_forces)
    if w.random_force is not None:
        forces += [(t,) + tuple(w.random_force) for t in range(w.max_type)]
    if forces:
        uni["forces"] = _wvec([_node("GaussianForce", type=_s(0, "int"), stateVectorIndex=_s(-1, "int"),
                                     mean=_s(m, "float"), std=_s(s, "float"), durration_steps=_s(d, "int"))
                               for (_, m, s, d) in forces])
        uni["forceType"] = _wvec([_s(t, "unsigned_int") for (t, _, _, _) in forces])
    meta = _node("MetaData", versionMajor=_s(0, "int"), versionMinor=_s(0, "int"), versionPatch=_s(0, "int"))
    return _node("Root", MetaData=meta, Simulator=sim, Universe=uni)


def save(w, path):
    with open(path, "w") as f:
        json.dump(from_workload(w), f, indent=1)
