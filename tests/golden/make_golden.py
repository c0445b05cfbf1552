"""Write the golden fixtures of this directory from the CPU oracle.

The reference engine cannot be built or imported here (its Magnum, Corrade and libsbml
submodules are empty and its build needs GL, GLFW and assimp), and its own test suite
holds no golden vectors for this path, so these fixtures are NOT reference outputs: they
record the oracle's results (the CPU restatement of the reference arithmetic, FP32, one
runner thread) on small seeded inputs.  They pin the oracle against regressions and give
the GPU tests a committed target; the oracle itself is pinned by the closed-form and
Philox known-answer tests in test_cpu_oracle.py.

    python tests/golden/make_golden.py          # rewrites tests/golden/*.npz
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "tissue-forge_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import oracle as O  # noqa: E402
from tfg import configs  # noqa: E402
from tfg.engine import setup_model  # noqa: E402


def cases():
    """name -> (workload factory, steps of the trajectory part)."""
    return {
        "cell_sorting_300": (lambda: configs.cell_sorting(n=300, side=10.0, seed=5), 5),
        "cell_sorting_rf_1200": (lambda: configs.cell_sorting(n=1200, side=13.0, depth_ab=1.4, seed=6,
                                                              random_force=(0.0, 0.1, 1)), 5),
        "dpd_flux_800": (lambda: configs.dpd_droplets(n=800, side=8.0, radius=2.2, seed=8), 3),
        "bonded_640": (lambda: configs.bonded_fluid(n=640, seed=10), 3),
    }


def oracle_engine(w):
    e = O.OracleEngine(w.desc(), 0, 1)
    keep = setup_model(e, w)
    e._keep = keep
    return e


def record(w, steps):
    out = {"x_in": w.x, "type_in": w.type}
    e = oracle_engine(w)
    d = e.download()
    out["load_cell"] = d["cell"]
    out["load_xrel"] = d["xrel"]
    e.force_only()
    cnt, hsh = e.signature()
    d = e.download()
    out["sig_count"] = cnt
    out["sig_hash"] = hsh
    out["force"] = d["f"]
    out["density"] = d["density"]
    out["fmag"] = e.fmag()
    if w.nr_species:
        out["q"] = d["q"]
    e2 = oracle_engine(w)
    e2.step(steps)
    d = e2.download()
    out["traj_x"] = d["x"]
    out["traj_cell"] = d["cell"]
    out["traj_v"] = d["v"]
    if w.nr_species:
        out["traj_species"] = d["species"]
    r = e2.reductions()
    out["traj_red"] = np.array([r.epot, r.kinetic, r.virial, r.migrations], np.float64)
    out["steps"] = np.array(steps)
    return out


def main():
    O.build()
    for name, (make, steps) in cases().items():
        w = make()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **record(w, steps))
        print("wrote", name, w.n)


if __name__ == "__main__":
    main()
