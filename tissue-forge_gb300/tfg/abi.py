"""ctypes mirror of include/tfg.h (structs, constants, prototypes).

The C-ABI is the product boundary; this module only describes it for Python
callers.  Struct layouts follow the header field for field.
"""
import ctypes as C

TFG_OK = 0
TFG_E_INVAL = -1
TFG_E_OOM = -2
TFG_E_CUDA = -3
TFG_E_TOOFAST = -4
TFG_E_TIMEOUT = -5
TFG_E_OVERFLOW = -6
TFG_E_RANGE = -7
TFG_E_STATE = -8
TFG_E_NAN = -9
TFG_E_NODEVICE = -10

STATUS_NAMES = {
    0: "TFG_OK", -1: "TFG_E_INVAL", -2: "TFG_E_OOM", -3: "TFG_E_CUDA", -4: "TFG_E_TOOFAST",
    -5: "TFG_E_TIMEOUT", -6: "TFG_E_OVERFLOW", -7: "TFG_E_RANGE", -8: "TFG_E_STATE",
    -9: "TFG_E_NAN", -10: "TFG_E_NODEVICE",
}

POTENTIAL_KIND_POTENTIAL = 0
POTENTIAL_KIND_DPD = 1
POTENTIAL_R2 = 1 << 4
POTENTIAL_ANGLE = 1 << 6
POTENTIAL_HARMONIC = 1 << 7
POTENTIAL_SCALED = 1 << 11
POTENTIAL_SHIFTED = 1 << 12
POTENTIAL_CHUNK = 8
# tfg_set_split / tfg_autotune: the home-particle-outer pair kernel (tabulated potentials only)
PAIR_HOME_OUTER = 32

FLUX_FICK = 0
FLUX_SECRETE = 1
FLUX_UPTAKE = 2

# boundary kinds (tfBoundaryConditions.h:39-45); walls 0..5 = left, right, front, back, bottom, top
BOUNDARY_VELOCITY = 1 << 0
BOUNDARY_PERIODIC = 1 << 1
BOUNDARY_FREESLIP = 1 << 2
BOUNDARY_POTENTIAL = 1 << 3
BOUNDARY_NO_SLIP = 1 << 4

NEWTONIAN = 0
OVERDAMPED = 1

PARTICLE_FROZEN_X = 1 << 3
PARTICLE_FROZEN_Y = 1 << 4
PARTICLE_FROZEN_Z = 1 << 5

# engine flags (tfg_engine_desc.flags)
ENGINE_DPD_REFERENCE_RANDOM = 1 << 0
ENGINE_NO_DENSITY = 1 << 1
ENGINE_VERLET = 1 << 2


class Potential(C.Structure):
    _fields_ = [
        ("kind", C.c_uint32), ("flags", C.c_uint32), ("alpha", C.c_float * 4),
        ("r0_plusone", C.c_float), ("a", C.c_float), ("b", C.c_float), ("n", C.c_int32),
        ("c", C.POINTER(C.c_float)),
        ("dpd_alpha", C.c_float), ("dpd_gamma", C.c_float), ("dpd_sigma", C.c_float),
    ]


class Flux(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("type_a", C.c_int32), ("type_b", C.c_int32),
        ("index_a", C.c_int32), ("index_b", C.c_int32),
        ("coef", C.c_float), ("decay", C.c_float), ("target", C.c_float), ("cutoff", C.c_float),
    ]


class EngineDesc(C.Structure):
    _fields_ = [
        ("origin", C.c_float * 3), ("dim", C.c_float * 3), ("cells", C.c_int32 * 3),
        ("cutoff", C.c_float), ("dt", C.c_float), ("max_type", C.c_int32),
        ("nr_species", C.c_int32), ("particle_max_dist_fraction", C.c_float),
        ("seed", C.c_uint64), ("capacity", C.c_int32), ("max_bonds", C.c_int32),
        ("max_angles", C.c_int32), ("device", C.c_int32), ("flags", C.c_uint32),
        ("nr_fluxsteps", C.c_int32),
    ]


class Boundary(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("velocity", C.c_float * 3), ("restore", C.c_float), ("radius", C.c_float)]


def boundary(kind, velocity=(0.0, 0.0, 0.0), restore=1.0, radius=0.0):
    b = Boundary()
    b.kind = kind
    for k in range(3):
        b.velocity[k] = float(velocity[k])
    b.restore = restore
    b.radius = radius
    return b


class Reductions(C.Structure):
    _fields_ = [
        ("epot", C.c_double), ("epot_nonbond", C.c_double), ("epot_bond", C.c_double),
        ("epot_angle", C.c_double), ("kinetic", C.c_double), ("virial", C.c_double),
        ("computed_volume", C.c_double), ("species_total", C.c_double * 8),
        ("steps", C.c_int64), ("migrations", C.c_int64),
    ]


P_POT = C.POINTER(Potential)
F_P = C.POINTER(C.c_float)
I_P = C.POINTER(C.c_int32)
U_P = C.POINTER(C.c_uint32)
V_P = C.c_void_p


def engine_desc(origin, dim, cells, cutoff, dt, max_type=1, nr_species=0,
                particle_max_dist_fraction=0.05, seed=0x5EED, capacity=0,
                max_bonds=0, max_angles=0, device=0, flags=0, nr_fluxsteps=1):
    d = EngineDesc()
    for k in range(3):
        d.origin[k] = float(origin[k])
        d.dim[k] = float(dim[k])
        d.cells[k] = int(cells[k])
    d.cutoff = cutoff
    d.dt = dt
    d.max_type = max_type
    d.nr_species = nr_species
    d.particle_max_dist_fraction = particle_max_dist_fraction
    d.seed = seed
    d.capacity = capacity
    d.max_bonds = max_bonds
    d.max_angles = max_angles
    d.nr_fluxsteps = nr_fluxsteps
    d.device = device
    d.flags = flags
    return d


def declare_potential_api(lib):
    """Prototypes of the table-construction entry points (shared by every lib that exports them)."""
    pp = C.POINTER(P_POT)
    lib.tfg_potential_morse.argtypes = [C.c_float] * 6 + [C.c_int, pp]
    lib.tfg_potential_lennard_jones_12_6.argtypes = [C.c_float] * 5 + [pp]
    lib.tfg_potential_harmonic.argtypes = [C.c_float] * 5 + [pp]
    lib.tfg_potential_harmonic_angle.argtypes = [C.c_float] * 5 + [pp]
    lib.tfg_potential_dpd.argtypes = [C.c_float] * 4 + [C.c_int, pp]
    lib.tfg_potential_free.argtypes = [P_POT]
    lib.tfg_potential_free.restype = None
    lib.tfg_potential_eval.argtypes = [P_POT, C.c_float, C.c_float, C.c_float, F_P, F_P]
