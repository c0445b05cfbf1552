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
BOUNDARY_RESETTING = 1 << 5

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


# ---- serving (tfg_server_*, tfg_request_*) ----
SERVER_LEAST_WORK = 0
SERVER_FIFO = 1
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class ServerDesc(C.Structure):
    _fields_ = [("device", C.c_int32), ("quantum", C.c_int32), ("budget_bytes", C.c_int64),
                ("max_particles", C.c_int64), ("policy", C.c_int32), ("discard_results", C.c_int32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("queued", C.c_int64), ("running", C.c_int64), ("particles_in_flight", C.c_int64),
                ("bytes_in_flight", C.c_int64), ("max_concurrent", C.c_int64), ("chunks", C.c_int64),
                ("admit_s", C.c_double), ("launch_s", C.c_double), ("retire_s", C.c_double),
                ("busy_s", C.c_double), ("gap_s", C.c_double)]


def declare_server_api(lib):
    """Prototypes of the serving entry points (the product library, or a test build of the
    same server code over a stand-in batch)."""
    S = R = C.c_void_p
    i64p = C.POINTER(C.c_int64)
    ip = C.POINTER(C.c_int)
    lib.tfg_server_create.argtypes = [C.POINTER(ServerDesc), C.POINTER(S)]
    lib.tfg_server_destroy.argtypes = [S]
    lib.tfg_server_last_error.argtypes = [S]
    lib.tfg_server_last_error.restype = C.c_char_p
    lib.tfg_request_create.argtypes = [C.POINTER(EngineDesc), C.c_int, C.c_int, C.c_int, C.POINTER(R)]
    lib.tfg_request_free.argtypes = [R]
    lib.tfg_request_set_type.argtypes = [R, C.c_int, C.c_int, C.c_float]
    lib.tfg_request_set_potential.argtypes = [R, C.c_int, C.c_int, P_POT]
    lib.tfg_request_add_flux.argtypes = [R, C.c_int, C.c_int, C.POINTER(Flux)]
    lib.tfg_request_set_species_flags.argtypes = [R, C.c_int, U_P]
    lib.tfg_request_set_random_force.argtypes = [R, C.c_int, C.c_float, C.c_float, C.c_int]
    lib.tfg_request_set_species_reset.argtypes = [R, C.c_int, F_P]
    lib.tfg_request_set_boundary.argtypes = [R, C.c_int, C.POINTER(Boundary)]
    lib.tfg_request_set_boundary_potential.argtypes = [R, C.c_int, C.c_int, P_POT]
    lib.tfg_request_set_bonded_potential.argtypes = [R, C.c_int, P_POT]
    lib.tfg_request_load_particles.argtypes = [R, C.c_int, F_P, F_P, I_P, F_P, F_P, U_P, F_P, F_P]
    lib.tfg_request_load_bonds.argtypes = [R, C.c_int, I_P, I_P, I_P]
    lib.tfg_request_load_angles.argtypes = [R, C.c_int, I_P, I_P, I_P, I_P]
    lib.tfg_server_submit.argtypes = [S, R, i64p]
    lib.tfg_server_poll.argtypes = [S, C.c_int, ip]
    lib.tfg_server_take_finished.argtypes = [S, i64p, C.c_int, ip]
    lib.tfg_server_request_info.argtypes = [S, C.c_int64, ip, ip, C.POINTER(C.c_double)]
    lib.tfg_server_result.argtypes = [S, C.c_int64, ip, F_P, F_P, F_P, C.POINTER(Reductions)]
    lib.tfg_server_release.argtypes = [S, C.c_int64]
    lib.tfg_server_get_stats.argtypes = [S, C.POINTER(ServerStats)]
