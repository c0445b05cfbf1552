"""Loader of the in-tree libtfg.so.  There is no fallback: if the library is missing the
import of an engine fails loudly."""
import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(_HERE)


def lib_path():
    return os.path.join(_PKG, "_build", "libtfg.so")


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise RuntimeError("libtfg.so is not built (%s); run __graft_entry__.build() or "
                           "python tissue-forge_gb300/build.py" % path)
    L = C.CDLL(path)
    E = C.c_void_p
    abi.declare_potential_api(L)
    L.tfg_build_info.restype = C.c_char_p
    L.tfg_last_error.argtypes = [E]
    L.tfg_last_error.restype = C.c_char_p
    L.tfg_engine_create.argtypes = [C.POINTER(abi.EngineDesc), C.POINTER(E)]
    L.tfg_engine_destroy.argtypes = [E]
    L.tfg_engine_set_stream.argtypes = [E, C.c_void_p]
    L.tfg_set_type.argtypes = [E, C.c_int, C.c_int, C.c_float]
    L.tfg_set_potential.argtypes = [E, C.c_int, C.c_int, abi.P_POT]
    L.tfg_add_flux.argtypes = [E, C.c_int, C.c_int, C.POINTER(abi.Flux)]
    L.tfg_set_species_flags.argtypes = [E, C.c_int, abi.U_P]
    L.tfg_set_species_reset.argtypes = [E, C.c_int, abi.F_P]
    L.tfg_batch_set_species_reset.argtypes = [E, C.c_int, C.c_int, abi.F_P]
    L.tfg_set_stop.argtypes = [E, C.c_int64]
    L.tfg_batch_set_stop.argtypes = [E, C.c_int, C.c_int64]
    L.tfg_set_random_force.argtypes = [E, C.c_int, C.c_float, C.c_float, C.c_int]
    L.tfg_load_particles.argtypes = [E, C.c_int, abi.F_P, abi.F_P, abi.I_P, abi.F_P, abi.F_P, abi.U_P, abi.F_P,
                                     abi.F_P]
    L.tfg_load_particles_binned.argtypes = [E, C.c_int, abi.I_P, abi.F_P, abi.F_P, abi.I_P, abi.F_P, abi.F_P,
                                            abi.U_P, abi.F_P, abi.F_P]
    L.tfg_set_bonded_potential.argtypes = [E, C.c_int, abi.P_POT]
    L.tfg_load_bonds.argtypes = [E, C.c_int, abi.I_P, abi.I_P, abi.I_P]
    L.tfg_load_angles.argtypes = [E, C.c_int, abi.I_P, abi.I_P, abi.I_P, abi.I_P]
    L.tfg_step.argtypes = [E, C.c_int]
    L.tfg_force_only.argtypes = [E, C.c_int]
    L.tfg_sync.argtypes = [E]
    L.tfg_query.argtypes = [E, C.POINTER(C.c_int)]
    L.tfg_set_graphs.argtypes = [E, C.c_int]
    L.tfg_pair_signature.argtypes = [E, abi.I_P, abi.U_P]
    L.tfg_pair_list.argtypes = [E, C.c_int64, abi.I_P, C.POINTER(C.c_int64)]
    L.tfg_autotune.argtypes = [E, C.POINTER(C.c_int)]
    L.tfg_set_split.argtypes = [E, C.c_int]
    L.tfg_get_tuning.argtypes = [E, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.tfg_set_tuning.argtypes = [E, C.c_int, C.c_int, C.c_int]
    L.tfg_get_count.argtypes = [E, C.POINTER(C.c_int)]
    L.tfg_download.argtypes = [E, abi.F_P, abi.F_P, abi.I_P, abi.F_P, abi.F_P, abi.F_P, abi.F_P, abi.F_P]
    L.tfg_get_reductions.argtypes = [E, C.POINTER(abi.Reductions)]
    L.tfg_get_verlet.argtypes = [E, C.POINTER(C.c_int64), C.POINTER(C.c_float)]
    L.tfg_set_pair_lists.argtypes = [E, C.c_int]
    L.tfg_get_phase_ms.argtypes = [E, C.POINTER(C.c_float)]
    L.tfg_set_phase_timing.argtypes = [E, C.c_int]
    L.tfg_probe_fp32_tflops.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.tfg_bin_noalloc.argtypes = [C.POINTER(abi.EngineDesc), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p]
    L.tfg_set_boundary.argtypes = [E, C.c_int, C.POINTER(abi.Boundary)]
    L.tfg_set_boundary_potential.argtypes = [E, C.c_int, C.c_int, abi.P_POT]
    L.tfg_batch_set_boundary.argtypes = [E, C.c_int, C.c_int, C.POINTER(abi.Boundary)]
    L.tfg_batch_set_boundary_potential.argtypes = [E, C.c_int, C.c_int, C.c_int, abi.P_POT]
    L.tfg_batch_create.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(E)]
    L.tfg_batch_add_sim.argtypes = [E, C.POINTER(abi.EngineDesc), C.POINTER(C.c_int)]
    L.tfg_batch_remove_sim.argtypes = [E, C.c_int]
    L.tfg_batch_sim_count.argtypes = [E, C.POINTER(C.c_int)]
    L.tfg_batch_step.argtypes = [E, C.c_int]
    L.tfg_batch_set_type.argtypes = [E, C.c_int, C.c_int, C.c_int, C.c_float]
    L.tfg_batch_set_potential.argtypes = [E, C.c_int, C.c_int, C.c_int, abi.P_POT]
    L.tfg_batch_add_flux.argtypes = [E, C.c_int, C.c_int, C.c_int, C.POINTER(abi.Flux)]
    L.tfg_batch_set_species_flags.argtypes = [E, C.c_int, C.c_int, abi.U_P]
    L.tfg_batch_set_random_force.argtypes = [E, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int]
    L.tfg_batch_load_particles.argtypes = [E, C.c_int, C.c_int, abi.F_P, abi.F_P, abi.I_P, abi.F_P, abi.F_P,
                                           abi.U_P, abi.F_P, abi.F_P]
    L.tfg_batch_load_particles_binned.argtypes = [E, C.c_int, C.c_int, abi.I_P, abi.F_P, abi.F_P, abi.I_P,
                                                  abi.F_P, abi.F_P, abi.U_P, abi.F_P, abi.F_P]
    L.tfg_batch_load_bonds.argtypes = [E, C.c_int, C.c_int, abi.I_P, abi.I_P, abi.I_P]
    L.tfg_batch_load_angles.argtypes = [E, C.c_int, C.c_int, abi.I_P, abi.I_P, abi.I_P, abi.I_P]
    L.tfg_batch_get_count.argtypes = [E, C.c_int, C.POINTER(C.c_int)]
    L.tfg_batch_download.argtypes = [E, C.c_int, abi.F_P, abi.F_P, abi.I_P, abi.F_P, abi.F_P, abi.F_P, abi.F_P,
                                     abi.F_P]
    L.tfg_batch_get_reductions.argtypes = [E, C.c_int, C.POINTER(abi.Reductions)]
    L.tfg_batch_get_verlet.argtypes = [E, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_float)]
    L.tfg_batch_sim_status.argtypes = [E, C.c_int, C.POINTER(C.c_int)]
    L.tfg_batch_resume.argtypes = [E, C.c_int, C.c_int64, abi.F_P]
    L.tfg_set_deterministic.argtypes = [E, C.c_int]
    abi.declare_server_api(L)
    _lib = L
    return L
