"""ctypes binding of the C ABI declared in include/atm_capi.h.

The shared library is built in-tree by ``build.py`` (or ``__graft_entry__.build()``)
into ``_build/libatmgb300.so`` next to this package.  There is no fallback: if
the library is missing, importing the API raises.
"""
from __future__ import annotations

import ctypes as C
import os

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libatmgb300.so")

NUM_RES = 17
RES_KEYS = ("energy", "pert", "sp", "W", "u", "e0", "bfp", "fp", "E1", "E2",
            "dW_dlambda1", "dW_dlambda2", "dW_dalpha", "dW_du0", "dW_dw0", "status", "dW_du")

ATM_ERRORS = {
    1: "invalid argument", 2: "index out of range", 3: "invalid state", 4: "CUDA failure",
    5: "unsupported", 6: "capacity overflow", 7: "XML parse error", 8: "force group conflict",
    9: "particle set changed", 10: "constraints did not converge",
}


class ATMError(Exception):
    """Raised for a non-zero status of the C ABI (the reference's SWIG layer
    raises ``Exception`` from C++ exceptions, python/atmmetaforceplugin.i:54-61)."""

    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p
_sz = C.c_size_t

# name -> argtypes (all return int status unless listed in _RESTYPES)
_SIGS = {
    "atm_force_create": [C.c_double] * 9 + [_ip, C.c_int, C.POINTER(_vp)],
    "atm_force_destroy": [_vp],
    "atm_force_add_particle": [_vp, C.c_int, C.c_double, C.c_double, C.c_double, _ip],
    "atm_force_get_particle_parameters": [_vp, C.c_int, _ip, _dp, _dp, _dp],
    "atm_force_set_particle_parameters": [_vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double],
    "atm_force_get_num_particles": [_vp, _ip],
    "atm_force_get_default": [_vp, C.c_int, _dp],
    "atm_force_get_variable_force_groups": [_vp, _ip, C.c_int, _ip],
    "atm_force_set_force_group": [_vp, C.c_int],
    "atm_force_get_force_group": [_vp, _ip],
    "atm_force_set_name": [_vp, C.c_char_p],
    "atm_force_get_name": [_vp, C.c_char_p, _sz, C.POINTER(_sz)],
    "atm_force_uses_periodic_boundary_conditions": [_vp, _ip],
    "atm_force_update_parameters_in_context": [_vp, _vp],
    "atm_force_get_perturbation_energy": [_vp, _vp, _dp],
    "atm_force_serialize": [_vp, C.c_char_p, _sz, C.POINTER(_sz)],
    "atm_force_deserialize": [C.c_char_p, C.POINTER(_vp)],
    "atm_nonbonded_create": [C.POINTER(_vp)],
    "atm_nonbonded_destroy": [_vp],
    "atm_nonbonded_add_particle": [_vp, C.c_double, C.c_double, C.c_double, _ip],
    "atm_nonbonded_set_particle_parameters": [_vp, C.c_int, C.c_double, C.c_double, C.c_double],
    "atm_nonbonded_get_particle_parameters": [_vp, C.c_int, _dp, _dp, _dp],
    "atm_nonbonded_get_num_particles": [_vp, _ip],
    "atm_nonbonded_add_exception": [_vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _ip],
    "atm_nonbonded_get_num_exceptions": [_vp, _ip],
    "atm_nonbonded_set_method": [_vp, C.c_int],
    "atm_nonbonded_set_cutoff": [_vp, C.c_double],
    "atm_nonbonded_set_reaction_field_dielectric": [_vp, C.c_double],
    "atm_nonbonded_set_ewald_error_tolerance": [_vp, C.c_double],
    "atm_nonbonded_set_pme_parameters": [_vp, C.c_double, C.c_int, C.c_int, C.c_int],
    "atm_nonbonded_set_use_dispersion_correction": [_vp, C.c_int],
    "atm_nonbonded_set_force_group": [_vp, C.c_int],
    "atm_nonbonded_get_force_group": [_vp, _ip],
    "atm_system_create": [C.POINTER(_vp)],
    "atm_system_destroy": [_vp],
    "atm_system_add_particle": [_vp, C.c_double, _ip],
    "atm_system_get_num_particles": [_vp, _ip],
    "atm_system_set_default_periodic_box_vectors": [_vp, _dp, _dp, _dp],
    "atm_system_add_nonbonded": [_vp, _vp],
    "atm_system_add_atm_force": [_vp, _vp],
    "atm_system_add_constraint": [_vp, C.c_int, C.c_int, C.c_double, _ip],
    "atm_system_get_num_constraints": [_vp, _ip],
    "atm_system_add_bond": [_vp, C.c_int, C.c_int, C.c_double, C.c_double],
    "atm_system_add_angle": [_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double],
    "atm_system_add_centroid_restraint": [_vp, C.c_int, _ip, C.c_int, _ip, C.c_double, C.c_double, _dp],
    "atm_system_add_position_restraint": [_vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_double],
    "atm_system_set_position_restraints_periodic": [_vp, C.c_int],
    "atm_context_create": [_vp, C.c_int, C.c_char_p, C.POINTER(_vp)],
    "atm_context_destroy": [_vp],
    "atm_context_set_positions": [_vp, _dp, C.c_int],
    "atm_context_set_periodic_box_vectors": [_vp, _dp, _dp, _dp],
    "atm_context_set_parameter": [_vp, C.c_char_p, C.c_double],
    "atm_context_get_parameter": [_vp, C.c_char_p, _dp],
    "atm_context_get_state": [_vp, C.c_int, _dp, _dp],
    "atm_context_get_results": [_vp, _dp],
    "atm_batch_create": [C.POINTER(_vp), C.c_int, C.c_int, C.c_char_p, C.POINTER(_vp)],
    "atm_batch_destroy": [_vp],
    "atm_batch_get_num_replicas": [_vp, _ip],
    "atm_batch_get_num_particles": [_vp, C.c_int, _ip],
    "atm_batch_set_positions": [_vp, C.c_int, _dp],
    "atm_batch_set_parameter": [_vp, C.c_int, C.c_char_p, C.c_double],
    "atm_batch_set_periodic_box_vectors": [_vp, C.c_int, _dp, _dp, _dp],
    "atm_batch_evaluate": [_vp, _dp, _dp, _dp, _dp],
    "atm_batch_evaluate_device": [_vp, _vp, _vp, _vp, _vp],
    "atm_batch_energy_matrix": [_vp, C.c_double, _dp],
    "atm_batch_get_list_info": [_vp, _dp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)],
    "atm_md_autotune": [_vp, C.c_int, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)],
    "atm_md_get_list_info": [_vp, _dp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), _ip],
    "atm_batch_set_displacements": [_vp, C.c_int, _dp],
    "atm_batch_set_nonbonded_parameters": [_vp, C.c_int, _dp, _dp, _dp],
    "atm_batch_backward_device": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "atm_batch_backward": [_vp, _dp, _dp, _dp, _dp, _dp, _dp, _dp],
    "atm_batch_set_profiling": [_vp, C.c_int],
    "atm_batch_autotune": [_vp, C.c_int, C.c_int, C.c_char_p, _sz, C.POINTER(_sz)],
    "atm_batch_get_kernel_times": [_vp, C.c_char_p, _sz, _dp, C.c_int, _ip],
    "atm_batch_get_launch_count": [_vp, _ip],
    "atm_batch_get_stats": [_vp, _ip, _ip, _ip],
    "atm_md_create": [C.POINTER(_vp), C.c_int, C.c_int, C.c_char_p, C.c_double, C.c_double, C.c_double,
                      C.c_ulonglong, C.POINTER(_vp)],
    "atm_md_destroy": [_vp],
    "atm_md_get_num_particles": [_vp, _ip],
    "atm_md_set_positions": [_vp, _dp],
    "atm_md_set_velocities": [_vp, _dp],
    "atm_md_set_velocities_to_temperature": [_vp, C.c_double, C.c_ulonglong],
    "atm_md_set_parameter": [_vp, C.c_int, C.c_char_p, C.c_double],
    "atm_md_set_integrator": [_vp, C.c_double, C.c_double, C.c_double],
    "atm_md_step": [_vp, C.c_int],
    "atm_md_get_state": [_vp, _dp, _dp, _dp, _dp, _dp, _dp],
    "atm_md_get_info": [_vp, C.POINTER(C.c_longlong), _ip, _ip],
    "atm_md_set_recording": [_vp, C.c_int, C.c_int],
    "atm_md_get_records": [_vp, C.POINTER(C.c_longlong), _dp, _dp, C.c_int, _ip],
    "atm_rf_nonbonded_noalloc": [C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _dp, C.c_double, C.c_double, _vp, _vp,
                                 _vp],
}
_RESTYPES = {
    "atm_last_error": C.c_char_p,
    "atm_version": C.c_char_p,
    "atm_global_name": C.c_char_p,
}
_NOARG = {"atm_last_error": [], "atm_version": [], "atm_global_name": [C.c_int]}

_lib = None


def exported_names():
    return sorted(list(_SIGS) + list(_RESTYPES))


def load():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python build.py` in {PKG_ROOT}")
    L = C.CDLL(LIB_PATH)
    for name, args in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    for name, rt in _RESTYPES.items():
        fn = getattr(L, name)
        fn.argtypes = _NOARG[name]
        fn.restype = rt
    _lib = L
    return L


def check(status):
    if status != 0:
        msg = load().atm_last_error().decode()
        raise ATMError(status, msg or ATM_ERRORS.get(status, f"error {status}"))


def call(name, *args):
    check(getattr(load(), name)(*args))
