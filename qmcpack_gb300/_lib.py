"""ctypes binding of libqmcg.so (the C ABI declared in include/qmcg.h)."""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqmcg.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

# every symbol the header declares, in declaration order
EXPORTS = [
    "qmcg_last_error", "qmcg_device_count", "qmcg_system_create", "qmcg_system_destroy",
    "qmcg_crowd_create", "qmcg_crowd_destroy", "qmcg_crowd_stream", "qmcg_load_walkers",
    "qmcg_get_positions", "qmcg_mw_evaluate_log", "qmcg_mw_recompute_walkers", "qmcg_mw_prepare_group", "qmcg_mw_eval_grad",
    "qmcg_mw_make_move", "qmcg_mw_calc_ratio_grad", "qmcg_mw_accept_reject_move",
    "qmcg_mw_complete_updates", "qmcg_get_log", "qmcg_get_inverse", "qmcg_get_jastrow_state",
    "qmcg_get_phi_vgl", "qmcg_vmc_sweeps", "qmcg_vmc_sweeps_async", "qmcg_vmc_sweeps_host", "qmcg_crowd_sync",
    "qmcg_mw_update_inv_mat", "qmcg_mw_update_inv_mat_ex", "qmcg_mw_update_inv_mat_noalloc", "qmcg_profile_ratio",
    "qmcg_profile_sweep", "qmcg_sweep_info", "qmcg_mw_evaluate_local_energy", "qmcg_vmc_sweeps_measure",
    "qmcg_proposal_init", "qmcg_proposal_get_params", "qmcg_proposal_set_params", "qmcg_proposal_forward",
    "qmcg_proposal_backward", "qmcg_proposal_features", "qmcg_vmc_sweeps_learned",
    "qmcg_group_create", "qmcg_group_destroy", "qmcg_group_sweeps", "qmcg_group_info", "qmcg_crowd_set_threads",
    "qmcg_mw_evaluate_gl", "qmcg_vmc_sweeps_trace", "qmcg_profile_recompute",
    "qmcg_dmc_init", "qmcg_dmc_step", "qmcg_dmc_copy_walkers", "qmcg_dmc_comb", "qmcg_dmc_reconfigure",
    "qmcg_mw_evaluate_ratios", "qmcg_profile_ratios", "qmcg_spline_from_planewaves",
]
TRACE_FIELDS = 12
PROPOSAL_NUM_PARAMS = 43408
_fp = C.POINTER(C.c_float)


class SystemDesc(C.Structure):
    _fields_ = [
        ("precision", C.c_int), ("n_up", C.c_int), ("n_dn", C.c_int), ("num_orbitals", C.c_int),
        ("num_orbitals_padded", C.c_int), ("lattice", C.c_double * 3), ("num_ions", C.c_int),
        ("ion_pos", _dp), ("ion_species", _ip), ("num_ion_species", C.c_int), ("grid", C.c_int * 3),
        ("spline_coefs", C.c_void_p), ("j1_num_params", C.c_int), ("j1_rcut", C.c_double),
        ("j1_params", _dp), ("j1_cusp", _dp), ("j2_num_params", C.c_int), ("j2_rcut", C.c_double),
        ("j2_params", _dp), ("j2_cusp", _dp), ("ion_charges", _dp),
    ]


class SweepParams(C.Structure):
    _fields_ = [("tau", C.c_double), ("use_drift", C.c_int), ("rng_mode", C.c_int), ("seed", C.c_uint64),
                ("recompute_every", C.c_int), ("path", C.c_int), ("flush", C.c_int)]


class BranchParams(C.Structure):
    _fields_ = [("e_trial", C.c_double), ("e_ref", C.c_double), ("tau_eff", C.c_double),
                ("branch_cutoff", C.c_double), ("branch_max", C.c_double)]


class SweepStats(C.Structure):
    _fields_ = [("accepted", C.c_uint64), ("rejected", C.c_uint64), ("repaired", C.c_uint64), ("status", C.c_int)]


_LIB = None


class QmcgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"qmcg error {code}: {msg}")
        self.code = code


def load(path: str = LIB_PATH):
    """Load the CUDA library; raises if it has not been built (no CPU fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with python -m qmcpack_gb300.build "
                          "(the move loop has no CPU fallback)")
    L = C.CDLL(path)
    L.qmcg_last_error.restype = C.c_char_p
    vp = C.c_void_p
    sig = {
        "qmcg_device_count": [_ip],
        "qmcg_system_create": [C.POINTER(SystemDesc), C.POINTER(vp)],
        "qmcg_system_destroy": [vp],
        "qmcg_crowd_create": [vp, C.c_int, C.c_int, C.POINTER(vp)],
        "qmcg_crowd_destroy": [vp],
        "qmcg_crowd_stream": [vp, C.POINTER(vp)],
        "qmcg_load_walkers": [vp, _dp],
        "qmcg_get_positions": [vp, _dp],
        "qmcg_mw_evaluate_log": [vp, _dp, _ip],
        "qmcg_mw_recompute_walkers": [vp, _ip],
        "qmcg_mw_prepare_group": [vp, C.c_int],
        "qmcg_mw_eval_grad": [vp, C.c_int, _dp],
        "qmcg_mw_make_move": [vp, C.c_int, _dp, _ip],
        "qmcg_mw_calc_ratio_grad": [vp, C.c_int, _dp, _dp],
        "qmcg_mw_accept_reject_move": [vp, C.c_int, _ip],
        "qmcg_mw_complete_updates": [vp],
        "qmcg_get_log": [vp, _dp, _ip, _dp],
        "qmcg_get_inverse": [vp, C.c_int, _dp],
        "qmcg_get_jastrow_state": [vp, _dp, _dp],
        "qmcg_get_phi_vgl": [vp, _dp],
        "qmcg_vmc_sweeps": [vp, C.POINTER(SweepParams), C.c_int, C.POINTER(SweepStats), _ip],
        "qmcg_vmc_sweeps_async": [vp, C.c_int],
        "qmcg_vmc_sweeps_host": [vp, C.POINTER(SweepParams), C.c_int, _dp, _dp, _dp, C.POINTER(SweepStats)],
        "qmcg_crowd_sync": [vp, C.POINTER(SweepStats)],
        "qmcg_profile_ratio": [vp, C.c_int, _dp],
        "qmcg_profile_sweep": [vp, C.c_int, _dp],
        "qmcg_sweep_info": [vp, C.c_int, _ip],
        "qmcg_mw_evaluate_local_energy": [vp, _dp, _dp, _dp],
        "qmcg_vmc_sweeps_measure": [vp, C.POINTER(SweepParams), C.c_int, _dp, _dp, C.POINTER(SweepStats)],
        "qmcg_proposal_init": [vp, C.c_uint64, C.c_double],
        "qmcg_proposal_get_params": [vp, _fp],
        "qmcg_proposal_set_params": [vp, _fp],
        "qmcg_proposal_forward": [vp, C.c_int, _fp, _fp, _fp],
        "qmcg_proposal_backward": [vp, C.c_int, _fp, _fp, _fp],
        "qmcg_proposal_features": [vp, C.c_int, C.c_int, _fp],
        "qmcg_vmc_sweeps_learned": [vp, C.POINTER(SweepParams), C.c_int, C.c_int, C.c_double, _dp,
                                    C.POINTER(SweepStats), _dp],
        "qmcg_group_create": [C.POINTER(vp), C.c_int, C.POINTER(vp)],
        "qmcg_group_destroy": [vp],
        "qmcg_group_sweeps": [vp, C.POINTER(SweepParams), C.c_int, C.POINTER(SweepStats)],
        "qmcg_group_info": [vp, _ip],
        "qmcg_crowd_set_threads": [vp, C.c_int],
        "qmcg_mw_evaluate_gl": [vp, _dp, _dp, _dp],
        "qmcg_vmc_sweeps_trace": [vp, C.POINTER(SweepParams), C.c_int, C.POINTER(SweepStats), _dp],
        "qmcg_profile_recompute": [vp, _dp],
        "qmcg_dmc_init": [vp, _dp],
        "qmcg_dmc_step": [vp, C.POINTER(SweepParams), C.POINTER(BranchParams), _dp, _dp, _ip, _dp,
                          C.POINTER(SweepStats), _dp],
        "qmcg_dmc_copy_walkers": [vp, _ip],
        "qmcg_dmc_comb": [C.c_int, _dp, C.c_double, _ip, _ip],
        "qmcg_dmc_reconfigure": [vp, C.c_double, _ip],
        "qmcg_mw_evaluate_ratios": [vp, C.c_int, _ip, _ip, _dp, _dp],
        "qmcg_profile_ratios": [vp, C.c_int, _ip, _ip, _dp, C.c_int, _dp],
        "qmcg_spline_from_planewaves": [C.c_int, C.c_int, C.c_int, _ip, _dp, _ip, C.c_int, vp, _dp],
        "qmcg_mw_update_inv_mat": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp],
        "qmcg_mw_update_inv_mat_ex": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp,
                                      C.c_int, vp],
        "qmcg_mw_update_inv_mat_noalloc": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp,
                                           vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    _LIB = L
    return L


def check(rc: int):
    if rc != 0:
        raise QmcgError(rc, load().qmcg_last_error().decode())
