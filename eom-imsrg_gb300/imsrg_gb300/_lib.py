"""ctypes binding of libimsrg_gb300.so (the C ABI of include/imsrg_gb300.h).

The library is built in-tree (eom-imsrg_gb300/build.py).  There is no fallback: if the
shared library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libimsrg_gb300.so")

IMSRG_OK = 0
STATUS_NAMES = {
    0: "IMSRG_OK", 1: "IMSRG_ERR_INVALID_ARGUMENT", 2: "IMSRG_ERR_CUDA", 3: "IMSRG_ERR_OUT_OF_MEMORY",
    4: "IMSRG_ERR_NOT_CONVERGED", 5: "IMSRG_ERR_MISMATCH", 6: "IMSRG_ERR_UNSUPPORTED", 7: "IMSRG_ERR_TIMEOUT",
}
PREC = {"fp64": 0, "bf16x3": 1, "bf16x6": 2, "tf32x3": 3}
COMM_E0 = 1


class ImsrgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class Basis_t(C.Structure):
    _fields_ = [("norbits", C.c_int32), ("nn", C.POINTER(C.c_int32)), ("ll", C.POINTER(C.c_int32)),
                ("jj", C.POINTER(C.c_int32)), ("itzp", C.POINTER(C.c_int32)), ("con", C.POINTER(C.c_int32)),
                ("eMax", C.c_int32), ("lMax", C.c_int32), ("hw", C.c_double), ("Aprot", C.c_int32),
                ("Aneut", C.c_int32)]


class HFInfo_t(C.Structure):
    _fields_ = [("e_hf", C.c_double), ("crit", C.c_double), ("iterations", C.c_int32)]


class TuneInfo_t(C.Structure):
    _fields_ = [("tiny_cap", C.c_int32), ("small_cap", C.c_int32), ("recouple_ctas", C.c_int32),
                ("gemm_order", C.c_int32), ("gemm_wmax", C.c_int32), ("gemm_narrow", C.c_int32),
                ("ms_before", C.c_double), ("ms_after", C.c_double), ("recouple_kind", C.c_int32),
                ("recouple_min_blocks", C.c_int32), ("gemm_merged", C.c_int32), ("gemm_wmax_x", C.c_int32),
                ("gemm_narrow_x", C.c_int32)]


class StepInfo_t(C.Structure):
    _fields_ = [("E0", C.c_double), ("mbpt2", C.c_double), ("magnus_terms", C.c_int32), ("bch_terms", C.c_int32),
                ("bch_converged", C.c_int32), ("graph_rebuilt", C.c_int32)]


# (name, restype-is-status, argtypes)
_vp, _i32, _i64, _d, _u64 = C.c_void_p, C.c_int32, C.c_int64, C.c_double, C.c_uint64
_pi32, _pi64, _pd, _pvp = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_void_p)
SIGNATURES = {
    "imsrg_ctx_create": [C.POINTER(Basis_t), _i32, _pvp],
    "imsrg_ctx_destroy": [_vp],
    "imsrg_ctx_sizes": [_vp, _pi64, _pi64, _pi64, _pi32, _pi32],
    "imsrg_block_info": [_vp, _pi32, _pi32, _pi32, _pi32, _pi32, _pi32],
    "imsrg_block_pairs": [_vp, _i32, _i32, _pi32],
    "imsrg_cc_info": [_vp, _pi32, _pi32, _pi32],
    "imsrg_set_precision": [_vp, _i32],
    "imsrg_autotune": [_vp, _vp, _vp, _vp, C.POINTER(TuneInfo_t)],
    "imsrg_synchronize": [_vp],
    "imsrg_op_create": [_vp, _i32, _pvp],
    "imsrg_op_destroy": [_vp, _vp],
    "imsrg_op_set_herm": [_vp, _vp, _i32],
    "imsrg_op_get_herm": [_vp, _vp, _pi32],
    "imsrg_op_upload": [_vp, _vp, _pvp, _pd, _pd, _pd, _d],
    "imsrg_op_download": [_vp, _vp, _pvp, _pd, _pd, _pd, _pd],
    "imsrg_op_upload_slab": [_vp, _vp, _vp],
    "imsrg_op_download_slab": [_vp, _vp, _vp],
    "imsrg_op_device_slab": [_vp, _vp, C.POINTER(C.c_void_p)],
    "imsrg_op_get_e0": [_vp, _vp, _pd],
    "imsrg_pinned_alloc": [_i64, _pvp],
    "imsrg_pinned_free": [_vp],
    "imsrg_copy_sq_op": [_vp, _vp, _vp],
    "imsrg_clear_sq_op": [_vp, _vp],
    "imsrg_add_sq_op": [_vp, _vp, _d, _vp, _d, _vp],
    "imsrg_scale_sq_op": [_vp, _vp, _d],
    "imsrg_mat_frob_norm": [_vp, _vp, _pd],
    "imsrg_mbpt2": [_vp, _vp, _pd],
    "imsrg_check_conversions": [_vp, _vp, _vp, _i64, _vp, _vp],
    "imsrg_cc_create": [_vp, _i32, _pvp],
    "imsrg_cc_destroy": [_vp, _vp],
    "imsrg_cc_download": [_vp, _vp, _vp],
    "imsrg_calculate_cross_coupled": [_vp, _vp, _vp],
    "imsrg_commutator_110": [_vp, _vp, _vp, _pd],
    "imsrg_commutator_111": [_vp, _vp, _vp, _vp],
    "imsrg_commutator_121": [_vp, _vp, _vp, _vp],
    "imsrg_commutator_122": [_vp, _vp, _vp, _vp],
    "imsrg_commutator_220": [_vp, _vp, _vp, _pd],
    "imsrg_commutator_221": [_vp, _vp, _vp, _vp, _vp, _vp],
    "imsrg_commutator_222_pp_hh": [_vp, _vp, _vp, _vp, _vp, _vp],
    "imsrg_commutator_222_ph": [_vp, _vp, _vp, _vp, _vp],
    "imsrg_commutator": [_vp, _vp, _vp, _vp, _i32],
    "imsrg_build_gs_white": [_vp, _vp, _vp],
    "imsrg_build_gs_atan": [_vp, _vp, _vp],
    "imsrg_build_gs_atanxx": [_vp, _vp, _vp, _vp],
    "imsrg_build_gs_w2": [_vp, _vp, _vp],
    "imsrg_magnus_expand": [_vp, _vp, _vp, _pi32],
    "imsrg_euler_step": [_vp, _vp, _vp, _pd, _d],
    "imsrg_bch_expand": [_vp, _vp, _vp, _vp, _i32, _d, _pi32],
    "imsrg_cr_expand": [_vp, _vp, _vp, _vp, _i32, _d, _pi32],
    "imsrg_bch_expand_quads": [_vp, _vp, _vp, _vp, _i32, _d, _pi32],
    "imsrg_restore_quadrupoles": [_vp, _vp, _vp, _vp],
    "imsrg_magnus_step": [_vp, _vp, _vp, _vp, _vp, _d, _i32, _d, _i32, C.POINTER(StepInfo_t)],
    "imsrg_magnus_step_host": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _i32, _d, _i32, C.POINTER(StepInfo_t)],
    "imsrg_magnus_step_counters": [_vp, _pi64, _pi64, _pi64, _pi64],
    "imsrg_tensor_sizes": [_vp, _i32, _i32, _pi64, _pi32],
    "imsrg_tensor_block_info": [_vp, _i32, _i32, _pi32, _pi32, _pi32, _pi32],
    "imsrg_tensor_create": [_vp, _i32, _i32, _i32, _pvp],
    "imsrg_tensor_destroy": [_vp, _vp],
    "imsrg_tensor_upload_slab": [_vp, _vp, _vp],
    "imsrg_tensor_download_slab": [_vp, _vp, _vp],
    "imsrg_tensor_commutator": [_vp, _vp, _vp, _vp, _i32],
    "imsrg_bch_tensor": [_vp, _vp, _vp, _i32, _d, _pi32],
    "imsrg_tensor_frob_norm": [_vp, _vp, _pd],
    "imsrg_restore_triples": [_vp, _vp, _vp, _pd, _pi64],
    "imsrg_eom_create": [_vp, _i32, _i32, _pvp],
    "imsrg_eom_destroy": [_vp, _vp],
    "imsrg_eom_dim": [_vp, _vp, _pi64, _pi64],
    "imsrg_eom_amplitude_map": [_vp, _vp, _vp, _vp, _vp, _vp],
    "imsrg_eom_matvec": [_vp, _vp, _vp, _vp, _vp],
    "imsrg_eom_matvec_device": [_vp, _vp, _vp, _vp, _vp],
    "imsrg_eom_unwrap": [_vp, _vp, _vp, _vp],
    "imsrg_eom_rewrap": [_vp, _vp, _vp, _vp],
    "imsrg_eom_lanczos": [_vp, _vp, _vp, _i32, _d, _i32, _vp, _vp, _pi32, _pi32],
    "imsrg_commutator_vjp": [_vp, _vp, _vp, _vp, _vp, _vp, _i32],
    "imsrg_white_vjp": [_vp, _vp, _vp, _vp],
    "imsrg_dot_sq_op": [_vp, _vp, _vp, _pd],
    "imsrg_synthetic_hamiltonian": [_vp, _u64, _d, _vp],
    "imsrg_synthetic_bare_hamiltonian": [_vp, _u64, _d, _vp],
    "imsrg_synthetic_me2j_values": [_vp, _u64, _d, _vp, _pi64],
    "imsrg_me2j_to_slab": [_vp, _vp, _i64, _i32, _i32, _vp],
    "imsrg_neq": [_vp, _pi64],
    "imsrg_vectorize_slab": [_vp, _vp, _vp],
    "imsrg_repackage_slab": [_vp, _vp, _i32, _vp],
    "imsrg_write_omega_checkpoint": [_vp, _vp, C.c_char_p],
    "imsrg_read_omega_checkpoint": [_vp, _vp, C.c_char_p],
    "imsrg_calc_hf": [_vp, _vp, _i32, _vp, C.POINTER(HFInfo_t)],
    "imsrg_calc_ho": [_vp, _vp, _vp, C.POINTER(HFInfo_t)],
    "imsrg_sqop_to_hf": [_vp, _vp, _vp],
    "imsrg_transform_2b_to_hf": [_vp, _vp, _vp],
    "imsrg_normal_order": [_vp, _vp],
    "imsrg_launch_count": [_vp, _pi64],
    "imsrg_timer_begin": [_vp],
    "imsrg_timer_end": [_vp, C.POINTER(C.c_float)],
    "imsrg_profile_phases": [_vp, _i32],
    "imsrg_profile_read": [_vp, C.POINTER(C.c_float), _pi32],
    "imsrg_mat_frob_norm_noalloc": [_vp, _vp, _vp, _vp],
    "imsrg_set_wait_limit": [_vp, _i64],
    "imsrg_set_tuning": [_vp, _vp],
    "imsrg_recouple_traffic": [_vp, _pi64, _pi64, _pi64, _pi64],
    "imsrg_test_unarmed_stage": [_vp, _i32],
}
PHASES = ["start", "pandya", "one_body", "c122", "pphh_split", "pphh_gemm", "pphh_small", "pphh_update", "c221",
          "ph_gemm", "recouple", "mirror"]

_lib = None


def load():
    """Load the shared library (raises if it is missing: no CPU fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libimsrg_gb300.so not built ({LIB_PATH}); run eom-imsrg_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = C.c_int32
        f.argtypes = args
    L.imsrg_last_error.restype = C.c_char_p
    L.imsrg_last_error.argtypes = [_vp]
    _lib = L
    return L


def exported_symbols():
    return list(SIGNATURES) + ["imsrg_last_error"]
