"""ctypes binding of the C ABI in include/ntgb300.h (no torch types cross it)."""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "lib", "libntgb300.so")

NTG_OK, NTG_ERR_INVALID, NTG_ERR_CUDA, NTG_ERR_ALLOC, NTG_ERR_UNSUPPORTED = 0, 1, 2, 3, 4
NTG_MAXITER, NTG_BREAKDOWN, NTG_NONFINITE, NTG_GUESS_REJECTED = 10, 11, 12, 13
GS_OP_ADD, GS_OP_MUL, GS_OP_MIN, GS_OP_MAX = 1, 2, 3, 4
KSP_CG, KSP_FCG_MIXED, KSP_CG_MIXED, KSP_GMRES, KSP_GMRES_MIXED = 0, 1, 2, 3, 4

_vp = C.c_void_p
_i = C.c_int
_i64 = C.c_int64
_d = C.c_double
_pi64 = C.POINTER(C.c_int64)
_pi = C.POINTER(C.c_int)
_pd = C.POINTER(C.c_double)


class ntg_monitor(C.Structure):
    _fields_ = [("iter", C.c_int), ("inner_iter", C.c_int), ("res_start", C.c_double),
                ("res_final", C.c_double), ("rhs_norm", C.c_double), ("status", C.c_int),
                ("fp64_ax", C.c_int), ("guess_rejected", C.c_int)]


class NtgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"ntgb300 status {status}: {msg}")
        self.status = status


# name -> (restype, argtypes); every symbol include/ntgb300.h declares
SIGNATURES = {
    "ntg_version": (C.c_char_p, []),
    "ntg_last_error": (C.c_char_p, []),
    "ntg_supported_lx": (_i, [_pi, _i]),
    "ntg_launch_count": (C.c_ulonglong, []),
    "ntg_timer_enable": (_i, [_i]),
    "ntg_timer_read": (_i, [_i, _pd, C.POINTER(C.c_longlong)]),
    "ntg_timer_reset": (_i, []),
    "ntg_plan_create": (_i, [C.POINTER(_vp), _i64, _i, _vp, _vp, _vp, _vp]),
    "ntg_plan_destroy": (_i, [_vp]),
    "ntg_plan_set_stream": (_i, [_vp, _vp]),
    "ntg_plan_info": (_i, [_vp, _pi64, _pi, _pi64, _pi64, _pi64]),
    "ntg_coef_get": (_i, [_vp] + [_vp] * 8),
    "ntg_coef_set": (_i, [_vp, _vp, _d, _vp, _d, _i]),
    "ntg_plan_set_mask": (_i, [_vp, _vp, _i64, _i]),
    "ntg_gs_export": (_i, [_vp, _vp, _vp]),
    "ntg_plan_set_ax_path": (_i, [_vp, _i]),
    "ntg_plan_set_gs_path": (_i, [_vp, _i]),
    "ntg_plan_check_error": (_i, [_vp, _pi]),
    "ntg_mesh_box": (_i, [_i, _i, _i, _i, _pd, _pd, _d, C.c_uint64, _vp, _vp, _vp, _vp, _vp]),
    "ntg_mask_face_xmax": (_i, [_i, _i, _i, _i, _vp, _pi64, _vp]),
    "ntg_field_uniform": (_i, [_vp, _i64, C.c_uint64, C.c_uint64, _d, _d, _vp, _vp]),
    "ntg_field_fourier": (_i, [_vp, _vp, _vp, _i64, _pd, _pd, _i, _i, C.c_uint64, _vp, _vp]),
    "ntg_field_blobs": (_i, [_vp, _vp, _vp, _i64, _pd, _pd, C.c_uint64, _i, _d, _vp, _vp]),
    "ntg_field_modes": (_i, [_vp, _vp, _vp, _i64, _pd, _pd, _i, _pi, _pd, _pd, _vp, _vp]),
    "ntg_ksp_set_fused_update": (_i, [_vp, _i]),
    "ntg_ksp_set_guess_guard": (_i, [_vp, _i]),
    "ntg_ksp_set_tol": (_i, [_vp, _d, _d]),
    "ntg_ksp_set_schwarz": (_i, [_vp, _vp]),
    "ntg_schwarz_create": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, C.POINTER(_vp)]),
    "ntg_schwarz_create_general": (_i, [_vp, _vp, _vp, _vp, C.POINTER(_vp)]),
    "ntg_schwarz_ghost_table": (_i, [C.c_int64, _i, _vp, _vp]),
    "ntg_nmsh_info": (_i, [C.c_char_p, _vp, _vp, _vp, _vp]),
    "ntg_nmsh_read": (_i, [C.c_char_p, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ntg_nmsh_write": (_i, [C.c_char_p, C.c_int32, C.c_int32, _vp, _vp, _vp, C.c_int32, _vp, C.c_int32, _vp, _vp, _vp]),
    "ntg_nodes_from_vertices": (_i, [C.c_int64, _i, _vp, _vp, _vp, _vp, _vp]),
    "ntg_schwarz_update": (_i, [_vp]),
    "ntg_schwarz_set_coarse": (_i, [_vp, _i]),
    "ntg_schwarz_set_mass_term": (_i, [_vp, _i]),
    "ntg_schwarz_set_fdm_path": (_i, [_vp, _i]),
    "ntg_schwarz_destroy": (_i, [_vp]),
    "ntg_schwarz_apply": (_i, [_vp, _vp, _vp]),
    "ntg_rhs_assemble": (_i, [_vp, _vp, _vp]),
    "ntg_ax_helm": (_i, [_vp, _vp, _vp]),
    "ntg_ax_helm_f32": (_i, [_vp, _vp, _vp]),
    "ntg_gs_op": (_i, [_vp, _vp, _i]),
    "ntg_gs_op_f32": (_i, [_vp, _vp, _i]),
    "ntg_bc_apply_scalar": (_i, [_vp, _vp]),
    "ntg_bc_apply_scalar_f32": (_i, [_vp, _vp]),
    "ntg_pc_jacobi_update": (_i, [_vp]),
    "ntg_pc_jacobi_solve": (_i, [_vp, _vp, _vp]),
    "ntg_pc_jacobi_get": (_i, [_vp, _vp]),
    "ntg_ksp_create": (_i, [_vp, _i, _i, _d, _d, C.POINTER(_vp)]),
    "ntg_ksp_destroy": (_i, [_vp]),
    "ntg_ksp_set_inner": (_i, [_vp, _d, _i]),
    "ntg_ksp_set_check_every": (_i, [_vp, _i]),
    "ntg_ksp_set_restart": (_i, [_vp, _i]),
    "ntg_ksp_solve": (_i, [_vp, _vp, _vp, C.POINTER(ntg_monitor)]),
    "ntg_ksp_solve_coupled": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(ntg_monitor)]),
    "ntg_proj_create": (_i, [_vp, _i, C.POINTER(_vp)]),
    "ntg_proj_destroy": (_i, [_vp]),
    "ntg_proj_pre_solving": (_i, [_vp, _vp]),
    "ntg_proj_post_solving": (_i, [_vp, _vp]),
    "ntg_proj_pre_solving_with": (_i, [_vp, _vp, _vp, _pi]),
    "ntg_proj_size": (_i, [_vp]),
    "ntg_proj_post_solving_full": (_i, [_vp, _vp]),
    "ntg_proj_state": (_i, [_vp, _pi, _vp, _vp, _i]),
    "ntg_profiler_start_region": (_i, [C.c_char_p, _i]),
    "ntg_profiler_end_region": (_i, []),
    "ntg_glsc3": (_i, [_vp, _vp, _vp, _vp, _i64, _pd]),
    "ntg_guess_create": (_i, [_vp, _i, _i, C.c_uint64, C.POINTER(_vp)]),
    "ntg_guess_destroy": (_i, [_vp]),
    "ntg_guess_set_lr": (_i, [_vp, _d]),
    "ntg_guess_predict": (_i, [_vp, _vp, _vp, _pi]),
    "ntg_guess_observe": (_i, [_vp, _vp, _vp, _i, _pd]),
    "ntg_guess_reset_history": (_i, [_vp]),
    "ntg_guess_state_len": (_i64, [_vp]),
    "ntg_guess_state": (_i, [_vp, _vp, C.POINTER(C.c_longlong), _pd, _i]),
    "ntg_guess_set_loss": (_i, [_vp, _i]),
    "ntg_guess_num_params": (_i64, [_vp]),
    "ntg_guess_params": (_i, [_vp, _vp, _i]),
    "ntg_guess_forward_raw": (_i, [_vp, _vp, _i64, _vp]),
    "ntg_guess_grad_raw": (_i, [_vp, _vp, _vp, _i64, _vp, _pd]),
    "ntg_guess_train_raw": (_i, [_vp, _vp, _vp, _i64, _pd]),
    "ntg_gemm_bf16": (_i, [_vp, _i64, _vp, _i64, _vp, _i64, _i64, _i64, _i64, _vp, _vp]),
    "ntg_ramp_forward": (_i, [_vp, _vp, _i64, _d, _d, _d, _i, _vp]),
    "ntg_ramp_backward": (_i, [_vp, _vp, _vp, _i64, _d, _d, _d, _i, _vp]),
    "ntg_brinkman_compute": (_i, [_vp] * 7 + [_i64, _vp, _i64, _i, _vp]),
    "ntg_permeability": (_i, [_vp, _vp, _i64, _d, _d, _d, _vp]),
    "ntg_sens_min_dissipation": (_i, [_vp] * 7 + [_i64, _i, _d, _vp]),
    "ntg_filter_apply": (_i, [_vp, _vp, _vp, _vp, _d, C.POINTER(ntg_monitor)]),
    "ntg_metrics_set": (_i, [_vp, _vp, _vp, _vp]),
    "ntg_dudxyz": (_i, [_vp, _vp, _vp, _i]),
    "ntg_opgrad": (_i, [_vp] * 5),
    "ntg_cdtp": (_i, [_vp, _vp, _vp, _i]),
    "ntg_conv1": (_i, [_vp] * 6),
    "ntg_curl": (_i, [_vp] * 7),
    "ntg_adjoint_advection_no_dealias": (_i, [_vp] * 10),
    "ntg_linear_advection_no_dealias": (_i, [_vp] * 10),
    "ntg_adjoint_min_dissipation": (_i, [_vp] * 7 + [_d, _vp, _i64, _i]),
    "ntg_pnpn_prs_res": (_i, [_vp] * 13 + [_d, _vp, _d, _d, _d, _vp, _vp, _i64, _vp, _vp, _i64, _i]),
    "ntg_pnpn_vel_res": (_i, [_vp] * 12 + [_d, _vp, _d, _d, _d]),
    "ntg_mma_create": (_i, [_vp, _i64, _i, _vp, _d, _pd, _pd, _pd, _vp, _vp, _i, _d, _d, _d, _d, _vp]),
    "ntg_mma_destroy": (_i, [_vp]),
    "ntg_mma_update": (_i, [_vp, _i, _vp, _vp, _pd, _vp]),
    "ntg_mma_kkt": (_i, [_vp, _vp, _vp, _pd, _vp, _pd, _pd]),
    "ntg_mma_info": (_i, [_vp, C.POINTER(C.c_longlong), _pd, _pd]),
    "ntg_fld_write": (_i, [C.c_char_p, _i, _i64, _vp, _d, _i, _i, _i] + [_vp] * 9 + [_i]),
    "ntg_fld_write_index": (_i, [C.c_char_p, C.c_char_p, _i, _i]),
    "ntg_fld_info": (_i, [C.c_char_p, _vp, _vp, _vp, _vp, _vp, C.c_char_p, _i]),
    "ntg_fld_read": (_i, [C.c_char_p, _i, _vp] + [_vp] * 8 + [_vp, _i]),
    "ntg_dealias_create": (_i, [_vp, _vp, _i]),
    "ntg_dealias_destroy": (_i, [_vp]),
    "ntg_dealias_info": (_i, [_vp, _vp, _vp]),
    "ntg_dealias_map": (_i, [_vp, _vp, _vp, _i]),
    "ntg_adjoint_advection_dealias": (_i, [_vp] * 10),
    "ntg_linear_advection_dealias": (_i, [_vp] * 10),
    "cuda_cadd_mask": (None, [_vp, _pd, _pi, _vp, _pi]),
    "cuda_invcol1_mask": (None, [_vp, _pi, _vp, _pi]),
    "cuda_col2_mask": (None, [_vp, _vp, _pi, _vp, _pi]),
    "cuda_col3_mask": (None, [_vp, _vp, _vp, _pi, _vp, _pi]),
    "cuda_sub3_mask": (None, [_vp, _vp, _vp, _pi, _vp, _pi]),
    "cuda_cmult_mask": (None, [_vp, _pd, _pi, _vp, _pi]),
    "cuda_glsc2_mask": (_d, [_vp, _vp, _pi, _vp, _pi]),
    "ntg_set_glb_queue": (None, [_vp]),
    "ntg_glsc2_mask_noalloc": (_i, [_vp, _vp, _vp, _i, _vp, _vp]),
}

_lib = None


def library_path() -> str:
    return _LIB


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            raise NtgError(-1, f"CUDA library missing: {_LIB} (run build() first); there is no CPU fallback")
        L = C.CDLL(_LIB)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> int:
    """Raise NtgError for hard errors; solver statuses (>= 10) are returned."""
    if status != NTG_OK and status < 10:
        raise NtgError(status, lib().ntg_last_error().decode())
    return status


def check_last(name: str) -> None:
    """For the void cuda_* kernels: raise if they recorded an error."""
    msg = lib().ntg_last_error().decode()
    if msg:
        raise NtgError(NTG_ERR_CUDA, f"{name}: {msg}")
