"""ctypes binding of ``libfsgpu.so`` (the C ABI of ``include/fsgpu.h``).

The product path is the CUDA library: importing this module loads it and
raises if it is missing or if no CUDA device is usable -- there is no CPU
fallback anywhere in the package.
"""
from __future__ import annotations

import ctypes as C
from functools import lru_cache
from pathlib import Path

from . import build as _build

LIB_PATH = _build.BUILD / "libfsgpu.so"

# enum fs_status
OK = 0
STATUS_NAMES = {0: "ok", 1: "bad handle", 2: "size mismatch", 3: "out of memory",
                4: "CUDA error", 5: "non-finite", 6: "breakdown", 7: "invalid argument",
                8: "no device", 9: "unsupported", 10: "file error"}
ERR_BAD_HANDLE, ERR_SIZE_MISMATCH, ERR_OUT_OF_MEMORY, ERR_CUDA = 1, 2, 3, 4
ERR_NON_FINITE, ERR_BREAKDOWN, ERR_INVALID_ARG, ERR_NO_DEVICE, ERR_UNSUPPORTED = 5, 6, 7, 8, 9
ERR_IO = 10
ERR_CALLBACK = 11

F64, F32 = 0, 1
BC_NONE, BC_DIRICHLET, BC_NEUMANN = 0, 1, 2
CG, BICGSTAB, GMRES, CG_MIXED, BICGSTAB_MIXED, GMRES_MIXED, FCG, CG_PIPELINED = 0, 1, 2, 3, 4, 5, 6, 7
PRECOND_NONE, PRECOND_JACOBI, PRECOND_DIAG, PRECOND_CSR, PRECOND_SOLVER = 0, 1, 2, 3, 4
LEFT, RIGHT = 0, 1
ORTHO_CGS2, ORTHO_MGS, ORTHO_AUTO, ORTHO_DCGS2 = 0, 1, 2, 3
REFINE_RESTART, REFINE_RELIABLE = 0, 1
SPMV_FMA, SPMV_EXACT = 0, 1

# solve_info::stop_reason, flecsolve/solvers/solver_settings.hh:64-72
STOP_REASONS = {0: "converged_atol", 1: "converged_rtol", 2: "converged_user",
                3: "diverged_dtol", 4: "diverged_iters", 5: "diverged_breakdown",
                6: "unknown"}


class SolverSettings(C.Structure):
    _fields_ = [("maxiter", C.c_int), ("rtol", C.c_float), ("atol", C.c_float),
                ("use_zero_guess", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("iters", C.c_int), ("restarts", C.c_int),
                ("res_norm_initial", C.c_float), ("res_norm_final", C.c_float),
                ("sol_norm_initial", C.c_float), ("sol_norm_final", C.c_float),
                ("rhs_norm", C.c_float)]


class KrylovSettings(C.Structure):
    _fields_ = [("base", SolverSettings), ("max_krylov_dim", C.c_int),
                ("pre_side", C.c_int), ("restart", C.c_int), ("ortho", C.c_int),
                ("k_readback", C.c_int), ("refine", C.c_int),
                ("inner_rtol", C.c_double), ("max_outer", C.c_int),
                ("fp64_head", C.c_double)]


class NkaSettings(C.Structure):
    _fields_ = [("base", SolverSettings), ("max_dim", C.c_int), ("angle_tol", C.c_double),
                ("max_fun_evals", C.c_int), ("freeze_pc", C.c_int), ("use_qr", C.c_int),
                ("use_damping", C.c_int), ("adaptive_damping", C.c_int),
                ("damping_factor", C.c_double)]


class FvmMesh(C.Structure):
    _fields_ = [("n", C.c_int64 * 3), ("box", (C.c_double * 2) * 3)]


class FvmOperatorSettings(C.Structure):
    _fields_ = [("mesh", FvmMesh), ("beta", C.c_double), ("alpha", C.c_double),
                ("bc_kind", C.c_int * 6), ("bc_value", C.c_double * 6),
                ("a_value", C.c_double), ("b_value", C.c_double)]


class BdfSettings(C.Structure):
    _fields_ = [("initial_time", C.c_double), ("final_time", C.c_double), ("max_steps", C.c_int),
                ("max_dt", C.c_double), ("min_dt", C.c_double), ("initial_dt", C.c_double),
                ("use_predictor", C.c_int), ("use_initial_predictor", C.c_int),
                ("has_source_term", C.c_int), ("combine_timestep_estimators", C.c_int),
                ("predictor", C.c_int), ("timestep_strategy", C.c_int),
                ("dt_cut_lower_bound", C.c_double), ("dt_growth_upper_bound", C.c_double),
                ("number_of_time_intervals", C.c_int), ("integrator", C.c_int),
                ("starting_integrator", C.c_int), ("calculate_time_trunc_error", C.c_int),
                ("time_trunc_err_norm", C.c_int), ("target_relative_change", C.c_double),
                ("use_pi_controller", C.c_int), ("pi_controller_type", C.c_int),
                ("control_timestep_variation", C.c_int), ("time_error_scaling", C.c_int),
                ("time_rtol", C.c_double), ("time_atol", C.c_double),
                ("num_problem_scales", C.c_int), ("problem_scale", C.c_double)]


class BdfState(C.Structure):
    _fields_ = [("current_time", C.c_double), ("current_dt", C.c_double), ("final_time", C.c_double),
                ("current_step", C.c_int), ("num_step_rejects", C.c_int), ("solver_success", C.c_int),
                ("solver_iters", C.c_int), ("gamma", C.c_double)]


class Precond(C.Structure):
    _fields_ = [("kind", C.c_int), ("diag", C.c_void_p), ("op", C.c_void_p),
                ("solver", C.c_void_p)]


DIAG_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_double)
RESIDUAL_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p)
OP_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p)
RHS_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p)
TIME_SOLVE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.POINTER(C.c_int))

_vp = C.c_void_p
_i64 = C.c_int64
_dp = C.POINTER(C.c_double)


# name -> (argtypes); every function returns int status
_PROTOS = {
    "fs_ctx_create": [C.c_int, C.POINTER(_vp)],
    "fs_ctx_destroy": [_vp],
    "fs_ctx_sync": [_vp],
    "fs_ctx_stream": [_vp, C.POINTER(_vp)],
    "fs_ctx_sm_count": [_vp, C.POINTER(C.c_int)],
    "fs_ctx_launch_count": [_vp, C.POINTER(_i64)],
    "fs_ctx_event_record": [_vp, C.c_int],
    "fs_ctx_event_elapsed": [_vp, C.c_int, C.c_int, C.POINTER(C.c_float)],
    "fs_vec_create": [_vp, _i64, C.c_int, C.POINTER(_vp)],
    "fs_vec_wrap": [_vp, _i64, C.c_int, _vp, C.POINTER(_vp)],
    "fs_vec_destroy": [_vp],
    "fs_vec_size": [_vp, C.POINTER(_i64)],
    "fs_vec_dtype": [_vp, C.POINTER(C.c_int)],
    "fs_vec_device_ptr": [_vp, C.POINTER(_vp)],
    "fs_vec_upload": [_vp, _vp, _i64],
    "fs_vec_download": [_vp, _vp, _i64],
    "fs_vec_copy": [_vp, _vp],
    "fs_vec_zero": [_vp],
    "fs_vec_set_scalar": [_vp, C.c_double],
    "fs_vec_scale": [C.c_double, _vp, _vp],
    "fs_vec_scale_self": [C.c_double, _vp],
    "fs_vec_add": [_vp, _vp, _vp],
    "fs_vec_subtract": [_vp, _vp, _vp],
    "fs_vec_multiply": [_vp, _vp, _vp],
    "fs_vec_divide": [_vp, _vp, _vp],
    "fs_vec_reciprocal": [_vp, _vp],
    "fs_vec_linear_sum": [C.c_double, _vp, C.c_double, _vp, _vp],
    "fs_vec_axpy": [C.c_double, _vp, _vp, _vp],
    "fs_vec_axpby": [C.c_double, C.c_double, _vp, _vp],
    "fs_vec_abs": [_vp, _vp],
    "fs_vec_add_scalar": [_vp, C.c_double, _vp],
    "fs_vec_set_random": [_vp, C.c_uint64],
    "fs_vec_dot": [_vp, _vp, _dp],
    "fs_vec_l1norm": [_vp, _dp],
    "fs_vec_l2norm": [_vp, _dp],
    "fs_vec_inf_norm": [_vp, _dp],
    "fs_vec_min": [_vp, _dp],
    "fs_vec_max": [_vp, _dp],
    "fs_csr_create": [_vp, _i64, _i64, _i64, _vp, _vp, C.c_int, _vp, C.POINTER(_vp)],
    "fs_csr_destroy": [_vp],
    "fs_csr_shape": [_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64)],
    "fs_csr_update_values": [_vp, _vp],
    "fs_csr_update_values_device": [_vp, _vp],
    "fs_csr_values_device_ptr": [_vp, C.POINTER(_vp)],
    "fs_csr_index_coding": [_vp, C.c_int, C.POINTER(C.c_int)],
    "fs_csr_row_blocks": [_vp, C.POINTER(_i64)],
    "fs_csr_grid_dims": [_vp, C.POINTER(_i64)],
    "fs_csr_tune": [_vp, C.c_int, C.POINTER(C.c_int)],
    "fs_csr_set_lanes": [_vp, C.c_int, C.c_int],
    "fs_parcsr_create": [_vp, _i64, _i64, _i64, _vp, _vp, _vp, C.POINTER(_vp)],
    "fs_parcsr_destroy": [_vp],
    "fs_parcsr_shape": [_vp] + [C.POINTER(_i64)] * 5,
    "fs_parcsr_ghosts": [_vp, _vp, C.POINTER(_i64)],
    "fs_parcsr_color_spmv": [_vp, _vp, _vp],
    "fs_csr_spmv": [_vp, _vp, _vp, C.c_int],
    "fs_csr_residual": [_vp, _vp, _vp, _vp],
    "fs_csr_spmv_transpose": [_vp, _vp, _vp],
    "fs_csr_diag_inv": [_vp, _vp],
    "fs_parcsr_spmv": [_vp, C.c_int, _vp, _vp],
    "fs_nka_settings_default": [C.POINTER(NkaSettings)],
    "fs_nka_create": [_vp, C.POINTER(NkaSettings), _vp, RESIDUAL_FN, _vp, _vp, C.POINTER(_vp)],
    "fs_nka_set_diagnostic": [_vp, DIAG_FN, _vp],
    "fs_nka_apply": [_vp, _vp, _vp, C.POINTER(SolveInfo)],
    "fs_nka_reset": [_vp],
    "fs_nka_destroy": [_vp],
    "fs_fvm_geometry": [C.POINTER(FvmMesh), _dp, _dp, _dp],
    "fs_fvm_boundary": [_vp, C.POINTER(FvmMesh), C.c_int, C.c_int, C.c_double, _vp],
    "fs_fvm_coef_constant": [_vp, C.POINTER(FvmMesh), C.c_double, _vp, _vp, _vp],
    "fs_fvm_coef_average": [_vp, C.POINTER(FvmMesh), _vp, _vp, _vp, _vp],
    "fs_fvm_diffusion": [_vp, C.POINTER(FvmMesh), C.c_double, C.c_double, _vp, _vp, _vp, _vp, _vp,
                         _vp],
    "fs_fvm_pack": [_vp, C.POINTER(FvmMesh), _vp, _vp],
    "fs_fvm_unpack": [_vp, C.POINTER(FvmMesh), _vp, _vp],
    "fs_fvm_operator_create": [_vp, C.POINTER(FvmOperatorSettings), _vp, _vp, _vp, _vp,
                               C.POINTER(_vp)],
    "fs_fvm_operator_info": [_vp, C.POINTER(C.c_int), C.POINTER(_i64)],
    "fs_bdf_settings_default": [C.POINTER(BdfSettings)],
    "fs_bdf_create": [_vp, C.POINTER(BdfSettings), _i64, RHS_FN, _vp, TIME_SOLVE_FN, _vp, C.POINTER(_vp)],
    "fs_bdf_create_linear": [_vp, C.POINTER(BdfSettings), _vp, C.c_int, C.POINTER(KrylovSettings),
                             C.POINTER(Precond), C.POINTER(_vp)],
    "fs_bdf_advance": [_vp, C.c_double, C.c_int, _vp, _vp],
    "fs_bdf_check_solution": [_vp, C.POINTER(C.c_int)],
    "fs_bdf_update": [_vp],
    "fs_bdf_get_next_dt": [_vp, C.c_int, C.POINTER(C.c_double)],
    "fs_bdf_state_get": [_vp, C.POINTER(BdfState)],
    "fs_bdf_destroy": [_vp],
    "fs_mm_read": [C.c_char_p, C.POINTER(_vp)],
    "fs_mm_shape": [_vp, C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64), C.POINTER(C.c_int)],
    "fs_mm_rows": [_vp, _i64, _i64, _vp, _vp, _vp, C.POINTER(_i64)],
    "fs_mm_destroy": [_vp],
    "fs_krylov_settings_default": [C.POINTER(KrylovSettings)],
    "fs_krylov_create": [_vp, C.c_int, C.POINTER(KrylovSettings), _vp,
                         C.POINTER(Precond), C.POINTER(_vp)],
    "fs_krylov_destroy": [_vp],
    "fs_krylov_set_diagnostic": [_vp, DIAG_FN, _vp],
    "fs_shell_create": [_vp, C.c_int64, C.c_int64, OP_FN, _vp, C.POINTER(_vp)],
    "fs_krylov_settings_get": [_vp, C.POINTER(KrylovSettings)],
    "fs_krylov_settings_set": [_vp, C.POINTER(KrylovSettings)],
    "fs_krylov_apply": [_vp, _vp, _vp, C.POINTER(SolveInfo)],
    "fs_krylov_history": [_vp, _dp, C.POINTER(_i64)],
    "fs_krylov_mixed_stats": [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "fs_batch_cg_solve": [_vp, C.POINTER(KrylovSettings), _vp, C.c_int, C.POINTER(_i64), _vp, _vp,
                          C.c_int, C.c_int, C.POINTER(SolveInfo)],
    "fs_batch_tuning": [_vp, _vp, C.c_int, C.POINTER(_i64), C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "fs_batch_schedule": [_vp, _vp, C.c_int, C.POINTER(_i64), C.POINTER(C.c_int), C.POINTER(C.c_int),
                          C.POINTER(C.c_int)],
    "fs_batch_format": [_vp, _vp, C.c_int, C.POINTER(_i64), C.POINTER(C.c_int)],
    "fs_batch_cg_solve_split": [_vp, C.POINTER(KrylovSettings), _vp, C.c_int, C.POINTER(_i64), _vp,
                                _vp, C.c_int, C.c_int, C.c_int, C.POINTER(SolveInfo)],
    "fs_krylov_apply_transpose": [_vp, _vp, _vp, C.POINTER(SolveInfo)],
    "fs_csr_transpose": [_vp, C.POINTER(_vp)],
    "fs_csr_value_grad": [_vp, _vp, _vp, _vp],
    "fs_fv_assemble": [_vp, C.c_int, _i64, _vp, C.c_double, C.c_double],
    "fs_fv_face_grad": [_vp, C.c_int, _i64, _vp, _vp, C.c_double, C.c_int, _vp],
    "fs_block_cg_solve": [_vp, C.POINTER(KrylovSettings), _vp, C.POINTER(Precond), C.c_int, _vp, _vp,
                          C.POINTER(SolveInfo)],
    "fs_block_cg_solve_mixed": [_vp, C.POINTER(KrylovSettings), _vp, C.POINTER(Precond), C.c_int,
                                _vp, _vp, C.POINTER(SolveInfo)],
}

# entry points that exist in the header but are optional for older builds
OPTIONAL = set()


def header_symbols() -> list[str]:
    """Every FS_API function declared in include/*.h."""
    import re
    names = []
    inc = _build.INCLUDE
    for h in sorted(inc.glob("*.h")):
        txt = h.read_text()
        names += re.findall(r"FS_API\s+[^;{]*?\b(fs_\w+)\s*\(", txt)
    return names


@lru_cache(maxsize=1)
def lib(build_if_missing: bool = True) -> C.CDLL:
    if not LIB_PATH.exists():
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build()")
        _build.build_gpu()
    L = C.CDLL(str(LIB_PATH))
    for name, args in _PROTOS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.fs_last_error.argtypes = [_vp]
    L.fs_last_error.restype = C.c_char_p
    L.fs_status_string.argtypes = [C.c_int]
    L.fs_status_string.restype = C.c_char_p
    return L


class FsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def check(status: int, ctx=None, what: str = ""):
    if status != OK:
        msg = ""
        if ctx is not None:
            raw = lib().fs_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise FsError(status, f"{what} {msg}".strip())
