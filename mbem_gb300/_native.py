"""ctypes binding of the C ABI in ``include/mbem_gb300.h``.

The library is the product path: there is no CPU fallback. If
``_lib/libmbem_gb300.so`` is missing, importing a GPU entry point raises
with the instruction to build it (``python -m mbem_gb300.build`` or
``__graft_entry__.build()``).
"""

from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, Structure, c_char_p, c_double, c_int, c_int64, c_size_t, c_void_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmbem_gb300.so")

# status codes (mbem_status)
OK = 0
ERR_ARG = 1
ERR_UNSUPPORTED = 2
ERR_CUDA = 3
ERR_WAIT = 4
ERR_SIZE = 5
ERR_NUMERIC = 6

STRESS_DD, STRESS_KELVIN, STRESS_EIGEN, STRESS_ELASTIC = 0, 1, 2, 3


class MbemError(RuntimeError):
    """A non-zero mbem_status from the CUDA library."""

    def __init__(self, code: int, what: str, message: str):
        super().__init__(f"{what}: status {code}: {message}")
        self.code = code


class FgmresParams(Structure):
    _fields_ = [("restart", c_int), ("maxiter", c_int), ("rtol", c_double),
                ("stagnation_window", c_int), ("stagnation_factor", c_double),
                ("n_u_ranges", c_int), ("u_ranges", POINTER(c_int64)),
                ("precond", c_int), ("precond_state", c_void_p), ("time_matvec", c_int),
                ("x_is_zero", c_int)]


class FgmresReport(Structure):
    _fields_ = [("converged", c_int), ("iterations", c_int), ("restarts", c_int),
                ("stagnated", c_int), ("true_relres", c_double), ("arnoldi_relres", c_double),
                ("history", POINTER(c_double)), ("matvecs", c_int), ("matvec_ms", c_double)]


class NearBlocks(Structure):
    _fields_ = [("row0", c_int64), ("col0", c_int64), ("n_field", c_int64), ("rowptr", c_void_p),
                ("cols", c_void_p), ("vals", c_void_p)]


class MixedOperator(Structure):
    _fields_ = [("n_rows", c_int64), ("n_cols", c_int64), ("A32", c_void_p), ("ld32", c_int64),
                ("n_near", c_int), ("near", POINTER(NearBlocks))]


class BlockJacobi(Structure):
    _fields_ = [("n", c_int64), ("n_chunks", c_int64), ("m_max", c_int), ("chunk_ptr", c_void_p),
                ("dofs", c_void_p), ("local", c_void_p), ("chunk_of", c_void_p), ("inv", c_void_p)]


BJ_MAX_DOF = 225


class NnPrecond(Structure):
    _fields_ = [("n", c_int64), ("n_coarse", c_int64), ("bj", POINTER(BlockJacobi)), ("basis", c_void_p),
                ("APhi", c_void_p), ("Ac_inv", c_void_p), ("work", c_void_p), ("APhi32", c_void_p),
                ("Ac_inv32", c_void_p), ("ld32", c_int64)]


class InnerBf16(Structure):
    _fields_ = [("n", c_int64), ("A16", c_void_p), ("ld16", c_int64), ("n_near", c_int),
                ("near", POINTER(NearBlocks)), ("iterations", c_int), ("rtol", c_double), ("n_u_ranges", c_int),
                ("u_ranges", c_void_p), ("work", c_void_p), ("work_bytes", c_size_t), ("precond", c_int),
                ("precond_state", c_void_p)]


INNER_MAX_ITERS = 64


class MmMesh(Structure):
    _fields_ = [("A32", c_void_p), ("ld32", c_int64), ("n", c_int64), ("offset", c_int64), ("rowptr", c_void_p),
                ("cols", c_void_p), ("vals", c_void_p), ("u_off", c_int64), ("u_len", c_int64), ("A16", c_void_p),
                ("ld16", c_int64)]


class MmReport(Structure):
    _fields_ = [("iterations", POINTER(c_int)), ("relres", POINTER(c_double)), ("converged", POINTER(c_int)),
                ("cycles", c_int)]


class PairGeometry(Structure):
    _fields_ = [("kernel", c_int), ("x_field", c_void_p), ("n_field", c_int64), ("tri_verts", c_void_p),
                ("normals", c_void_p), ("eps", c_void_p), ("n_src", c_int64), ("coeffs", c_double * 6),
                ("near_factor", c_double), ("prep", c_void_p)]


class AcaBatch(Structure):
    _fields_ = [("n_blocks", c_int64), ("r0", c_void_p), ("nr", c_void_p), ("c0", c_void_p), ("nc", c_void_p),
                ("max_pivots", c_void_p), ("u_off", c_void_p), ("v_off", c_void_p), ("U", c_void_p),
                ("V", c_void_p), ("rank", c_void_p), ("status", c_void_p), ("err", c_void_p), ("tol", c_double),
                ("seed", ctypes.c_uint64), ("first_index", c_int64), ("max_nr", c_int), ("max_nc", c_int),
                ("max_pivots_all", c_int)]


class AcaRecompression(Structure):
    _fields_ = [("n_blocks", c_int64), ("r0", c_void_p), ("nr", c_void_p), ("c0", c_void_p), ("nc", c_void_p),
                ("rank", c_void_p), ("u_off", c_void_p), ("v_off", c_void_p), ("U", c_void_p), ("V", c_void_p),
                ("ur_off", c_void_p), ("vr_off", c_void_p), ("Ur", c_void_p), ("Vr", c_void_p),
                ("rank_out", c_void_p), ("err_out", c_void_p), ("index", c_void_p), ("tol", c_double),
                ("seed", ctypes.c_uint64), ("max_rank", c_int)]


RC_KMAX = 64


class CompressedView(Structure):
    _fields_ = [("n_field", c_int64), ("n_src", c_int64), ("field_order", c_void_p), ("src_order", c_void_p),
                ("n_lr", c_int64), ("lr_r0", c_void_p), ("lr_nr", c_void_p), ("lr_c0", c_void_p),
                ("lr_nc", c_void_p), ("lr_rank", c_void_p), ("lr_u", c_void_p), ("lr_v", c_void_p),
                ("lr_w", c_void_p), ("U", c_void_p), ("V", c_void_p), ("n_w", c_int64), ("n_dense", c_int64),
                ("d_r0", c_void_p), ("d_nr", c_void_p), ("d_c0", c_void_p), ("d_nc", c_void_p),
                ("d_off", c_void_p), ("D", c_void_p), ("n_strips", c_int64), ("strip_r0", c_void_p),
                ("strip_nr", c_void_p), ("strip_ptr", c_void_p), ("strip_items", c_void_p), ("max_strip", c_int),
                ("max_lr_nc", c_int), ("unit_ptr", c_void_p), ("unit_item", c_void_p), ("unit_k0", c_void_p),
                ("n_proj", c_int64), ("proj_block", c_void_p), ("proj_k0", c_void_p)]


COMPRESSED_UNIT = 32


ACA_LOWRANK, ACA_CAPPED, ACA_FAILED, ACA_RETRIED = 0, 1, 2, 4

MM_SEGMENT = 512
MM_MAX_RESTART = 64

TUNE_MIXED_MATVEC, TUNE_BF16_MATVEC, TUNE_MM_MATVEC, TUNE_GEMM_SPLIT = 0, 1, 2, 3

NN_FEAT, NN_HIDDEN = 16, 32
NN_PARAMS = NN_HIDDEN * NN_FEAT + NN_HIDDEN + NN_HIDDEN * NN_HIDDEN + NN_HIDDEN + 9 * NN_HIDDEN + 9

_P = c_void_p
_I = c_int64
_D = c_double

# name -> (restype, argtypes)
_SIGNATURES = {
    "mbem_version": (c_int, []),
    "mbem_last_error": (ctypes.c_char_p, []),
    "mbem_launch_count": (ctypes.c_ulonglong, []),
    "mbem_fp32_fma_probe": (c_int, [_P, _I, c_int, c_int, c_int, _P]),
    "mbem_fp64_fma_probe": (c_int, [_P, _I, c_int, c_int, _P]),
    "mbem_t_matrix_direct": (c_int, [_P, _I, _P, _P, _P, _I, _P, c_int, _D, c_int, _P, _I, _P]),
    "mbem_u_matrix_direct": (c_int, [_P, _I, _P, _P, _I, _P, c_int, _D, c_int, _P, _I, _P]),
    "mbem_t_basis_matrices": (c_int, [_P, _I, _P, _P, _P, _I, c_int, _P, _P]),
    "mbem_u_basis_matrices": (c_int, [_P, _I, _P, _P, _I, c_int, _P, _P]),
    "mbem_t_disp_contract": (c_int, [_P, _I, _P, _P, _P, _I, _P, _P, c_int, _D, c_int, _P, _P]),
    "mbem_u_disp_contract": (c_int, [_P, _I, _P, _P, _I, _P, _P, c_int, _D, c_int, _P, _P]),
    "mbem_stress_contract": (c_int, [c_int, _P, _I, _P, _P, _P, _I, _P, _D, _D, c_int, _D, c_int,
                                     _P, _P]),
    "mbem_traction_matrix": (c_int, [_P, _P, _I, _P, _P, _P, _I, _P, _I, _D, _D, c_int, c_int, _D,
                                     _P, _I, _P]),
    "mbem_block_rowsum3": (c_int, [_P, _I, _I, _I, _D, c_int, _P, _P]),
    "mbem_add_block_diagonal": (c_int, [_P, _I, _P, _I, c_int, _P, _P]),
    "mbem_rotate_row_triples": (c_int, [_P, _I, _I, _P, _I, _P, _P]),
    "mbem_dgemv": (c_int, [_P, _I, _I, _I, _P, _D, _D, _P, _P]),
    "mbem_dgemm_multi": (c_int, [_P, _I, _I, _I, _P, _I, _P, _P]),
    "mbem_project_translation": (c_int, [_P, _P, _I, _P, c_int, _P, _P]),
    "mbem_gemm_bf16": (c_int, [_P, _I, _P, _I, _I, _I, c_int, _P, _I, _P]),
    "mbem_gemm_bf16_check": (c_int, [_P]),
    "mbem_gemm_bf16_t": (c_int, [_P, _I, _P, _I, _I, _I, c_int, _P, _I, _P]),
    "mbem_gemm_bf16_workspace_size": (c_size_t, [_I, c_int]),
    "mbem_gemm_bf16_t_split": (c_int, [_P, _I, _P, _I, _I, _I, c_int, _P, _I, _P, c_size_t, _P]),
    "mbem_to_bf16": (c_int, [_P, c_int, _I, _I, _I, _P, _I, _P]),
    "mbem_mixed_to_bf16": (c_int, [POINTER(MixedOperator), _P, _I, _P]),
    "mbem_to_bf16x2": (c_int, [_P, c_int, _I, _I, _I, _P, _P, _I, _P]),
    "mbem_mixed_to_bf16x2": (c_int, [POINTER(MixedOperator), _P, _P, _I, _P]),
    "mbem_batch_dots": (c_int, [_P, c_int, _P, _I, _I, _P, _P]),
    "mbem_batch_axpy": (c_int, [_P, _P, c_int, _P, _D, _I, _I, _P]),
    "mbem_batch_normalize": (c_int, [_P, c_int, _I, _I, _P, _P, _P, _P]),
    "mbem_batch_update": (c_int, [_P, _P, c_int, _P, _I, _I, _P]),
    "mbem_batch_project": (c_int, [_P, c_int, _I, _I, _P, c_int, _P]),
    "mbem_batch_residual_workspace_size": (c_size_t, [_I, _I]),
    "mbem_batch_residual_mixed": (c_int, [POINTER(MixedOperator), _P, _P, _I, _P, _P, c_size_t, _P]),
    "mbem_readout_record_bytes": (c_size_t, [_I]),
    "mbem_t_disp_readout": (c_int, [_P, _I, _P, _P, _P, _I, _P, _P, _D, _D, c_int, _P, _P]),
    "mbem_geom_record_bytes": (c_size_t, [_I]),
    "mbem_geom_prepare": (c_int, [_P, _I, _P, _P]),
    "mbem_solid_angle_sum": (c_int, [_P, _P, _I, _P, _I, _D, c_int, _P, _P]),
    "mbem_mesh_distance": (c_int, [_P, _P, _I, _P, _I, _D, _P, _P, _P]),
    "mbem_readout_prepare": (c_int, [_P, _I, _P, _P, _P, _I, _P, c_int, _D, _P, _P, _P, POINTER(c_int64), _P]),
    "mbem_readout_evaluate": (c_int, [_P, _I, _P, _P, _P, _I, _P, _D, _D, c_int, _P, _P, _I, _P, _P, _P, _D, c_int,
                                      _P, _P]),
    "mbem_readout_evaluate_parts": (c_int, [_P, _I, _P, _P, _P, _I, _P, _D, _D, c_int, _P, _P, _I, _P, _P, _P, _P,
                                            _D, c_int, _P, _P, _P]),
    "mbem_bj_inverse_bytes": (c_size_t, [_I, c_int]),
    "mbem_bj_build_dense": (c_int, [_P, _I, POINTER(BlockJacobi), _P]),
    "mbem_bj_build_mixed": (c_int, [POINTER(MixedOperator), POINTER(BlockJacobi), _P]),
    "mbem_bj_apply": (c_int, [POINTER(BlockJacobi), _P, _P, _P]),
    "mbem_nn_forward": (c_int, [_P, _I, _P, _P, _P, _P]),
    "mbem_nn_coarse_loss_grad": (c_int, [POINTER(BlockJacobi), _P, _P, _P, _I, _P, _P, _P, _P]),
    "mbem_nn_backward_workspace_size": (c_size_t, [_I]),
    "mbem_nn_backward": (c_int, [_P, _I, _P, _P, _P, _P, _P, c_size_t, _P]),
    "mbem_nn_adam": (c_int, [_P, _P, _P, _P, _I, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                             ctypes.c_float, c_int, _P]),
    "mbem_nn_basis": (c_int, [POINTER(BlockJacobi), _P, _P, c_int, _P, _P, _P]),
    "mbem_nn_setup_workspace_size": (c_size_t, [_I]),
    "mbem_nn_coarse_operator_dense": (c_int, [_P, _I, POINTER(NnPrecond), _P, c_int, _P]),
    "mbem_dense_inverse_workspace_size": (c_size_t, [_I]),
    "mbem_dense_inverse": (c_int, [_P, _I, _P, c_size_t, _P]),
    "mbem_nn_setup_dense": (c_int, [_P, _I, POINTER(NnPrecond), _P, c_int, _P, c_size_t, _P]),
    "mbem_nn_apply_workspace_size": (c_size_t, [_I, _I]),
    "mbem_nn_apply": (c_int, [POINTER(NnPrecond), _P, _P, _P]),
    "mbem_fgmres_workspace_size": (c_size_t, [_I, c_int]),
    "mbem_fgmres_dense": (c_int, [_P, _I, _I, _P, _P, POINTER(FgmresParams), _P, c_size_t,
                                  POINTER(FgmresReport), _P]),
    "mbem_fgmres_mixed": (c_int, [POINTER(MixedOperator), _P, _P, POINTER(FgmresParams), _P, c_size_t,
                                  POINTER(FgmresReport), _P]),
    "mbem_far_matrix": (c_int, [c_int, _P, _I, _P, _P, _P, _I, _P, _D, _D, _P, _I, _P, _P]),
    "mbem_far_matrix_bf16": (c_int, [c_int, _P, _I, _P, _P, _P, _I, _P, _D, _D, _P, _I, _P, _I, _P, _P]),
    "mbem_far_matrix_nodal": (c_int, [c_int, c_int, _P, _I, _P, _P, _P, _I, _P, _D, _D, _P, _I, _P, _I, _P, _P]),
    "mbem_near_eval_nodal": (c_int, [c_int, c_int, _P, _I, _P, _P, _P, _P, _P, _I, _P, _D, _P, _P]),
    "mbem_near_add_diagonal_nodal": (c_int, [_P, _P, _P, _I, _P, c_int, _P, _P, _P]),
    "mbem_near_mask_count": (c_int, [_P, _I, _I, _P, _P, c_size_t, POINTER(c_int64), _P]),
    "mbem_near_mask_fill": (c_int, [_P, _I, _I, _P, _P, _P]),
    "mbem_near_list_workspace_size": (c_size_t, [_I]),
    "mbem_near_count": (c_int, [_P, _I, _P, _P, _I, _D, _P, _P, c_size_t, POINTER(c_int64), _P]),
    "mbem_near_fill": (c_int, [_P, _I, _P, _P, _I, _D, _P, _P, _P]),
    "mbem_near_eval": (c_int, [c_int, _P, _I, _P, _P, _P, _P, _P, _I, _P, _D, _P, _P]),
    "mbem_mixed_rowsum3": (c_int, [_P, _I, _I, _I, _P, _P, _P, _P]),
    "mbem_near_add_diagonal": (c_int, [_P, _P, _P, _I, _P, _P, _P]),
    "mbem_mixed_matvec": (c_int, [POINTER(MixedOperator), _P, _P, _P, c_size_t, _P]),
    "mbem_bf16_matvec": (c_int, [_P, _I, _I, _I, c_int, POINTER(NearBlocks), _P, _P, _P, c_size_t, _P]),
    "mbem_inner_bf16_workspace_size": (c_size_t, [_I, c_int]),
    "mbem_inner_bf16_apply": (c_int, [POINTER(InnerBf16), _P, _P, _P]),
    "mbem_inner_bf16_stats": (None, [c_int, POINTER(c_int64), POINTER(c_int64), POINTER(c_double)]),
    "mbem_mixed_matvec_noalloc": (c_int, [POINTER(MixedOperator), _P, _P, _P]),
    "mbem_mixed_wait_check": (c_int, [_P]),
    "mbem_gemm_bf16_sub": (c_int, [_P, _I, _P, _I, _I, _I, _I, _P, _I, _P]),
    "mbem_lu_workspace_size": (c_size_t, [_I, c_int]),
    "mbem_lu_factor_f32": (c_int, [_P, _I, _I, _P, _P, c_size_t, _P, _P]),
    "mbem_lu_solve_f32": (c_int, [_P, _I, _I, _P, _P, _P, _P, _P]),
    "mbem_nn_setup_dense32": (c_int, [_P, _I, _P, _P, c_int, _P, c_size_t, _P]),
    "mbem_nn_setup_mixed": (c_int, [_P, _P, _P, c_int, _P, c_size_t, _P]),
    "mbem_knn": (c_int, [_P, _I, c_int, _P, _P]),
    "mbem_dense_inverse_f32_workspace_size": (c_size_t, [_I]),
    "mbem_dense_inverse_f32": (c_int, [_P, _I, _I, _P, c_size_t, _P]),
    "mbem_dense_inverse_f32_stats": (None, [POINTER(c_int64), POINTER(c_int64)]),
    "mbem_cluster_stats": (c_int, [_P, _P, _P, _P, _I, c_int, _P, _P, _P]),
    "mbem_cluster_split": (c_int, [_P, _P, _P, _P, _P, _I, c_int, _P, _P, _P, _P, _P]),
    "mbem_lu_solve_t_f32": (c_int, [_P, _I, _I, _P, _P, _P, _P, _P]),
    "mbem_lu_stats": (None, [c_int, POINTER(c_double)]),
    "mbem_lu_solve_many_workspace_size": (c_size_t, [_I, _I]),
    "mbem_lu_solve_many_f32": (c_int, [_P, _I, _I, _P, _P, _I, _I, _P, _I, _P, c_size_t, _P]),
    "mbem_tune_count": (c_int, [c_int]),
    "mbem_tune_get": (c_int, [c_int]),
    "mbem_tune_set": (c_int, [c_int, c_int]),
    "mbem_tune_describe": (c_int, [c_int, c_int, c_char_p, c_int]),
    "mbem_mm_total": (c_int64, [POINTER(MmMesh), c_int]),
    "mbem_mm_workspace_size": (c_size_t, [POINTER(MmMesh), c_int, c_int]),
    "mbem_mm_create": (c_int, [POINTER(MmMesh), c_int, c_int, _P, c_size_t, _P, POINTER(c_void_p)]),
    "mbem_mm_destroy": (None, [_P]),
    "mbem_mm_matvec": (c_int, [_P, _P, _P, _P]),
    "mbem_mm_solve": (c_int, [_P, _P, _P, c_double, c_int, c_int, POINTER(MmReport), _P]),
    "mbem_mm_check": (c_int, [_P]),
    "mbem_mm_solve_mixed": (c_int, [_P, _P, _P, c_double, c_double, c_int, c_int, c_int, POINTER(MmReport), _P]),
    "mbem_traction_matrix_mixed": (c_int, [_P, _P, _I, _P, _P, _P, _I, _D, _D, _D, _D, _P, _P, _I, _P, _I, _P]),
    "mbem_pair_prep_bytes": (c_size_t, [_I, _I]),
    "mbem_pair_prepare": (c_int, [POINTER(PairGeometry), _P]),
    "mbem_aca_compress": (c_int, [POINTER(PairGeometry), POINTER(AcaBatch), _P]),
    "mbem_aca_compact": (c_int, [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "mbem_aca_recompress": (c_int, [POINTER(PairGeometry), POINTER(AcaRecompression), _P]),
    "mbem_pair_dense_blocks": (c_int, [POINTER(PairGeometry), _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "mbem_compressed_matvec_workspace_size": (c_size_t, [POINTER(CompressedView)]),
    "mbem_compressed_matvec": (c_int, [POINTER(CompressedView), _P, _P, _P, c_size_t, _P]),
    "mbem_compressed_to_dense": (c_int, [POINTER(CompressedView), _P, _I, _P]),
}

_lib = None


def lib():
    """The loaded library (loaded once; raises if it was never built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"mbem_gb300 CUDA library not found at {LIB_PATH}: build it with "
                f"`python -m mbem_gb300.build` (nvcc, sm_103a). There is no CPU fallback.")
        h = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def call(name: str, *args) -> None:
    """Call an entry point and raise MbemError on a non-zero status."""
    st = getattr(lib(), name)(*args)
    if st != OK:
        msg = lib().mbem_last_error()
        msg = msg.decode(errors="replace") if msg else ""
        if st == ERR_ARG:
            raise ValueError(f"{name}: {msg}")
        raise MbemError(st, name, msg)


def dbl_array(values) -> ctypes.Array:
    vals = [float(v) for v in values]
    return (c_double * len(vals))(*vals)
