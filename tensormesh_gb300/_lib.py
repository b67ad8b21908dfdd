"""ctypes binding of the C ABI declared in ``include/tensormesh_gb300.h``.

The shared library is built in-tree by ``tensormesh_gb300.build``.  There is
no fallback: if the library is missing or CUDA is unavailable, every GPU
entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

TM_OK, TM_ERR_INVALID, TM_ERR_INDEX, TM_ERR_MAXITER, TM_ERR_BREAKDOWN, TM_ERR_CUDA, \
    TM_ERR_UNSUPPORTED, TM_ERR_TIMEOUT = range(8)
TM_TRI3, TM_TRI6, TM_TET4, TM_TET10 = range(4)
TM_FORM_LAPLACE, TM_FORM_MASS, TM_FORM_ELASTICITY, TM_FORM_LOAD = range(4)
TM_F32, TM_F64 = 0, 1
TM_PREC_EMULATED, TM_PREC_NATIVE = 0, 1
TM_PCG_STANDARD, TM_PCG_PIPELINED, TM_PCG_NARROW = 0, 1, 2
TM_COEF_SCALAR, TM_COEF_ELEMENT, TM_COEF_POINT, TM_COEF_QUAD = range(4)

STATUS_NAMES = {
    TM_OK: "ok", TM_ERR_INVALID: "invalid argument", TM_ERR_INDEX: "index or size out of range",
    TM_ERR_MAXITER: "iteration cap reached", TM_ERR_BREAKDOWN: "solver breakdown",
    TM_ERR_CUDA: "CUDA launch failure", TM_ERR_UNSUPPORTED: "unsupported combination",
    TM_ERR_TIMEOUT: "bounded device wait timed out",
}

# Every exported symbol the header declares (checked by the CPU test suite).
EXPORTS = [
    "tm_assemble", "tm_quadrature_points", "tm_spmv_csr",
    "tm_pcg_workspace_bytes", "tm_pcg_max_blocks", "tm_pcg_jacobi", "tm_pcg_result",
    "tm_csr_diagonal_inverse", "tm_gather", "tm_scatter", "tm_condense_rhs",
    "tm_assemble_backward", "tm_segment_sum",
    "tm_batched_assemble_pcg", "tm_batched_max_clusters", "tm_patch_smem_bytes",
    "tm_mpnn_input_fwd", "tm_mpnn_layer_fwd", "tm_mpnn_readout_fwd", "tm_mpnn_readout_bwd",
    "tm_mpnn_layer_bwd", "tm_mpnn_input_bwd", "tm_gather_axpy_f32",
    "tm_pcg_jacobi_noalloc", "tm_twolevel_apply", "tm_neohookean", "tm_facet_load",
    "tm_selftest_barrier_timeout", "tm_pattern_workspace_bytes", "tm_pattern_count", "tm_pattern_fill",
    "tm_morton_keys",
    "tm_sell_plan", "tm_pcg_sell_workspace_bytes", "tm_pcg_jacobi_sell",
    "tm_fcg_workspace_doubles", "tm_fcg_twolevel_iterations", "tm_kp_count", "tm_kp_fill",
    "tm_sell_fill", "tm_spmv_sell",
]

P = ctypes.c_void_p


class PatchPlan(ctypes.Structure):
    _fields_ = [
        ("n_patches", ctypes.c_int32), ("n_elements", ctypes.c_int32),
        ("n_points", ctypes.c_int32), ("n_basis", ctypes.c_int32),
        ("vptr", P), ("vtx", P), ("eptr", P), ("elem", P), ("econn", P),
        ("rptr", P), ("rows", P), ("racc", P), ("iptr", P),
        ("inc_elem", P), ("inc_a", P), ("inc_pos", P), ("indptr", P),
        ("max_vtx", ctypes.c_int32), ("max_slots", ctypes.c_int32),
        ("max_rows", ctypes.c_int32), ("max_elems", ctypes.c_int32),
        ("inc_pack", P), ("inc_pack32", P), ("rdiag", P),
        ("max_deg", ctypes.c_int32), ("pad1", ctypes.c_int32),
    ]


class TwoLevel(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64), ("nc", ctypes.c_int32), ("pad0", ctypes.c_int32),
        ("agg", P), ("agg_ptr", P), ("agg_perm", P), ("kc_inv", P),
        ("kp_indptr", P), ("kp_indices", P), ("kp_values", P),
        ("k_nnz", ctypes.c_int64), ("k_indptr", P), ("k_indices", P), ("k_values", P),
        ("sw", P), ("work", P),
        ("k_slice_ptr", P), ("k_scol", P), ("k_sval", P), ("k_narrow", ctypes.c_int32), ("pad1", ctypes.c_int32),
        ("kc_half", P), ("kc_scale", P),
    ]


class AssembleArgs(ctypes.Structure):
    _fields_ = [
        ("element", ctypes.c_int32), ("form", ctypes.c_int32), ("dtype", ctypes.c_int32),
        ("precision", ctypes.c_int32), ("coef_kind", ctypes.c_int32), ("n_comp", ctypes.c_int32),
        ("n_quad", ctypes.c_int32), ("pad0", ctypes.c_int32),
        ("tables", P), ("points", P), ("coef", P),
        ("scal", ctypes.c_double * 3), ("lam", ctypes.c_double), ("mu", ctypes.c_double), ("out", P),
    ]


class BackwardArgs(ctypes.Structure):
    _fields_ = [("grad_out", P), ("pair_dX", P), ("pair_dcoef", P)]


class BatchedArgs(ctypes.Structure):
    _fields_ = [
        ("element", ctypes.c_int32), ("cluster", ctypes.c_int32), ("n_clusters", ctypes.c_int32),
        ("n_inst", ctypes.c_int32), ("maxiter", ctypes.c_int32), ("chunk", ctypes.c_int32),
        ("rtol", ctypes.c_float), ("pad0", ctypes.c_int32),
        ("n_rows", ctypes.c_int64), ("smem_bytes", ctypes.c_int64),
        ("plan", ctypes.POINTER(PatchPlan)), ("mat", ctypes.POINTER(AssembleArgs)),
        ("load", ctypes.POINTER(AssembleArgs)),
        ("order", P), ("inst_pbeg", P), ("inst_rbeg", P), ("indices", P), ("dirichlet", P),
        ("x", P), ("work", P), ("status", P), ("iters", P), ("resid", P), ("queue", P), ("stream", P),
    ]


class TensorMeshCudaError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, fn: str, status: int):
        super().__init__(f"{fn} failed: {STATUS_NAMES.get(status, status)} (status {status})")
        self.status = status


_lib = None
_lock = threading.Lock()


def _declare(lib):
    i32, i64 = ctypes.c_int32, ctypes.c_int64
    sig = {
        "tm_assemble": [ctypes.POINTER(PatchPlan), ctypes.POINTER(AssembleArgs), P],
        "tm_quadrature_points": [i32, i32, i32, P, P, P, i64, P, P],
        "tm_spmv_csr": [i32, i64, i64, P, P, P, P, P, P],
        "tm_pcg_jacobi": [i32, i64, P, P, P, P, P, ctypes.c_double, ctypes.c_double, i32, P, i64, P],
        "tm_pcg_result": [P, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_double),
                          ctypes.POINTER(ctypes.c_double), P],
        "tm_csr_diagonal_inverse": [i32, i64, P, P, P, P, P],
        "tm_gather": [i32, i64, P, P, P, P],
        "tm_scatter": [i32, i64, P, P, P, P],
        "tm_condense_rhs": [i32, i64, P, P, P, P, P, P, P, P],
        "tm_assemble_backward": [ctypes.POINTER(PatchPlan), ctypes.POINTER(AssembleArgs),
                                 ctypes.POINTER(BackwardArgs), P],
        "tm_segment_sum": [i32, i64, P, P, i32, P, P, P],
        "tm_batched_assemble_pcg": [ctypes.POINTER(BatchedArgs), P],
        "tm_batched_max_clusters": [i32, i32, i64],
        "tm_mpnn_input_fwd": [i64, P, P, P, P, P, P, P, P],
        "tm_mpnn_layer_fwd": [i64, P, P, P, P, P, P, P, i32, P],
        "tm_mpnn_readout_fwd": [i64, P, P, P, P, P, P, P, P, P, P],
        "tm_mpnn_readout_bwd": [i64, P, P, P, P, P, P, P, P, P, P],
        "tm_mpnn_layer_bwd": [i64, P, P, P, P, P, P, P, i32, P, P, P, P, P, P, P, P],
        "tm_mpnn_input_bwd": [i64, P, P, P, P, P, P, P],
        "tm_gather_axpy_f32": [i64, P, P, P, P, P, P, P, P],
        "tm_pcg_jacobi_noalloc": [i64, P, P, P, P, P, ctypes.c_double, ctypes.c_double, i32,
                                  ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_double), P],
        "tm_twolevel_apply": [ctypes.POINTER(TwoLevel), P, P, P],
        "tm_fcg_twolevel_iterations": [ctypes.POINTER(TwoLevel), i64, P, P, P, P, i32, P, P, P, P, P, P, P, P, P, i32,
                                       P],
        "tm_sell_fill": [i32, i64, P, P, P, P, i64, i32, P, P, P, P],
        "tm_spmv_sell": [i32, i64, P, i32, P, P, P, P, P],
        "tm_kp_count": [i64, P, P, P, P, P],
        "tm_kp_fill": [i64, P, P, P, P, P, P, P, P],
        "tm_neohookean": [i32, i32, i32, P, P, P, i64, P, ctypes.c_double, ctypes.c_double, P, P, P],
        "tm_facet_load": [i32, i32, i32, P, P, P, P, i64, i32, P, ctypes.POINTER(ctypes.c_double), i32, P, P, P],
        "tm_selftest_barrier_timeout": [i32, i64, ctypes.POINTER(i32), P, P],
        "tm_pattern_count": [P, i64, i32, i64, P, P, P],
        "tm_pattern_fill": [P, i64, i32, i64, P, P, P, P, P],
        "tm_morton_keys": [i64, i32, P, P, P, i32, P, P],
        "tm_pcg_jacobi_sell": [i32, i64, P, P, P, P, i64, P, P, ctypes.c_double, ctypes.c_double, i32, i32, P, i64,
                               P],
    }
    lib.tm_sell_plan.argtypes = [i64, P, P, P, ctypes.POINTER(i32), P]
    lib.tm_fcg_workspace_doubles.argtypes = []
    lib.tm_fcg_workspace_doubles.restype = i64
    lib.tm_sell_plan.restype = i64
    lib.tm_pcg_sell_workspace_bytes.argtypes = [i32, i64, i64]
    lib.tm_pcg_sell_workspace_bytes.restype = i64
    lib.tm_pattern_workspace_bytes.argtypes = [i64, i32, i64]
    lib.tm_pattern_workspace_bytes.restype = i64
    lib.tm_patch_smem_bytes.argtypes = [i32, i32, i32, i32, ctypes.POINTER(PatchPlan), i32, i32]
    lib.tm_patch_smem_bytes.restype = i64
    lib.tm_pcg_workspace_bytes.argtypes = [i32, i64, i64, i32]
    lib.tm_pcg_workspace_bytes.restype = i64
    lib.tm_pcg_max_blocks.argtypes = [i32]
    lib.tm_pcg_max_blocks.restype = ctypes.c_int
    for name, argtypes in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = ctypes.c_int


def library_path() -> str:
    return _build.lib_path()


def load(build_if_missing: bool = True):
    """Load (building first if needed) the shared library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"tensormesh_gb300 native library not built: {path}")
            _build.build()
        lib = ctypes.CDLL(path)
        _declare(lib)
        _lib = lib
        return lib


def call(name: str, *args):
    """Call a C-ABI function and raise TensorMeshCudaError on a bad status."""
    fn = getattr(load(), name)
    status = fn(*args)
    if status != TM_OK:
        raise TensorMeshCudaError(name, status)
    return status


def call_status(name: str, *args) -> int:
    """Call a C-ABI function and return its status (solvers report
    non-convergence through the status rather than raising)."""
    return getattr(load(), name)(*args)


def ptr(t) -> int:
    """Device (or host) address of a tensor; None -> NULL."""
    return 0 if t is None else t.data_ptr()


def stream_handle(device) -> int:
    import torch
    return torch.cuda.current_stream(device).cuda_stream
