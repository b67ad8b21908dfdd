"""SpMV and Jacobi-PCG on the GPU (``SparseMatrix.__matmul__`` / ``.solve``).

``solve`` mirrors the reference's ``K.solve(b, **kw)`` (torch_sla signature;
docs user_guide/linear_solvers.rst:80-110) for SPD systems: the solve runs
as one cooperative CUDA launch (``tm_pcg_jacobi``), then the true residual
||b - K x|| / ||b|| is recomputed with a plain SpMV; if it is above the
target although the recurrence met it, the solve continues by iterative
refinement (a bounded number of correction solves).  Non-convergence warns, as the reference does
(sparse/solve/torch_solve.py:125-126, 245-246).  Gradients flow through the
adjoint rule of SparseSolveScipy.backward (sparse/solve/scipy_solve.py:42-53):
grad_b = K^-T g (one more PCG; K is symmetric), grad_values = -grad_b[row] u[col].
"""
from __future__ import annotations

import math
import warnings
from dataclasses import dataclass

import torch

from . import _lib


@dataclass
class SolveInfo:
    status: int
    iterations: int
    residual: float          # true ||b - Kx|| / ||b|| (FP64 SpMV)
    recurrence_residual: float
    restarts: int


def _dt(t: torch.Tensor) -> int:
    if t.dtype == torch.float64:
        return _lib.TM_F64
    if t.dtype == torch.float32:
        return _lib.TM_F32
    raise TypeError(f"unsupported dtype {t.dtype}")


def spmv_raw(indptr, indices, values, x, out=None):
    n = indptr.shape[0] - 1
    if out is None:
        out = torch.empty(n, dtype=values.dtype, device=values.device)
    _lib.call("tm_spmv_csr", _dt(values), n, int(values.shape[0]), indptr.data_ptr(), indices.data_ptr(),
              values.data_ptr(),
              x.data_ptr(), out.data_ptr(), _lib.stream_handle(values.device))
    return out


class _SpMV(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, x, A):
        ctx.A = A
        ctx.save_for_backward(values, x)
        return spmv_raw(A.indptr, A.indices, values.detach().contiguous(), x.detach().contiguous())

    @staticmethod
    def backward(ctx, g):
        values, x = ctx.saved_tensors
        A = ctx.A
        gv = gx = None
        if ctx.needs_input_grad[0]:
            gv = g[A.row] * x[A.col]
        if ctx.needs_input_grad[1]:
            # A^T g = per column c, the sum over its entries k of values[k] g[row[k]],
            # reduced in a fixed (row-ascending) order by tm_segment_sum so the
            # gradient is bitwise repeatable (no atomics)
            from .adjoint import segment_sum
            ptr, perm = _column_order(A)
            prod = (values.detach() * g[A.row]).contiguous()
            gx = segment_sum(ptr, perm, prod, 1).view(-1)[: A.shape[1]]
        return gv, gx, None


def _column_order(A):
    """CSC view of A's pattern: column pointer and the CSR positions of every
    column's entries in ascending row order (cached on the matrix)."""
    cached = getattr(A, "_csc", None)
    if cached is not None:
        return cached
    col = A.col
    ncol = A.shape[1]
    perm = torch.argsort(col * max(1, A.shape[0]) + A.row)
    counts = torch.bincount(col, minlength=ncol)
    ptr = torch.zeros(ncol + 1, dtype=torch.int64, device=col.device)
    ptr[1:] = torch.cumsum(counts, 0)
    A._csc = (ptr, perm)
    return A._csc


def spmv(A, x: torch.Tensor) -> torch.Tensor:
    if not A.values.is_cuda:
        raise RuntimeError("SparseMatrix @ runs on CUDA only")
    x = x.to(dtype=A.dtype)
    if x.dim() == 2:
        return torch.stack([spmv(A, x[:, j]) for j in range(x.shape[1])], 1)
    if A.values.requires_grad or x.requires_grad:
        return _SpMV.apply(A.values, x, A)
    return spmv_raw(A.indptr, A.indices, A.values.detach().contiguous(), x.contiguous())


def csr_diagonal(A) -> torch.Tensor:
    """diag(A) (missing entries -> 1, as torch_solve.py:24-49)."""
    out = torch.empty(A.shape[0], dtype=A.dtype, device=A.device)
    _lib.call("tm_csr_diagonal_inverse", _dt(A.values), A.shape[0], A.indptr.data_ptr(), A.indices.data_ptr(),
              A.values.detach().contiguous().data_ptr(), out.data_ptr(), _lib.stream_handle(A.device))
    return 1.0 / out


class PCGWorkspace:
    """Device scratch for tm_pcg_jacobi, reused across solves of one size."""

    def __init__(self, n: int, nnz: int, dtype: torch.dtype, device):
        lib = _lib.load()
        code = _lib.TM_F64 if dtype == torch.float64 else _lib.TM_F32
        self.max_blocks = lib.tm_pcg_max_blocks(code)
        self.nbytes = int(lib.tm_pcg_workspace_bytes(code, n, nnz, self.max_blocks))
        self.buf = torch.empty(self.nbytes, dtype=torch.uint8, device=device)
        self.n, self.nnz, self.dtype = n, nnz, dtype


class SellWorkspace:
    """Device scratch for tm_pcg_jacobi_sell (n rows, n_pad SELL-32 entries)."""

    def __init__(self, n: int, n_pad: int, dtype: torch.dtype, device):
        lib = _lib.load()
        code = _lib.TM_F64 if dtype == torch.float64 else _lib.TM_F32
        self.nbytes = int(lib.tm_pcg_sell_workspace_bytes(code, n, n_pad))
        if self.nbytes < 0:
            raise _lib.TensorMeshCudaError("tm_pcg_sell_workspace_bytes", -self.nbytes)
        self.buf = torch.empty(self.nbytes, dtype=torch.uint8, device=device)


_WS = {}


def _cached(key, make):
    ws = _WS.get(key)
    if ws is None:
        if len(_WS) > 4:
            _WS.clear()
        ws = _WS[key] = make()
    return ws


def workspace(n, nnz, dtype, device) -> PCGWorkspace:
    return _cached(("csr", n, nnz, dtype, str(device)), lambda: PCGWorkspace(n, nnz, dtype, device))


def sell_plan(indptr: torch.Tensor, indices: torch.Tensor):
    """(slice_ptr, n_pad, narrow) of the SELL-32 layout of a CSR pattern
    (tm_sell_plan; narrow: every |column - row| fits 16 bits), cached on the
    indices tensor while the pattern tensors are unmodified."""
    key = (indptr.data_ptr(), indptr._version, indices._version)
    cached = getattr(indices, "_tm_sell", None)
    if cached is not None and cached[0] == key:
        return cached[1], cached[2], cached[3]
    n = indptr.shape[0] - 1
    sp = torch.empty((n + 31) // 32 + 1, dtype=torch.int64, device=indptr.device)
    narrow = _lib.ctypes.c_int32(0)
    n_pad = int(_lib.load().tm_sell_plan(n, indptr.data_ptr(), indices.data_ptr(), sp.data_ptr(),
                                         _lib.ctypes.byref(narrow), _lib.stream_handle(indptr.device)))
    if n_pad < 0:
        raise _lib.TensorMeshCudaError("tm_sell_plan", -n_pad)
    indices._tm_sell = (key, sp, n_pad, bool(narrow.value))
    return sp, n_pad, bool(narrow.value)


# "sell": standard PCG over the SELL-32 copy (tm_pcg_jacobi_sell); "sell-pipelined":
# the one-barrier pipelined form over the same copy (a breakdown restarts it
# from the current iterate); "csr": the CSR kernel (tm_pcg_jacobi).
LAYOUT = "sell"


def pcg_jacobi_raw(indptr, indices, values, b, x, rtol=1e-8, atol=0.0, maxiter=100000, max_restarts=5):
    """Solve in place into x; returns SolveInfo.

    The first pass solves from x.  If the true residual ||b - K x|| / ||b||
    (recomputed with the plain SpMV in the value type) is still above the
    target although the recurrence met it -- FP64 systems iterate in
    double-float, whose ~48-bit products floor the attainable residual near
    cond(K) * 2^-48 -- each restart is one step of iterative refinement: the
    residual r = b - K x in the value type, a solve K d = r from zero to the
    accuracy the remaining gap needs, and x += d."""
    n = b.shape[0]
    dev = values.device
    s = _lib.stream_handle(dev)
    code = _dt(values)
    pipelined = LAYOUT == "sell-pipelined"
    if LAYOUT in ("sell", "sell-pipelined"):
        sp, n_pad, narrow = sell_plan(indptr, indices)
        ws = _cached(("sell", n, n_pad, values.dtype, str(dev)), lambda: SellWorkspace(n, n_pad, values.dtype, dev))
        method = (_lib.TM_PCG_PIPELINED if pipelined else _lib.TM_PCG_STANDARD) | (_lib.TM_PCG_NARROW if narrow else 0)

        def launch(rhs, sol, rt, at, budget):
            _lib.call("tm_pcg_jacobi_sell", code, n, indptr.data_ptr(), indices.data_ptr(), values.data_ptr(),
                      sp.data_ptr(), n_pad, rhs.data_ptr(), sol.data_ptr(), rt, at, budget, method,
                      ws.buf.data_ptr(), ws.nbytes, s)
    else:
        ws = workspace(n, int(values.shape[0]), values.dtype, dev)

        def launch(rhs, sol, rt, at, budget):
            _lib.call("tm_pcg_jacobi", code, n, indptr.data_ptr(), indices.data_ptr(), values.data_ptr(),
                      rhs.data_ptr(), sol.data_ptr(), rt, at, budget, ws.buf.data_ptr(), ws.nbytes, s)
    bnorm = float(torch.linalg.vector_norm(b.double()))
    target = max(rtol, atol / max(bnorm, 1e-300))
    total_it = 0
    restarts = 0
    info = None
    rhs, sol, inner_rtol, inner_atol = b, x, float(rtol), float(atol)
    while True:
        budget = max(0, maxiter - total_it)
        launch(rhs, sol, inner_rtol, inner_atol, int(budget))
        it = _lib.ctypes.c_int32(0)
        res = _lib.ctypes.c_double(0.0)
        bn = _lib.ctypes.c_double(0.0)
        status = _lib.load().tm_pcg_result(ws.buf.data_ptr(), _lib.ctypes.byref(it), _lib.ctypes.byref(res),
                                           _lib.ctypes.byref(bn), s)
        total_it += it.value
        if status in (_lib.TM_ERR_TIMEOUT, _lib.TM_ERR_CUDA, _lib.TM_ERR_INDEX):
            raise _lib.TensorMeshCudaError("tm_pcg_jacobi", status)
        if sol is not x:
            x.add_(sol)
        true_res = true_relative_residual(indptr, indices, values, b, x, bnorm)
        info = SolveInfo(status, total_it, true_res, res.value / max(bnorm, 1e-300), restarts)
        retry = status == _lib.TM_OK or (pipelined and status == _lib.TM_ERR_BREAKDOWN)
        if not retry or true_res <= target * 1.0000001 or restarts >= max_restarts or total_it >= maxiter:
            return info
        restarts += 1
        rhs = (b - spmv_raw(indptr, indices, values, x)).contiguous()
        rnorm = float(torch.linalg.vector_norm(rhs.double()))
        sol = torch.zeros_like(x)
        # ||rhs - K d|| <= target ||b|| / 2 leaves room for the update's rounding
        inner_rtol = min(0.5, 0.5 * target * bnorm / max(rnorm, 1e-300))
        inner_atol = 0.0


def true_relative_residual(indptr, indices, values, b, x, bnorm=None) -> float:
    """||b - A x|| / ||b|| with the plain SpMV in the matrix's dtype
    (FP64 for FP64 systems), accumulated in float64."""
    Ax = spmv_raw(indptr, indices, values, x)
    r = (b.double() - Ax.double())
    bn = float(torch.linalg.vector_norm(b.double())) if bnorm is None else bnorm
    return float(torch.linalg.vector_norm(r)) / max(bn, 1e-300)


class _Solve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, b, A, kw):
        x = _solve_nograd(A, values.detach(), b.detach(), kw)
        ctx.A, ctx.kw = A, kw
        ctx.save_for_backward(values, x)
        return x

    @staticmethod
    def backward(ctx, g):
        values, x = ctx.saved_tensors
        A = ctx.A
        # K symmetric (built-in forms): K^-T g = K^-1 g
        gb = _solve_nograd(A, values.detach(), g.contiguous(), ctx.kw)
        gv = -gb[A.row] * x[A.col] if ctx.needs_input_grad[0] else None
        return gv, gb if ctx.needs_input_grad[1] else None, None, None


def _solve_nograd(A, values, b, kw):
    rtol = kw.get("rtol", kw.get("tol", 1e-8))
    atol = kw.get("atol", 0.0)
    maxiter = int(kw.get("maxiter", max(1000, 20 * int(math.sqrt(A.shape[0])) * 10)))
    pre = kw.get("preconditioner", "jacobi")
    b = b.to(dtype=values.dtype).contiguous()
    x = torch.zeros_like(b) if kw.get("x0") is None else kw["x0"].to(b).clone()
    if pre == "jacobi" or pre is None:
        info = pcg_jacobi_raw(A.indptr, A.indices, values.contiguous(), b, x, rtol, atol, maxiter)
    else:
        info = pre.solve(A.with_values(values), b, x, rtol=rtol, atol=atol, maxiter=maxiter)
    A.last_solve_info = info
    if info.status != _lib.TM_OK or info.residual > max(rtol, 1e-300) * 1.0000001 + atol / max(
            float(torch.linalg.vector_norm(b.double())), 1e-300):
        warnings.warn(f"PCG did not converge: status={_lib.STATUS_NAMES.get(info.status)} after "
                      f"{info.iterations} iterations, relative residual {info.residual:.3e}")
    return x


def solve(A, b: torch.Tensor, **kw) -> torch.Tensor:
    if not A.values.is_cuda:
        raise RuntimeError("SparseMatrix.solve runs on CUDA only")
    method = kw.pop("method", "cg")
    kw.pop("backend", None)
    kw.pop("verbose", None)
    if method not in ("cg", "pcg", "jacobi-pcg", "auto", None):
        raise NotImplementedError(f"method {method!r}: the GPU path implements Jacobi-PCG for SPD systems")
    if A.values.requires_grad or b.requires_grad:
        return _Solve.apply(A.values, b, A, kw)
    return _solve_nograd(A, A.values, b, kw)
