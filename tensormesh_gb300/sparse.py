"""SparseMatrix: the assembled operator in canonical CSR form.

Mirrors the accessors of TensorMesh's ``SparseMatrix`` (sparse/matrix.py:
28-636 on top of ``torch_sla.SparseTensor``): ``values``/``edata``,
``row``/``col`` (COO view), ``shape``, ``nnz``, ``@``, ``solve``,
``to_dense``, ``to_scipy_coo``, ``from_block_coo``, ``layout_signature``,
``+``/``-``/scalar ``*``, ``transpose``/``T``, ``degree``, ``from_dense``,
``eye``.

Storage is CSR (``indptr`` int64, ``indices`` int32) in canonical order:
rows ascending, columns ascending inside a row.  For scalar forms that is
exactly the order of the reference's ``edges`` (element_assembler.py:
851-856); for block (vector) forms the reference's COO is edge-major
(matrix.py:355-375) and this class holds the canonical CSR of the same
matrix.  ``@`` and ``solve`` run hand-written CUDA kernels.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np
import torch



class SparseMatrix:
    def __init__(self, values: torch.Tensor, row: Optional[torch.Tensor] = None,
                 col: Optional[torch.Tensor] = None, shape: Optional[Tuple[int, int]] = None, *,
                 indptr: Optional[torch.Tensor] = None, indices: Optional[torch.Tensor] = None):
        if indptr is None:
            if row is None or col is None or shape is None:
                raise ValueError("SparseMatrix needs (values, row, col, shape) or indptr/indices")
            indptr, indices, values = _coo_to_csr(values, row.long(), col.long(), shape)
        self.values = values
        self.indptr = indptr
        self.indices = indices
        self.shape = (int(shape[0]), int(shape[1])) if shape is not None else (indptr.shape[0] - 1,) * 2
        self._row = None

    # -- reference accessors ---------------------------------------------------
    @property
    def edata(self) -> torch.Tensor:
        return self.values

    @property
    def row(self) -> torch.Tensor:
        if self._row is None:
            n = self.indptr.shape[0] - 1
            deg = self.indptr[1:] - self.indptr[:-1]
            self._row = torch.repeat_interleave(torch.arange(n, device=self.indptr.device), deg)
        return self._row

    row_indices = row

    @property
    def col(self) -> torch.Tensor:
        return self.indices.long()

    col_indices = col

    @property
    def edges(self) -> torch.Tensor:
        return torch.stack([self.row, self.col], 0)

    @property
    def nnz(self) -> int:
        return int(self.values.shape[0])

    @property
    def device(self) -> torch.device:
        return self.values.device

    @property
    def dtype(self) -> torch.dtype:
        return self.values.dtype

    @property
    def layout_signature(self):
        """Hashable identity of the sparsity pattern (sparse/mixin.py:48-72):
        the pattern tensors are shared by every matrix one assembler returns,
        so equal signatures mean an identical CSR pattern."""
        return (self.indptr.data_ptr(), self.indptr._version, self.indices.data_ptr(),
                self.indices._version, self.nnz, self.shape)

    def has_same_layout(self, other) -> bool:
        sig = other if isinstance(other, tuple) else other.layout_signature
        return self.layout_signature == sig

    def with_values(self, values: torch.Tensor) -> "SparseMatrix":
        m = SparseMatrix(values, shape=self.shape, indptr=self.indptr, indices=self.indices)
        m._row = self._row
        return m

    def double(self) -> "SparseMatrix":
        return self.with_values(self.values.double())

    def float(self) -> "SparseMatrix":
        return self.with_values(self.values.float())

    def to(self, device) -> "SparseMatrix":
        return SparseMatrix(self.values.to(device), shape=self.shape, indptr=self.indptr.to(device),
                            indices=self.indices.to(device))

    def to_dense(self) -> torch.Tensor:
        d = torch.zeros(self.shape, dtype=self.dtype, device=self.device)
        d[self.row, self.col] = self.values
        return d

    def to_scipy_coo(self):
        import scipy.sparse as sp
        return sp.coo_matrix((self.values.detach().cpu().numpy(),
                              (self.row.cpu().numpy(), self.col.cpu().numpy())), shape=self.shape)

    def to_scipy_csr(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.values.detach().cpu().numpy(), self.indices.cpu().numpy(),
                              self.indptr.cpu().numpy()), shape=self.shape)

    def diagonal(self) -> torch.Tensor:
        from .solve import csr_diagonal
        return csr_diagonal(self)

    @property
    def grad(self) -> Optional["SparseMatrix"]:
        """The gradient of the values as a matrix of the same pattern, or None."""
        g = self.values.grad
        return None if g is None else self.with_values(g)

    def detach(self) -> "SparseMatrix":
        return self.with_values(self.values.detach())

    def cpu(self) -> "SparseMatrix":
        return self.to("cpu")

    def cuda(self, device=None) -> "SparseMatrix":
        return self.to("cuda" if device is None else device)

    def degree(self, axis: int = 0) -> torch.Tensor:
        """Entries per row (axis 0) or per column (axis 1) (matrix.py:213-229)."""
        if axis == 0:
            return self.indptr[1:] - self.indptr[:-1]
        return torch.bincount(self.col, minlength=self.shape[1])

    def transpose(self) -> "SparseMatrix":
        """A^T in canonical CSR (matrix.py:231-243); differentiable in the values."""
        return SparseMatrix(self.values, self.col, self.row, (self.shape[1], self.shape[0]))

    @property
    def T(self) -> "SparseMatrix":
        return self.transpose()

    # -- arithmetic (matrix.py:154-178): on the values, so autograd flows ------
    def _same_pattern(self, other: "SparseMatrix") -> bool:
        if self.shape != other.shape or self.nnz != other.nnz:
            return False
        return self.has_same_layout(other) or (
            torch.equal(self.indptr, other.indptr.to(self.indptr.device)) and
            torch.equal(self.indices, other.indices.to(self.indices.device)))

    def __add__(self, other):
        if isinstance(other, SparseMatrix):
            assert self.shape == other.shape, f"shape mismatch {self.shape} vs {other.shape}"
            ov = other.values.to(device=self.device, dtype=self.dtype)
            if self._same_pattern(other):
                return self.with_values(self.values + ov)
            # union of the two patterns; a position holds at most one entry of
            # each operand, so the sum does not depend on the order of the adds
            return SparseMatrix(torch.cat([self.values, ov]), torch.cat([self.row, other.row.to(self.device)]),
                                torch.cat([self.col, other.col.to(self.device)]), self.shape)
        if isinstance(other, (int, float)) and other == 0:
            return self
        return NotImplemented

    __radd__ = __add__

    def __neg__(self) -> "SparseMatrix":
        return self.with_values(-self.values)

    def __sub__(self, other):
        if isinstance(other, SparseMatrix):
            return self + (-other)
        if isinstance(other, (int, float)) and other == 0:
            return self
        return NotImplemented

    def __rsub__(self, other):
        if isinstance(other, (int, float)) and other == 0:
            return -self
        return NotImplemented

    def __mul__(self, other):
        if isinstance(other, SparseMatrix):
            if not self._same_pattern(other):
                raise NotImplementedError("elementwise product of matrices with different patterns")
            return self.with_values(self.values * other.values.to(device=self.device, dtype=self.dtype))
        if isinstance(other, (int, float)) or (torch.is_tensor(other) and other.dim() == 0):
            return self.with_values(self.values * other)
        return NotImplemented

    __rmul__ = __mul__

    def __truediv__(self, other):
        if isinstance(other, (int, float)) or (torch.is_tensor(other) and other.dim() == 0):
            return self.with_values(self.values / other)
        return NotImplemented

    @staticmethod
    def from_dense(tensor: torch.Tensor) -> "SparseMatrix":
        """The nonzero entries of a dense 2-D tensor (matrix.py:309-324)."""
        assert tensor.dim() == 2, f"a 2-D tensor is required, got {tuple(tensor.shape)}"
        r, c = torch.nonzero(tensor, as_tuple=True)
        return SparseMatrix(tensor[r, c], r, c, tuple(tensor.shape))

    @staticmethod
    def eye(n: int, value: float = 1.0, dtype=None, device=None) -> "SparseMatrix":
        """value * I (matrix.py:439-459)."""
        i = torch.arange(n, device=device)
        v = torch.full((n,), value, dtype=dtype or torch.get_default_dtype(), device=device)
        return SparseMatrix(v, i, i, (n, n))

    # -- operators -------------------------------------------------------------
    def __matmul__(self, x: torch.Tensor) -> torch.Tensor:
        from .solve import spmv
        return spmv(self, x)

    def solve(self, b: torch.Tensor, **kwargs) -> torch.Tensor:
        """Solve K x = b with Jacobi-preconditioned CG on the GPU.

        Keyword arguments follow the reference's ``K.solve`` (torch_sla
        signature, docs user_guide/linear_solvers.rst:80-110): ``atol``,
        ``rtol``/``tol`` (relative to ||b||, default 1e-8), ``maxiter``,
        ``method`` ("cg"/"pcg"/"jacobi-pcg"; "auto" accepted),
        ``preconditioner`` ("jacobi" or a learned preconditioner object).
        Non-convergence warns (torch_solve.py:125-126).
        """
        from .solve import solve
        return solve(self, b, **kwargs)

    @staticmethod
    def from_block_coo(edata: torch.Tensor, row: torch.Tensor, col: torch.Tensor,
                       shape: Tuple[int, int]) -> "SparseMatrix":
        """Expand [n, H, H] blocks at (row, col) to a flat matrix with
        dof (H*row + a, H*col + b) (sparse/matrix.py:325-375)."""
        H = edata.shape[1]
        a = torch.arange(H, device=row.device)
        r = (row.long()[:, None, None] * H + a[None, :, None]).expand(-1, H, H).reshape(-1)
        c = (col.long()[:, None, None] * H + a[None, None, :]).expand(-1, H, H).reshape(-1)
        return SparseMatrix(edata.reshape(-1), r, c, (shape[0] * H, shape[1] * H))


def _coo_to_csr(values, row, col, shape):
    """Canonical CSR of a COO triple (duplicates summed in input order)."""
    n = int(shape[0])
    key = row * int(shape[1]) + col
    uniq, inv = torch.unique(key, sorted=True, return_inverse=True)
    vals = torch.zeros(uniq.shape[0], dtype=values.dtype, device=values.device).index_add(0, inv, values)
    r = torch.div(uniq, int(shape[1]), rounding_mode="floor")
    cidx = (uniq - r * int(shape[1])).to(torch.int32)
    indptr = torch.zeros(n + 1, dtype=torch.int64, device=values.device)
    indptr[1:] = torch.cumsum(torch.bincount(r, minlength=n), 0)
    return indptr, cidx, vals
