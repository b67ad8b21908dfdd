"""Static condensation of Dirichlet dofs (TensorMesh ``Condenser``).

Interface and semantics of operator/condense.py:26-533: ``Condenser(mask,
value=None)``; ``__call__(K, rhs) -> (K_ii, f_i)`` with f_i = f[inner] -
K_io u_o (:238-309); ``condense_rhs`` (:388-427); ``recover`` (:429-458);
``restrict`` / ``prolong``; ``update_dirichlet``.  Boolean-mask compaction
keeps CSR order, so K_ii is again canonical CSR.

Unlike the reference (whose layout assert fires when a matrix is re-wrapped
with fresh index tensors, condense.py:291), the layout here is cached per
sparsity pattern identity, so one Condenser serves every matrix an
assembler returns.  The value gathers, the right-hand-side correction and
the recovery scatter run as CUDA kernels; gradients flow through all three.
"""
from __future__ import annotations

from typing import Optional

import torch
import torch.nn as nn

from . import _lib
from .sparse import SparseMatrix


def _dt(t):
    return _lib.TM_F64 if t.dtype == torch.float64 else _lib.TM_F32


def gather(src: torch.Tensor, index: torch.Tensor) -> torch.Tensor:
    out = torch.empty(index.shape[0], dtype=src.dtype, device=src.device)
    _lib.call("tm_gather", _dt(src), index.shape[0], index.data_ptr(), src.contiguous().data_ptr(), out.data_ptr(),
              _lib.stream_handle(src.device))
    return out


def scatter_into(dst: torch.Tensor, index: torch.Tensor, src: torch.Tensor) -> torch.Tensor:
    _lib.call("tm_scatter", _dt(src), index.shape[0], index.data_ptr(), src.contiguous().data_ptr(), dst.data_ptr(),
              _lib.stream_handle(src.device))
    return dst


class _Gather(torch.autograd.Function):
    @staticmethod
    def forward(ctx, src, index):
        ctx.save_for_backward(index)
        ctx.n = src.shape[0]
        return gather(src.detach(), index)

    @staticmethod
    def backward(ctx, g):
        (index,) = ctx.saved_tensors
        out = torch.zeros(ctx.n, dtype=g.dtype, device=g.device)
        return scatter_into(out, index, g.contiguous()), None


def gather_ad(src, index):
    if src.requires_grad:
        return _Gather.apply(src, index)
    return gather(src.detach(), index)


class Condenser(nn.Module):
    def __init__(self, dirichlet_mask: torch.Tensor, dirichlet_value: Optional[torch.Tensor] = None):
        super().__init__()
        assert dirichlet_mask.dtype == torch.bool, f"dirichlet_mask must be a bool tensor, got {dirichlet_mask.dtype}"
        assert dirichlet_mask.ndim == 1, f"dirichlet_mask must be 1D, got shape {tuple(dirichlet_mask.shape)}"
        self.register_buffer("dirichlet_mask", dirichlet_mask)
        self.register_buffer("dirichlet_value", self._normalize_value(dirichlet_value))
        self._layouts = {}
        self.K_ou2in = None
        self._io = None
        self.n_dof = int(dirichlet_mask.shape[0])
        self.n_outer_dof = int(dirichlet_mask.sum())
        self.n_inner_dof = self.n_dof - self.n_outer_dof

    def _normalize_value(self, value):
        """Prescribed values on the Dirichlet dofs only (condense.py:167-180
        accepts the same two layouts).  ``None`` means homogeneous; a vector
        over all dofs is restricted through the mask; a vector already over
        the Dirichlet dofs passes through.  Anything else is an
        AssertionError, as in the reference."""
        mask = self.dirichlet_mask
        n_all, n_fixed = int(mask.shape[0]), int(mask.sum())
        if value is None:
            return torch.zeros(n_fixed, device=mask.device)
        assert value.ndim == 1, f"expected a 1-D dirichlet_value, got {value.ndim}-D {tuple(value.shape)}"
        length = int(value.shape[0])
        assert length in (n_all, n_fixed), \
            f"dirichlet_value has {length} entries; expected {n_all} (every dof) or {n_fixed} (Dirichlet dofs)"
        if length == n_all and n_all != n_fixed:
            return value[mask.to(value.device)]
        return value

    def update_dirichlet(self, dirichlet_value: torch.Tensor):
        self.dirichlet_value = self._normalize_value(dirichlet_value)

    def _layout(self, K: SparseMatrix):
        sig = K.layout_signature
        lay = self._layouts.get(sig)
        if lay is not None:
            return lay
        dev = K.device
        mask = self.dirichlet_mask.to(dev)
        inner = ~mask
        rows, cols = K.row, K.col
        is_inner_edge = inner[rows] & inner[cols]
        is_ou2in_edge = inner[rows] & mask[cols]
        local = torch.full((K.shape[0],), -1, dtype=torch.int64, device=dev)
        inner_dof = torch.nonzero(inner).reshape(-1)
        outer_dof = torch.nonzero(mask).reshape(-1)
        local[inner_dof] = torch.arange(inner_dof.shape[0], device=dev)
        local[outer_dof] = torch.arange(outer_dof.shape[0], device=dev)
        ni = int(inner_dof.shape[0])

        def csr(sel):
            idx = torch.nonzero(sel).reshape(-1)
            r = local[rows[idx]]
            ptr = torch.zeros(ni + 1, dtype=torch.int64, device=dev)
            ptr[1:] = torch.cumsum(torch.bincount(r, minlength=ni), 0)
            return idx, ptr, local[cols[idx]].to(torch.int32)

        lay = dict(inner_dof=inner_dof, outer_dof=outer_dof, ii=csr(is_inner_edge), io=csr(is_ou2in_edge),
                   is_inner_edge=is_inner_edge, is_ou2in_edge=is_ou2in_edge, K=K)
        if len(self._layouts) > 4:
            self._layouts.clear()
        self._layouts[sig] = lay
        self.n_dof = K.shape[0]
        return lay

    @property
    def is_inner_dof(self):
        return ~self.dirichlet_mask

    @property
    def is_outer_dof(self):
        return self.dirichlet_mask

    def __call__(self, matrix: SparseMatrix, rhs: Optional[torch.Tensor] = None):
        if rhs is None:
            rhs = torch.zeros(matrix.shape[0], dtype=matrix.dtype, device=matrix.device)
        assert matrix.shape[0] == self.dirichlet_mask.shape[0] and matrix.shape[1] == matrix.shape[0], \
            f"the shape of matrix must be [{self.dirichlet_mask.shape[0]}, {self.dirichlet_mask.shape[0]}], " \
            f"but got {matrix.shape}"
        assert rhs.shape[0] == matrix.shape[0], f"the shape of rhs must be [{matrix.shape[0]}, ...], but got {rhs.shape}"
        lay = self._layout(matrix)
        ni = int(lay["inner_dof"].shape[0])
        ii_idx, ii_ptr, ii_ind = lay["ii"]
        io_idx, io_ptr, io_ind = lay["io"]
        K_ii = SparseMatrix(gather_ad(matrix.values, ii_idx), shape=(ni, ni), indptr=ii_ptr, indices=ii_ind)
        K_io = SparseMatrix(gather_ad(matrix.values, io_idx), shape=(ni, int(lay["outer_dof"].shape[0])),
                            indptr=io_ptr, indices=io_ind)
        self.K_ou2in = K_io
        self._io = lay
        self.dirichlet_value = self.dirichlet_value.to(device=matrix.device, dtype=matrix.dtype)
        return K_ii, self._condense(rhs.to(device=matrix.device, dtype=matrix.dtype), K_io, lay)

    def _condense(self, rhs, K_io, lay):
        inner_dof = lay["inner_dof"]
        uo = self.dirichlet_value
        if rhs.dim() > 1 or rhs.requires_grad or K_io.values.requires_grad or uo.requires_grad:
            minus = K_io @ uo if uo.numel() else torch.zeros(inner_dof.shape[0], dtype=rhs.dtype, device=rhs.device)
            for _ in range(rhs.dim() - 1):
                minus = minus.unsqueeze(-1)
            return rhs[inner_dof] - minus
        out = torch.empty(inner_dof.shape[0], dtype=rhs.dtype, device=rhs.device)
        io_idx, io_ptr, io_ind = lay["io"]
        _lib.call("tm_condense_rhs", _dt(rhs), inner_dof.shape[0], inner_dof.data_ptr(), rhs.contiguous().data_ptr(),
                  io_ptr.data_ptr(), io_ind.data_ptr(), K_io.values.contiguous().data_ptr(),
                  uo.contiguous().data_ptr(), out.data_ptr(), _lib.stream_handle(rhs.device))
        return out

    def condense_rhs(self, rhs: torch.Tensor) -> torch.Tensor:
        assert self.K_ou2in is not None, \
            "call the Condenser on a matrix first; condense_rhs reuses the cached K_io block"
        rhs = rhs.to(device=self.K_ou2in.device, dtype=self.K_ou2in.dtype)
        return self._condense(rhs, self.K_ou2in, self._io)

    def recover(self, u: torch.Tensor) -> torch.Tensor:
        mask = self.dirichlet_mask.to(u.device)
        n_inner = int((~mask).sum())
        assert u.shape[0] == n_inner, f"the shape of u must be [{n_inner}, ...], but got {u.shape}"
        shape = list(u.shape)
        shape[0] = mask.shape[0]
        full = torch.zeros(shape, dtype=u.dtype, device=u.device)
        bv = self.dirichlet_value.to(device=u.device, dtype=u.dtype)
        for _ in range(u.dim() - 1):
            bv = bv.unsqueeze(-1)
        full = full.index_put((torch.nonzero(~mask).reshape(-1),), u, accumulate=True)
        full = full.index_put((torch.nonzero(mask).reshape(-1),), bv.expand((int(mask.sum()),) + tuple(shape[1:])),
                              accumulate=True)
        return full

    def restrict(self, f: torch.Tensor) -> torch.Tensor:
        return f[~self.dirichlet_mask.to(f.device)]

    def prolong(self, u: torch.Tensor) -> torch.Tensor:
        mask = self.dirichlet_mask.to(u.device)
        shape = list(u.shape)
        shape[0] = mask.shape[0]
        full = torch.zeros(shape, dtype=u.dtype, device=u.device)
        return full.index_put((torch.nonzero(~mask).reshape(-1),), u, accumulate=True)
