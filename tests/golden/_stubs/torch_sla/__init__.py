"""Minimal stand-in for the ``torch_sla`` package (``SparseTensor``
container only), used only to import the reference TensorMesh package when
generating golden fixtures.

The reference subclasses ``torch_sla.SparseTensor`` for its ``SparseMatrix``
(tensormesh/sparse/matrix.py:28, 78-84) and reads ``.values``,
``.row_indices``, ``.col_indices``, ``.shape``; ``@`` is used by the
Condenser (tensormesh/operator/condense.py:305).  ``solve`` is not stubbed:
golden solves use scipy directly.
"""
import torch

from . import distributed  # noqa: F401


class SparseTensor:
    def __init__(self, values, row, col, shape):
        self.values = values
        self.row_indices = row
        self.col_indices = col
        self.shape = tuple(int(s) for s in shape)

    @property
    def nnz(self):
        return self.values.shape[0]

    @property
    def device(self):
        return self.values.device

    @property
    def dtype(self):
        return self.values.dtype

    def to_dense(self):
        d = torch.zeros(self.shape, dtype=self.values.dtype, device=self.values.device)
        d.index_put_((self.row_indices, self.col_indices), self.values, accumulate=True)
        return d

    def __matmul__(self, x):
        y = torch.zeros((self.shape[0],) + tuple(x.shape[1:]), dtype=self.values.dtype,
                        device=self.values.device)
        contrib = self.values.reshape((-1,) + (1,) * (x.dim() - 1)) * x[self.col_indices]
        return y.index_add(0, self.row_indices, contrib)
