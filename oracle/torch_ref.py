"""The reference's own CPU operation sequence for the element assembly, in
torch (test infrastructure: the timed CPU baseline of ``bench.py`` and its
tests; never part of the product).

``oracle.fem`` restates the algorithm in numpy; this module instead repeats
the *operations* TensorMesh runs on the CPU for ``ElementAssembler.__call__``
with a per-element coefficient, in the same order and with the same torch
primitives, so its timing stands for the reference's CPU path on any machine
(the reference package itself cannot be shipped to a machine without its
source tree):

  1. element coordinates ``points[elements]``
     (element/transformation.py:1236-1293 ``batch_elements_coords``);
  2. Jacobians ``einsum("ebj,qib->eqij")``, ``torch.inverse``, physical
     gradients ``einsum("qib,eqji->eqbj")`` (element/element.py:874-968);
  3. ``JxW = einsum("q,eq->eq", w, |det J|)`` (transformation.py:1289);
  4. the integrand ``kappa * (gradu @ gradv)`` mapped by four nested
     ``torch.func.vmap`` over (element, quadrature point, u basis, v basis)
     with the reference's in_dims (assemble/element_assembler.py:326-395);
  5. ``einsum("eqij,eq->eij")`` (``_integrate``, element_assembler.py:196-221);
  6. ``index_add_`` of the flattened element matrices into the CSR values by
     the precomputed slot map (``ReduceProjector``, assemble/projector.py:125);
  7. the per-call work around them: the gather of the point data ``x`` the
     reference always registers (element_assembler.py:318, 414) and the
     int64 copies of the int32 edge pattern made when the result is wrapped
     (``_build_output``, sparse/matrix.py:78-84).

It is pinned to the reference's own outputs by tests/test_cpu_baseline.py.
"""
from __future__ import annotations

import numpy as np
import torch
from torch.func import vmap

from . import fem


def _integrand(gradu, gradv, kappa):
    return kappa * (gradu @ gradv)


# in_dims per argument (gradu, gradv, kappa) at each vmap level, from the
# reference's broadcast table: gradu maps over (element, quadrature, u),
# gradv over (element, quadrature, v), element data over element only.
_PARALLEL = vmap(vmap(vmap(vmap(_integrand, in_dims=(None, 0, None)),
                           in_dims=(0, None, None)),
                      in_dims=(0, 0, None)),
                 in_dims=(0, 0, 0))


class ReferenceOps:
    """Set-up once per mesh (quadrature tables, slot map as torch tensors),
    then ``values(points, kappa)`` per call, as the reference splits
    ``from_mesh`` and ``__call__``."""

    def __init__(self, points: np.ndarray, elements: np.ndarray, element_type: str, quadrature_order: int):
        w, xi = fem.quadrature(element_type, quadrature_order)
        _, dN = fem.shape_functions(element_type, xi)           # [Q, D, B]
        self.w = torch.from_numpy(np.ascontiguousarray(w))
        self.dN = torch.from_numpy(np.ascontiguousarray(dN))
        self.elements = torch.from_numpy(np.ascontiguousarray(elements)).long()
        ip, ix, slots = fem.node_pattern(elements, points.shape[0])
        self.slots = torch.from_numpy(np.ascontiguousarray(slots)).reshape(-1).long()
        self.nnz = int(ix.shape[0])
        ip, ix = np.asarray(ip), np.asarray(ix)
        rows = np.repeat(np.arange(ip.shape[0] - 1), np.diff(ip))
        self.edges = torch.from_numpy(np.stack([rows, ix]).astype(np.int32))

    def values(self, points: torch.Tensor, kappa: torch.Tensor) -> torch.Tensor:
        ele_point_data = {"x": points[self.elements]}                    # noqa: F841 (unused, as in the reference)
        X = points[self.elements]                                        # [E, B, D]
        J = torch.einsum("ebj,qib->eqij", X, self.dN)
        Jinv = torch.inverse(J)
        grad = torch.einsum("qib,eqji->eqbj", self.dN, Jinv)             # [E, Q, B, D]
        jxw = torch.einsum("q,eq->eq", self.w, torch.linalg.det(J).abs())
        integral = _PARALLEL(grad, grad, kappa)                          # [E, Q, B, B]
        Ke = torch.einsum("eqij,eq->eij", integral, jxw)
        out = torch.zeros(self.nnz, dtype=Ke.dtype)
        out = out.index_add_(0, self.slots, Ke.reshape(-1))
        row, col = self.edges[0].long(), self.edges[1].long()            # noqa: F841
        return out


class ReferenceJacobiPCG:
    """The reference's iterative-solve operation sequence on the CPU: its CG
    loop (``cg_py``, sparse/solve/torch_solve.py:70-128: a torch CSR matrix,
    one torch call per SpMV, dot and axpy) with its Jacobi preconditioner
    applied the way ``jacobi_precond`` does it (torch_solve.py:24-59: the
    diagonal with missing entries taken as 1, z = r * (1 / diag)).  The
    reference's default ``K.solve`` backend (torch_sla) is not available, so
    this stands for its Jacobi-PCG; it times iterations, it does not decide
    convergence (the product's solver does that on the GPU)."""

    def __init__(self, indptr: np.ndarray, indices: np.ndarray, values: np.ndarray):
        n = indptr.shape[0] - 1
        self.A = torch.sparse_csr_tensor(torch.from_numpy(indptr.astype(np.int64)),
                                         torch.from_numpy(indices.astype(np.int64)),
                                         torch.from_numpy(values), size=(n, n))
        rows = np.repeat(np.arange(n), np.diff(indptr))
        diag = np.ones(n)
        on = rows == indices
        diag[rows[on]] = values[on]
        self.dinv = 1.0 / torch.from_numpy(diag)

    def iterate(self, b: torch.Tensor, iters: int) -> torch.Tensor:
        """``iters`` Jacobi-PCG iterations from x = 0; returns x."""
        A, dinv = self.A, self.dinv
        x = torch.zeros_like(b)
        r = b - A @ x
        z = r * dinv
        p = z.clone()
        rz = torch.dot(r, z)
        for _ in range(iters):
            Ap = A @ p
            alpha = rz / torch.dot(p, Ap)
            x = x + alpha * p
            r = r - alpha * Ap
            z = r * dinv
            rz_new = torch.dot(r, z)
            p = z + (rz_new / rz) * p
            rz = rz_new
        return x
