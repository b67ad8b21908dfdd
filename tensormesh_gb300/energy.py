"""Energy assembly: the reference's ``ElementAssembler.energy`` for the
Neo-Hookean hyperelastic density (``NeoHookeanModel``,
assemble/builtin.py:220-334; element_assembler.py:468-680).

The quadrature loop and the density run in one kernel (``tm_neohookean``):
per element the energy and the gradient with respect to the element's nodal
displacements.  The total is a deterministic sum of the per-element energies;
the gradient (what ``energy.backward()`` puts in ``u.grad``: the internal
force vector) is reduced to the nodes by a segment sum in element order.
Gradients with respect to the points (shape derivatives) are not provided.
"""
from __future__ import annotations

from typing import Optional

import torch

from . import _lib
from . import element as E_
from .assemble import ElementAssembler, _dtype_code


def _node_maps(topo):
    """(ptr [N+1], perm) grouping the (element, local node) pairs by node, in
    element order inside each node."""
    maps = topo.__dict__.get("_energy_node_maps")
    if maps is None:
        node = topo.elements.long().reshape(-1)
        perm = torch.argsort(node, stable=True)
        ptr = torch.zeros(topo.n_points + 1, dtype=torch.int64, device=node.device)
        ptr[1:] = torch.cumsum(torch.bincount(node, minlength=topo.n_points), 0)
        maps = topo.__dict__["_energy_node_maps"] = (ptr, perm)
    return maps


class _NeoHookeanEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, points, asm, mu, lam):
        from .adjoint import segment_sum
        topo = asm.topology
        dev = points.device
        n_el, B, D = topo.n_elements, topo.n_basis, topo.dim
        tables = E_.kernel_tables(topo.element_type, asm.quadrature_order, dev)
        Q = E_.n_quadrature(topo.element_type, asm.quadrature_order)
        uu = u.detach().to(points.dtype).contiguous()
        e_el = torch.empty(n_el, dtype=torch.float64, device=dev)
        want = ctx.needs_input_grad[0]
        g_el = torch.empty(n_el * B * D, dtype=points.dtype, device=dev) if want else None
        _lib.call("tm_neohookean", topo.el_id, _dtype_code(points.dtype), Q, tables.data_ptr(),
                  points.data_ptr(), topo.elements.data_ptr(), n_el, uu.data_ptr(), float(mu), float(lam),
                  e_el.data_ptr(), 0 if g_el is None else g_el.data_ptr(), _lib.stream_handle(dev))
        if want:
            ptr, perm = _node_maps(topo)
            ctx.save_for_backward(segment_sum(ptr, perm, g_el, D).view(topo.n_points, D))
        ctx.keep = tables
        return e_el.sum().to(points.dtype)

    @staticmethod
    def backward(ctx, g):
        (gn,) = ctx.saved_tensors
        return (g * gn).to(gn.dtype), None, None, None, None


def neo_hookean_energy(asm: ElementAssembler, u: torch.Tensor, points: Optional[torch.Tensor], mu: float,
                       lam: float) -> torch.Tensor:
    topo = asm.topology
    pts = asm.points if points is None else points
    if not pts.is_cuda:
        raise RuntimeError("energy assembly runs on CUDA only")
    if pts.requires_grad:
        raise NotImplementedError("the energy's gradient with respect to the points is not provided; "
                                  "pass detached points")
    assert u.shape[0] == topo.n_points, f"the shape of displacement should be [n_point, ...], but got {u.shape}"
    assert u.dim() == 2 and u.shape[1] == topo.dim, f"displacement must be [n_point, {topo.dim}], got {u.shape}"
    return _NeoHookeanEnergy.apply(u, pts.detach().contiguous(), asm, mu, lam)


class NeoHookeanModel(ElementAssembler):
    r"""Neo-Hookean hyperelastic model (assemble/builtin.py:220-334):
    psi = mu/2 (I1 - d) - mu ln J + lam/2 (ln J)^2 with F = I + grad u,
    mu = E / (2 (1 + nu)), lam = E nu / ((1 + nu)(1 - 2 nu))."""

    def __post_init__(self, E=1.0, nu=0.3):
        self.mu = E / (2 * (1 + nu))
        self.lam = E * nu / ((1 + nu) * (1 - 2 * nu))

    def element_energy(self, graddisplacement):
        """The density at one quadrature point (the same formula the kernel
        evaluates; kept for callers that evaluate it directly)."""
        dim = graddisplacement.shape[-1]
        F = torch.eye(dim, device=graddisplacement.device, dtype=graddisplacement.dtype) + graddisplacement
        log_J = torch.log(torch.linalg.det(F))
        I1 = (F * F).sum()
        return (self.mu / 2) * (I1 - dim) - self.mu * log_J + (self.lam / 2) * (log_J ** 2)

    def energy(self, u, points: Optional[torch.Tensor] = None):
        """Total strain energy for the displacement u [n_points, dim]."""
        return super().energy(points=points, point_data={"displacement": u})
