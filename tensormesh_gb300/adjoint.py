"""Autograd for the assembly kernels: torch.autograd.Function wrappers whose
backward runs the hand-written adjoint assembly (``tm_assemble_backward``)
and the deterministic segmented reductions (``tm_segment_sum``).

Gradients are returned for the nodal coordinates and for the integrand's
coefficient (element data, point data or values at quadrature points), the
two inputs the reference differentiates through its autograd chain
(element/element.py:962-966 Jacobian/inverse,
element/transformation.py:1289 JxW, assemble/projector.py:125 scatter).
"""
from __future__ import annotations

import torch

from . import _lib
from . import element as E_

_FORM_CODE = {"laplace": _lib.TM_FORM_LAPLACE, "mass": _lib.TM_FORM_MASS, "elasticity": _lib.TM_FORM_ELASTICITY,
              "load": _lib.TM_FORM_LOAD}


def needs_grad(*ts) -> bool:
    return torch.is_grad_enabled() and any(t is not None and t.requires_grad for t in ts)


def _dt(t):
    return _lib.TM_F64 if t.dtype == torch.float64 else _lib.TM_F32


class BackwardMaps:
    """Fixed-order reduction maps of one patch plan: the (patch, element)
    pairs of each element, and the (pair, local node) entries of each node."""

    def __init__(self, topo, plan):
        dev = plan.elem.device
        E, N, B = topo.n_elements, topo.n_points, topo.n_basis
        pe = plan.elem.long()
        self.elem_perm = torch.argsort(pe, stable=True)
        self.elem_ptr = torch.zeros(E + 1, dtype=torch.int64, device=dev)
        self.elem_ptr[1:] = torch.cumsum(torch.bincount(pe, minlength=E), 0)
        node = topo.elements.long()[pe]                      # [n_pairs, B] global node of each entry
        flat = node.reshape(-1)
        self.node_perm = torch.argsort(flat, stable=True)
        self.node_ptr = torch.zeros(N + 1, dtype=torch.int64, device=dev)
        self.node_ptr[1:] = torch.cumsum(torch.bincount(flat, minlength=N), 0)
        self.n_pairs = int(pe.shape[0])


def backward_maps(topo, H: int = 1):
    """(BackwardMaps, plan struct) of the plan used for H x H block slots."""
    cache = topo.__dict__.setdefault("_bw_maps", {})
    if H not in cache:
        plan, struct = topo.plan_for(H)
        cache[H] = (BackwardMaps(topo, plan), struct)
    return cache[H]


def segment_sum(ptr, perm, src, width):
    n = ptr.shape[0] - 1
    out = torch.empty(n * width, dtype=src.dtype, device=src.device)
    _lib.call("tm_segment_sum", _dt(src), n, ptr.data_ptr(), perm.data_ptr(), width, src.data_ptr(), out.data_ptr(),
              _lib.stream_handle(src.device))
    return out


def _args(topo, form_code, points, quadrature_order, kind, coef, scal, lame, n_comp, precision="emulated"):
    from .assemble import PRECISION, _dtype_code
    tables = E_.kernel_tables(topo.element_type, quadrature_order, points.device)
    a = _lib.AssembleArgs()
    a.element, a.form, a.dtype = topo.el_id, form_code, _dtype_code(points.dtype)
    a.precision = PRECISION[precision]
    a.coef_kind, a.n_comp = kind, n_comp
    a.n_quad = E_.n_quadrature(topo.element_type, quadrature_order)
    a.tables, a.points = tables.data_ptr(), points.data_ptr()
    a.coef = 0 if coef is None else coef.data_ptr()
    for i in range(3):
        a.scal[i] = float(scal[i]) if i < len(scal) else 0.0
    a.lam, a.mu = float(lame[0]), float(lame[1])
    return a, tables


def run_backward(topo, form_code, points, quadrature_order, kind, coef, scal, lame, n_comp, grad_out,
                 want_points: bool, want_coef: bool):
    """Returns (grad_points [N, D] or None, grad_coef (coef's shape) or None)."""
    Hb = topo.dim if form_code == _lib.TM_FORM_ELASTICITY else 1
    maps, plan_struct = backward_maps(topo, Hb)
    P, B, D = maps.n_pairs, topo.n_basis, topo.dim
    Q = E_.n_quadrature(topo.element_type, quadrature_order)
    dev, dtype = points.device, points.dtype
    pts = points.detach().contiguous()
    c = None if coef is None else coef.detach().contiguous()
    a, _tables = _args(topo, form_code, pts, quadrature_order, kind, c, scal, lame, n_comp)
    bw = _lib.BackwardArgs()
    g = grad_out.detach().to(dtype).contiguous()
    bw.grad_out = g.data_ptr()
    pair_dX = torch.empty(P * B * D, dtype=dtype, device=dev) if want_points else None
    comp = n_comp if form_code == _lib.TM_FORM_LOAD else 1
    pair_dc = None
    if want_coef and kind != _lib.TM_COEF_SCALAR:
        size = {_lib.TM_COEF_ELEMENT: P, _lib.TM_COEF_POINT: P * B * comp, _lib.TM_COEF_QUAD: P * Q * comp}[kind]
        pair_dc = torch.empty(size, dtype=dtype, device=dev)
    bw.pair_dX = 0 if pair_dX is None else pair_dX.data_ptr()
    bw.pair_dcoef = 0 if pair_dc is None else pair_dc.data_ptr()
    _lib.call("tm_assemble_backward", plan_struct, a, bw, _lib.stream_handle(dev))
    gp = gc = None
    if pair_dX is not None:
        gp = segment_sum(maps.node_ptr, maps.node_perm, pair_dX, D).view(topo.n_points, D)
    if pair_dc is not None:
        if kind == _lib.TM_COEF_ELEMENT:
            gc = segment_sum(maps.elem_ptr, maps.elem_perm, pair_dc, 1)
        elif kind == _lib.TM_COEF_POINT:
            gc = segment_sum(maps.node_ptr, maps.node_perm, pair_dc, comp)
        else:
            gc = segment_sum(maps.elem_ptr, maps.elem_perm, pair_dc, Q * comp)
        gc = gc.view(coef.shape)
    return gp, gc


class AssembleMatrixFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, points, coef, asm, form, kind, scal):
        from .assemble import launch_assemble
        topo = asm.topology
        H = topo.dim if form.kind == "elasticity" else 1
        dptr, dind = topo.dof_pattern(H)
        out = torch.empty(dind.shape[0], dtype=points.dtype, device=points.device)
        launch_assemble(topo, _FORM_CODE[form.kind], points.detach().contiguous(), out,
                        quadrature_order=asm.quadrature_order, coef_kind=kind,
                        coef=None if coef is None else coef.detach().contiguous(), scal=(scal, 0.0, 0.0),
                        lame=(form.lam, form.mu), precision=asm.precision)
        ctx.save_for_backward(points, coef)
        ctx.meta = (asm, form, kind, scal)
        return out

    @staticmethod
    def backward(ctx, g):
        points, coef = ctx.saved_tensors
        asm, form, kind, scal = ctx.meta
        gp, gc = run_backward(asm.topology, _FORM_CODE[form.kind], points, asm.quadrature_order, kind, coef,
                              (scal, 0.0, 0.0), (form.lam, form.mu), 1, g,
                              ctx.needs_input_grad[0], ctx.needs_input_grad[1])
        return gp, gc, None, None, None, None


class AssembleLoadFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, points, coef, asm, kind, scal, H):
        from .assemble import launch_assemble
        topo = asm.topology
        out = torch.empty(topo.n_points * H, dtype=points.dtype, device=points.device)
        launch_assemble(topo, _lib.TM_FORM_LOAD, points.detach().contiguous(), out,
                        quadrature_order=asm.quadrature_order, coef_kind=kind,
                        coef=None if coef is None else coef.detach().contiguous(), scal=tuple(scal), n_comp=H,
                        precision=asm.precision)
        ctx.save_for_backward(points, coef)
        ctx.meta = (asm, kind, scal, H)
        return out

    @staticmethod
    def backward(ctx, g):
        points, coef = ctx.saved_tensors
        asm, kind, scal, H = ctx.meta
        gp, gc = run_backward(asm.topology, _lib.TM_FORM_LOAD, points, asm.quadrature_order, kind, coef, scal,
                              (0.0, 0.0), H, g, ctx.needs_input_grad[0], ctx.needs_input_grad[1])
        return gp, gc, None, None, None, None
