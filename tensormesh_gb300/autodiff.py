"""Forward launches of the assembly kernels (and, where inputs require
gradients, the autograd wiring to the hand-written backward kernels)."""
from __future__ import annotations

import torch

from . import _lib
from . import element as E_
from .sparse import SparseMatrix
from .validate import check_finite

_FORM_CODE = {"laplace": _lib.TM_FORM_LAPLACE, "mass": _lib.TM_FORM_MASS, "elasticity": _lib.TM_FORM_ELASTICITY}


def _coefficient(form, points, element_data, point_data, scalar_data):
    """(coef_kind, coef tensor or None, scalar) for a bilinear form."""
    key = form.coef_key
    scale = float(form.scale)
    if key is None:
        return _lib.TM_COEF_SCALAR, None, scale
    if key in element_data:
        c = element_data[key].to(device=points.device, dtype=points.dtype).reshape(-1)
        return _lib.TM_COEF_ELEMENT, (c * scale if scale != 1.0 else c).contiguous(), 1.0
    if key in point_data:
        c = point_data[key].to(device=points.device, dtype=points.dtype).reshape(-1)
        return _lib.TM_COEF_POINT, (c * scale if scale != 1.0 else c).contiguous(), 1.0
    v = scalar_data[key]
    return _lib.TM_COEF_SCALAR, None, float(torch.as_tensor(v)) * scale


def assemble_matrix(asm, form, points, element_data, point_data, scalar_data) -> SparseMatrix:
    topo = asm.topology
    H = topo.dim if form.kind == "elasticity" else 1
    dptr, dind = topo.dof_pattern(H)
    kind, coef, scal = _coefficient(form, points, element_data, point_data, scalar_data)
    check_finite((("points", points), ("the coefficient", coef)))
    pts = points.detach().contiguous()
    out = torch.empty(dind.shape[0], dtype=points.dtype, device=points.device)
    from .adjoint import needs_grad, AssembleMatrixFn
    if needs_grad(points, coef):
        values = AssembleMatrixFn.apply(points, coef, asm, form, kind, scal)
    else:
        _tables = E_.kernel_tables  # noqa: F841  (keeps symbol referenced)
        from .assemble import launch_assemble
        launch_assemble(topo, _FORM_CODE[form.kind], pts, out, quadrature_order=asm.quadrature_order,
                        coef_kind=kind, coef=None if coef is None else coef.detach(), scal=(scal, 0.0, 0.0),
                        lame=(form.lam, form.mu), precision=asm.precision, slot_budget=asm.slot_budget)
        values = out
    n = topo.n_points * H
    return SparseMatrix(values, shape=(n, n), indptr=dptr, indices=dind)


def _load_coefficient(asm, form, points, point_data, scalar_data):
    topo = asm.topology
    if form.kind == "const":
        c = [float(x) for x in form.const.reshape(-1)]
        return _lib.TM_COEF_SCALAR, None, c, len(c)
    if form.kind == "scalar":
        v = float(torch.as_tensor(scalar_data[form.coef_key])) * float(form.const[0])
        return _lib.TM_COEF_SCALAR, None, [v], 1
    if form.kind == "point":
        f = point_data[form.coef_key].to(device=points.device, dtype=points.dtype)
        ratio = float(form.const[0]) if form.const is not None else 1.0
        if ratio != 1.0:
            f = f * ratio
        H = 1 if f.dim() == 1 else int(f.shape[1])
        return _lib.TM_COEF_POINT, f.reshape(-1).contiguous(), [0.0], H
    if form.kind == "func":
        Q = E_.n_quadrature(topo.element_type, asm.quadrature_order)
        if points.requires_grad and torch.is_grad_enabled():
            # differentiable interpolation so f(x_q) carries d/dX through torch
            _, Nq = E_.shape_values(topo.element_type, asm.quadrature_order)
            Nt = torch.as_tensor(Nq, dtype=points.dtype, device=points.device)
            xq = torch.einsum("ebd,qb->eqd", points[topo.elements.long()], Nt)
        else:
            xq = quadrature_points(topo, asm.quadrature_order, points.detach())
        flat = xq.reshape(-1, topo.dim)
        try:
            fq = torch.func.vmap(form.func)(flat)
        except Exception:
            fq = form.func(flat)
        fq = torch.as_tensor(fq).to(device=points.device, dtype=points.dtype)
        H = 1 if fq.dim() == 1 else int(fq.shape[1])
        assert fq.shape[0] == flat.shape[0], "f(x) must return one value (or one [H] vector) per point"
        return _lib.TM_COEF_QUAD, fq.reshape(-1).contiguous(), [0.0], H
    raise NotImplementedError(form.kind)


def quadrature_points(topo, order: int, points: torch.Tensor) -> torch.Tensor:
    Q = E_.n_quadrature(topo.element_type, order)
    tables = E_.kernel_tables(topo.element_type, order, points.device)
    out = torch.empty(topo.n_elements, Q, topo.dim, dtype=points.dtype, device=points.device)
    _lib.call("tm_quadrature_points", topo.el_id, _dtype(points), Q, tables.data_ptr(), points.contiguous().data_ptr(),
              topo.elements.data_ptr(), topo.n_elements, out.data_ptr(), _lib.stream_handle(points.device))
    return out


def _dtype(t):
    return _lib.TM_F64 if t.dtype == torch.float64 else _lib.TM_F32


def assemble_load(asm, form, points, point_data, scalar_data) -> torch.Tensor:
    topo = asm.topology
    kind, coef, scal, H = _load_coefficient(asm, form, points, point_data, scalar_data)
    check_finite((("points", points), ("the load coefficient", coef)))
    from .adjoint import needs_grad, AssembleLoadFn
    if needs_grad(points, coef):
        out = AssembleLoadFn.apply(points, coef, asm, kind, tuple(scal), H)
    else:
        from .assemble import launch_assemble
        out = torch.empty(topo.n_points * H, dtype=points.dtype, device=points.device)
        launch_assemble(topo, _lib.TM_FORM_LOAD, points.detach().contiguous(), out,
                        quadrature_order=asm.quadrature_order, coef_kind=kind,
                        coef=None if coef is None else coef.detach(), scal=tuple(scal), n_comp=H,
                        precision=asm.precision)
    return out
