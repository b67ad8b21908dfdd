"""Boundary (facet) loads on the GPU: the reference's ``FacetAssembler``
(assemble/facet_assembler.py).

Interface parity: ``FacetAssembler.from_mesh(mesh, boundary_mask=None,
quadrature_order=2, project='reduce', *args, **kwargs)`` (:527-567; the mask
is ``mesh.boundary_mask``, a ``point_data`` key or a bool tensor),
``from_elements`` (:412-525), ``from_assembler`` (:382-410), the
``__post_init__`` hook, and ``__call__(points=None, func=None,
point_data=None) -> Tensor[N*H]`` (:130-235).  ``forward`` is written per
facet quadrature point with the basis dimension kept: ``v`` is the cell's
shape values ``[B]``, ``x`` the physical point ``[D]``, a ``point_data`` key
its interpolated value.

Selection follows the reference: a facet is integrated when every one of its
nodes is flagged (facet_assembler.py:491-508), so an interior facet whose
nodes all lie on the boundary is integrated from both of its elements, and
the contributions go to all of the cell's nodes (those off the facet get the
basis values there, zero up to rounding).

The GPU path covers integrands that are a coefficient times ``v``: a
constant (scalar or vector), a function of ``x``, or a ``point_data`` field
(with a constant factor).  One kernel (``tm_facet_load``) integrates every
selected facet with the facet rule's tables in float64; a fixed-order segment sum
reduces the per-(facet, node) values to the nodes, so the result is bitwise
reproducible.  The reference builds its facet rule in float32
(element/transformation.py:519-531 keeps get_facet_quadrature's float32
default), so its float64 facet loads carry float32 rounding of the points
and weights (about 3e-7 relative against the exact rule).  The default
``facet_rule="reference"`` uses that same float32 rule, so the loads agree
with the reference's to rounding; ``facet_rule="exact"`` integrates with the
float64 rule.
Gradients flow to the ``point_data`` field of a point-data integrand (the load is
linear in it with a symmetric facet mass matrix); gradients with respect to
the points are not provided.
"""
from __future__ import annotations

import ctypes
import functools
import inspect
from dataclasses import dataclass
from typing import Callable, Dict, Optional

import numpy as np
import torch
import torch.nn as nn

from . import _lib
from . import element as E_
from .assemble import _dtype_code, _mesh_single_type, _require_cuda

# Facet f of a simplex is the facet opposite vertex f (Triangle.edge,
# Tetrahedron.face in element/element.py); P2 facets add the midpoints of the
# edges between those vertices (element_to_facet, element.py:1411-1440).
FACET_VERTICES = {2: ((1, 2), (0, 2), (0, 1)), 3: ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2))}
MAX_COMPONENTS = 3


def facet_nodes(element_type: str) -> np.ndarray:
    """Local node ids of each facet [F, nodes per facet]."""
    _, dim, _, order = E_.element_info(element_type)
    edges = E_.TRI_EDGES if dim == 2 else E_.TET_EDGES
    out = []
    for vs in FACET_VERTICES[dim]:
        nodes = list(vs)
        if order == 2:
            nodes += [dim + 1 + k for k, (i, j) in enumerate(edges) if i in vs and j in vs]
        out.append(nodes)
    return np.array(out, dtype=np.int64)


def facet_rule(dim: int, order: int):
    """Facet-local rule (weights [Qf], points [Qf, D-1]): ``order``-point
    Gauss-Legendre on [0, 1] for edges (element/quadrature.py:9-66), the
    triangle rule of that order for faces (quadrature.py:68-116)."""
    if not 1 <= order <= E_.MAX_QUADRATURE_ORDER:
        raise NotImplementedError(f"facet quadrature order {order} (supported 1..{E_.MAX_QUADRATURE_ORDER})")
    if dim == 2:
        x, w = np.polynomial.legendre.leggauss(order)
        return 0.5 * w, (0.5 * (x + 1.0))[:, None]
    return E_.quadrature("triangle", order)


FACET_RULES = ("reference", "exact")


@functools.lru_cache(maxsize=None)
def facet_tables(element_type: str, order: int, rule: str = "reference"):
    """(w [F, Qf], N [F, Qf, B], Tc [F, Qf, D-1, B], xi [F, Qf, D]) in float64.

    ``rule="reference"`` (the default) reproduces the reference's facet rule,
    which it builds in float32 (transformation.py:519-531 keeps
    get_facet_quadrature's float32 default): the weights are the float32
    roundings of the exact weights, and the points (where the shape values
    N are evaluated) are the reference's own float32 points
    (``facet_reference_points``).  The facet tangents Tc stay exact, as in the
    reference's facet Jacobian.  ``rule="exact"`` keeps the float64 rule.

    Facet f is the affine image r -> P_a + sum_k r_k (P_{v_k} - P_a) of the
    reference segment / triangle (P the reference simplex's vertices, (a, v_1,
    ...) the facet's vertices in order; element.py:993-1066
    get_local_facet_mapping_fns), xi its quadrature points in cell
    coordinates.  Tc[f][q][k][b] = grad N_b(xi_fq) . (P_{v_k} - P_a), so the
    physical facet tangents are t_k = sum_b Tc[..][k][b] X_b and the facet
    measure |F| = sqrt(det(t t^T)) (transformation.py:993-1003 detF)."""
    if rule not in FACET_RULES:
        raise ValueError(f"facet_rule should be one of {FACET_RULES}, but got {rule!r}")
    _, dim, _, _ = E_.element_info(element_type)
    P = np.concatenate([np.zeros((1, dim)), np.eye(dim)], 0)
    w, r = facet_rule(dim, order)
    if rule == "reference":
        from .facet_reference_points import POINTS
        w = w.astype(np.float32).astype(np.float64)
        ref_pts = np.array(POINTS[("triangle" if dim == 2 else "tetra", order)], dtype=np.float64)
    W, NN, TT, XI = [], [], [], []
    for f, vs in enumerate(FACET_VERTICES[dim]):
        T = np.stack([P[v] - P[vs[0]] for v in vs[1:]], 0)           # [D-1, D]
        xi = P[vs[0]][None, :] + r @ T                                 # [Qf, D]
        _, dN = E_.shape_tables(element_type, xi)                      # [Qf, B, D]
        xi_n = ref_pts[f] if rule == "reference" else xi
        N, _ = E_.shape_tables(element_type, xi_n)                     # [Qf, B]
        W.append(w)
        NN.append(N)
        TT.append(np.einsum("ki,qbi->qkb", T, dN))
        XI.append(xi_n)
    return np.stack(W), np.stack(NN), np.stack(TT), np.stack(XI)


_DEVICE_TABLES: Dict[tuple, torch.Tensor] = {}


def facet_kernel_tables(element_type: str, order: int, device, rule: str = "reference") -> torch.Tensor:
    """Flat float64 [w, N, Tc] as tm_facet_load reads it (cached per device)."""
    key = (element_type, order, str(torch.device(device)), rule)
    t = _DEVICE_TABLES.get(key)
    if t is None:
        w, N, Tc, _ = facet_tables(element_type, order, rule)
        flat = np.concatenate([w.ravel(), N.ravel(), Tc.ravel()])
        t = _DEVICE_TABLES[key] = torch.from_numpy(flat).to(device=device, dtype=torch.float64)
    return t


def select_facets(elements: torch.Tensor, element_type: str, boundary_mask: torch.Tensor) -> torch.Tensor:
    """Codes e * F + f of the facets whose nodes are all flagged, element-major
    (the reference's ``mask[facets].all(-1)`` then ``nonzero``)."""
    fn = facet_nodes(element_type)
    flagged = boundary_mask.to(device=elements.device, dtype=torch.bool)[elements.long()]   # [E, B]
    cols = [flagged[:, list(nodes)].all(-1) for nodes in fn]
    return torch.nonzero(torch.stack(cols, 1).reshape(-1)).reshape(-1)


class FacetTopology:
    """Selected facets of one connectivity and boundary mask, with the
    grouping of their (facet, cell node) pairs by node for the reduction."""

    def __init__(self, elements: torch.Tensor, n_points: int, element_type: str, boundary_mask: torch.Tensor):
        self.element_type = element_type
        self.el_id, self.dim, self.n_basis, _ = E_.element_info(element_type)
        self.n_facets = len(FACET_VERTICES[self.dim])
        self.elements = elements.to(torch.int32).contiguous()
        self.n_points = int(n_points)
        self.n_elements = int(elements.shape[0])
        self.sel = select_facets(elements, element_type, boundary_mask).contiguous()
        self.n_sel = int(self.sel.shape[0])
        nodes = elements.long()[torch.div(self.sel, self.n_facets, rounding_mode="floor")].reshape(-1)
        self.perm = torch.argsort(nodes, stable=True)
        self.ptr = torch.zeros(self.n_points + 1, dtype=torch.int64, device=elements.device)
        self.ptr[1:] = torch.cumsum(torch.bincount(nodes, minlength=self.n_points), 0)

    def to(self, device) -> "FacetTopology":
        """This topology with its index arrays on ``device`` (copied once)."""
        device = torch.device(device)
        if self.elements.device == device:
            return self
        copies = self.__dict__.setdefault("_copies", {})
        t = copies.get(str(device))
        if t is None:
            t = object.__new__(FacetTopology)
            t.__dict__.update({k: v for k, v in self.__dict__.items() if k != "_copies"})
            for k in ("elements", "sel", "perm", "ptr"):
                setattr(t, k, getattr(self, k).to(device))
            copies[str(device)] = t
        return t


@dataclass
class FacetForm:
    kind: str                               # "const" | "func" | "point"
    n_comp: int = 1
    const: Optional[torch.Tensor] = None    # [H] for "const"
    func: Optional[Callable] = None         # x [M, D] -> [M, H] for "func"
    coef_key: Optional[str] = None          # point_data key for "point"
    scale: Optional[torch.Tensor] = None    # [H] factor on the field for "point"


def _row_factor(o, r: torch.Tensor) -> Optional[torch.Tensor]:
    """c [H] when o == r (x) c (o [B] or [B, H]), else None."""
    o = torch.as_tensor(o, dtype=torch.float64)
    B = r.shape[0]
    if o.dim() == 1 and o.shape[0] == B:
        o = o[:, None]
    if o.dim() != 2 or o.shape[0] != B:
        return None
    c = o[0] / r[0]
    if not torch.allclose(o, r[:, None] * c[None, :], rtol=1e-12, atol=1e-12 * float(c.abs().max() + 1)):
        return None
    return c


def recognise_facet(fn, n_basis: int, dim: int, point_shapes: Dict[str, tuple]) -> FacetForm:
    params = list(inspect.signature(fn).parameters)
    if "v" not in params:
        raise NotImplementedError(f"forward{tuple(params)}: a facet load must take v")
    others = [p for p in params if p != "v"]
    gen = torch.Generator().manual_seed(4321)
    r = torch.rand(n_basis, generator=gen, dtype=torch.float64) + 0.5

    def call(vv, **kw):
        with torch.no_grad():
            return fn(*[vv if p == "v" else kw[p] for p in params])

    if not others:
        c = _row_factor(call(r), r)
        c2 = _row_factor(call(2.5 * r), r)
        if c is not None and c2 is not None and torch.allclose(c2, 2.5 * c, rtol=1e-12, atol=0):
            return FacetForm("const", n_comp=int(c.numel()), const=c)
    elif others == ["x"]:
        x = torch.rand(dim, generator=gen, dtype=torch.float64)
        c = _row_factor(call(r, x=x), r)
        c2 = _row_factor(call(2.5 * r, x=x), r)
        if c is not None and c2 is not None and torch.allclose(c2, 2.5 * c, rtol=1e-12, atol=1e-300):
            def g(xq, _call=call, _B=n_basis):
                ones = torch.ones(_B, dtype=xq.dtype, device=xq.device)
                return torch.func.vmap(lambda xx: torch.as_tensor(_call(ones, x=xx)).reshape(_B, -1)[0])(xq)
            return FacetForm("func", n_comp=int(c.numel()), func=g)
    elif len(others) == 1 and others[0] in point_shapes:
        key = others[0]
        shape = point_shapes[key]
        g1 = torch.rand(shape, generator=gen, dtype=torch.float64) + 0.5
        g2 = torch.rand(shape, generator=gen, dtype=torch.float64) + 0.5
        c1 = _row_factor(call(r, **{key: g1}), r)
        c2 = _row_factor(call(r, **{key: g2}), r)
        c3 = _row_factor(call(2.5 * r, **{key: 2.0 * g1}), r)
        if c1 is not None and c2 is not None and c3 is not None:
            if g1.numel() == 1:
                a = c1 / g1.reshape(())
                ok = torch.allclose(c2, a * g2.reshape(()), rtol=1e-12, atol=0)
            elif g1.numel() == c1.numel():
                a = c1 / g1.reshape(-1)
                ok = torch.allclose(c2, a * g2.reshape(-1), rtol=1e-12, atol=0)
            else:
                ok = False
            if ok and torch.allclose(c3, 5.0 * c1, rtol=1e-12, atol=0):
                return FacetForm("point", n_comp=int(c1.numel()), coef_key=key, scale=a)
    raise NotImplementedError(f"forward{tuple(params)} is not one of the facet integrands built for the GPU path "
                              "(a constant, f(x) or a point_data field, times v)")


class FacetAssembler(nn.Module):
    """Assemble a facet (boundary) integrand into a node vector on the GPU.

    ``facet_rule`` (class attribute, settable per instance): "reference"
    (default) integrates with the reference's float32-built facet rule, so the
    loads match the reference's to rounding; "exact" uses the float64 rule."""

    facet_rule = "reference"

    def __init__(self, topology: FacetTopology, points: torch.Tensor, quadrature_order: int, *args, **kwargs):
        super().__init__()
        facet_rule(topology.dim, int(quadrature_order))   # validates the order
        self.topology = topology
        self.quadrature_order = int(quadrature_order)
        self.register_buffer("points", points, persistent=False)
        self.element_types = [topology.element_type]
        self.dimension = topology.dim
        self.n_points = topology.n_points
        self._form_cache = {}
        self.__post_init__(*args, **kwargs)

    def __post_init__(self, *args, **kwargs):
        pass

    def forward(self, *args):
        raise NotImplementedError("forward is not implemented")

    @property
    def device(self) -> torch.device:
        return self.points.device

    @property
    def dtype(self) -> torch.dtype:
        return self.points.dtype

    @classmethod
    def from_assembler(cls, obj, *args, **kwargs):
        assert isinstance(obj, FacetAssembler), f"the object {obj} should inherit from FacetAssembler"
        return cls(obj.topology, obj.points, obj.quadrature_order, *args, **kwargs)

    @classmethod
    def from_elements(cls, points: torch.Tensor, elements: Dict[str, torch.Tensor], boundary_mask: torch.Tensor,
                      quadrature_order: int = 2, device="cpu", dtype=torch.float32, project: str = "reduce",
                      *args, **kwargs):
        if project not in ("reduce", "sparse"):
            raise ValueError(f"project should be either 'reduce' or 'sparse', but got {project}")
        if len(elements) != 1:
            raise NotImplementedError("mixed element types are not on the GPU path")
        (etype, el), = elements.items()
        points = points.to(device=device, dtype=dtype)
        topo = FacetTopology(el.to(points.device), points.shape[0], etype, boundary_mask.to(points.device))
        return cls(topo, points, quadrature_order, *args, **kwargs)

    @classmethod
    def from_mesh(cls, mesh, boundary_mask=None, quadrature_order: int = 2, project: str = "reduce", *args,
                  **kwargs):
        points = mesh.points
        etype, elements = _mesh_single_type(mesh)
        if boundary_mask is None:
            boundary_mask = mesh.boundary_mask
        elif isinstance(boundary_mask, str):
            boundary_mask = mesh.point_data[boundary_mask]
        assert boundary_mask.dim() == 1 and boundary_mask.shape[0] == points.shape[0]
        return cls.from_elements(points, {etype: elements}, boundary_mask, quadrature_order, points.device,
                                 points.dtype, project, *args, **kwargs)

    def _resolve_form(self, fn, point_data) -> FacetForm:
        shapes = {k: tuple(v.shape[1:]) for k, v in point_data.items()}
        key = (fn.__func__ if hasattr(fn, "__func__") else fn, tuple(sorted(shapes.items())))
        if key not in self._form_cache:
            self._form_cache[key] = recognise_facet(fn, self.topology.n_basis, self.dimension, shapes)
        return self._form_cache[key]

    def __call__(self, points: Optional[torch.Tensor] = None, func: Optional[Callable] = None,
                 point_data: Optional[Dict[str, torch.Tensor]] = None) -> torch.Tensor:
        point_data = dict(point_data or {})
        pts = self.points if points is None else points
        for k, v in point_data.items():
            assert v.shape[0] == self.n_points, f"the shape of {k} should be [n_point, ...], but got {v.shape}"
        _require_cuda(pts, "points")
        if pts.requires_grad:
            raise NotImplementedError("gradients of facet loads with respect to the points are not provided")
        form = self._resolve_form(self.forward if func is None else func, point_data)
        if form.kind == "point" and point_data[form.coef_key].requires_grad:
            return _FacetPointLoad.apply(point_data[form.coef_key], self, form, pts)
        if any(v.requires_grad for v in point_data.values()):
            raise NotImplementedError("gradients through facet loads are provided for the point_data field "
                                      "of a point-data integrand only")
        return facet_load(self, form, pts, point_data)


class _FacetPointLoad(torch.autograd.Function):
    """b = (M g) scaled per component, M_ij = sum over selected facets and
    facet points of w |F| N_i N_j (symmetric), so dL/dg = M (dL/db scaled
    back): the same kernel run on the incoming gradient."""

    @staticmethod
    def forward(ctx, g, asm, form, pts):
        ctx.asm, ctx.form, ctx.pts = asm, form, pts
        ctx.g_shape = g.shape
        return facet_load(asm, form, pts, {form.coef_key: g.detach()})

    @staticmethod
    def backward(ctx, gb):
        form, N = ctx.form, ctx.asm.n_points
        H = form.n_comp
        gb = gb.reshape(N, H)
        a = form.scale.to(device=gb.device, dtype=gb.dtype)
        if len(ctx.g_shape) == 1:
            # scalar field times the factor vector a: dL/dg = M (gb . a)
            back = FacetForm("point", n_comp=1, coef_key=form.coef_key, scale=torch.ones(1, dtype=torch.float64))
            grad = facet_load(ctx.asm, back, ctx.pts, {form.coef_key: (gb @ a).contiguous()})
        else:
            grad = facet_load(ctx.asm, form, ctx.pts, {form.coef_key: gb.contiguous()})
        return grad.reshape(ctx.g_shape), None, None, None


def facet_load(asm: FacetAssembler, form: FacetForm, pts: torch.Tensor, point_data) -> torch.Tensor:
    topo = asm.topology.to(pts.device)
    dev, dtype = pts.device, pts.dtype
    H, B, D, S = form.n_comp, topo.n_basis, topo.dim, topo.n_sel
    if H > MAX_COMPONENTS:
        raise NotImplementedError(f"facet loads with {H} components (at most {MAX_COMPONENTS})")
    if S == 0:
        return torch.zeros(topo.n_points * H, dtype=dtype, device=dev)
    pts = pts.detach().contiguous()
    tables = facet_kernel_tables(topo.element_type, asm.quadrature_order, dev, asm.facet_rule)
    Qf = int(facet_tables(topo.element_type, asm.quadrature_order, asm.facet_rule)[0].shape[1])
    stream = _lib.stream_handle(dev)
    code = _dtype_code(dtype)
    scal, coef = None, None
    if form.kind == "const":
        kind = _lib.TM_COEF_SCALAR
        scal = (ctypes.c_double * H)(*[float(c) for c in form.const.reshape(-1)])
    elif form.kind == "point":
        kind = _lib.TM_COEF_POINT
        field = point_data[form.coef_key].detach().to(device=dev, dtype=dtype).reshape(topo.n_points, -1)
        coef = (field * form.scale.to(device=dev, dtype=dtype)[None, :]).contiguous()
    else:
        kind = _lib.TM_COEF_QUAD
        xq = torch.empty(S * Qf * D, dtype=dtype, device=dev)
        _lib.call("tm_facet_load", topo.el_id, code, Qf, tables.data_ptr(), pts.data_ptr(), topo.elements.data_ptr(),
                  topo.sel.data_ptr(), S, kind, 0, None, H, 0, xq.data_ptr(), stream)
        coef = torch.as_tensor(form.func(xq.view(S * Qf, D))).to(dtype).reshape(S * Qf, -1).contiguous()
        if coef.shape[1] != H:
            raise AssertionError(f"the integrand returned {coef.shape[1]} components, expected {H}")
    contrib = torch.empty(S * B * H, dtype=dtype, device=dev)
    _lib.call("tm_facet_load", topo.el_id, code, Qf, tables.data_ptr(), pts.data_ptr(), topo.elements.data_ptr(),
              topo.sel.data_ptr(), S, kind, _lib.ptr(coef), scal, H, contrib.data_ptr(), 0, stream)
    from .adjoint import segment_sum
    return segment_sum(topo.ptr, topo.perm, contrib, H)
