"""Parity of the CUDA facet (boundary) loads against the oracle and the
reference's own FacetAssembler outputs (golden fixtures).

Bars: with the default facet rule (the reference's float32-built rule),
float64 within 1e-12 relative (max-norm, relative to max|b|) of the
reference's own outputs and of the oracle handed the reference's table;
with ``facet_rule="exact"``, within 1e-12 of the oracle's exact float64 rule
(and 1e-6 of the reference, whose rule is rounded to float32); float32
within 1e-5; bitwise determinism run to run."""
import math

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem

pytestmark = pytest.mark.gpu
DEV = "cuda"
MESHES = ["triangle", "triangle6", "tetra", "tetra10", "triangle6c", "tetra10c"]


def ref_table(et, q):
    """The reference's float32 facet table (weights, points) of the family of
    ``et``, as stored in the facet fixture."""
    g = np.load(fem_fixture())
    fam = "triangle" if et.startswith("tri") else "tetra"
    return g[f"facet_table/{fam}/q{q}/w"], g[f"facet_table/{fam}/q{q}/p"]


def fem_fixture():
    import os
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_facet.npz")


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


class FacetOne(tg.FacetAssembler):
    def forward(self, v):
        return v


class FacetVector(tg.FacetAssembler):
    def forward(self, v):
        t = torch.tensor([0.5, -1.0] if v.shape[0] in (3, 6) else [0.0, 0.3, -1.0], dtype=v.dtype, device=v.device)
        return v[:, None] * t


class FacetFunc(tg.FacetAssembler):
    def forward(self, x, v):
        return (torch.sin(math.pi * x[0]) + x[1] ** 2) * v


class FacetPoint(tg.FacetAssembler):
    def forward(self, v, g):
        return g * v


def mesh_of(g, et, dtype=torch.float64):
    pts = torch.tensor(g[f"{et}/points"], dtype=dtype, device=DEV)
    el = torch.tensor(g[f"{et}/elements"], device=DEV)
    return tg.Mesh(points=pts, cells={et.rstrip("c"): el},
                   point_data={"is_boundary": torch.tensor(g[f"{et}/boundary"], device=DEV),
                               "is_top": torch.tensor(g[f"{et}/top"], device=DEV)})


def run_case(mesh, case, q, gfield, rule="reference"):
    def make(cls, **kw):
        asm = cls.from_mesh(mesh, quadrature_order=q, **kw)
        asm.facet_rule = rule
        return asm
    if case == "const":
        return make(FacetOne)(mesh.points)
    if case == "vector":
        return make(FacetVector)(mesh.points)
    if case == "func":
        return make(FacetFunc)(mesh.points)
    if case == "point":
        return make(FacetPoint)(mesh.points, point_data={"g": gfield})
    return make(FacetOne, boundary_mask="is_top")(mesh.points)


def oracle_case(g, et, case, q, rule="reference"):
    pts, el = g[f"{et}/points"], g[f"{et}/elements"]
    dim = pts.shape[1]
    bd, top = g[f"{et}/boundary"], g[f"{et}/top"]
    kind, val, mask = {
        "const": ("const", 1.0, bd),
        "vector": ("const", [0.5, -1.0] if dim == 2 else [0.0, 0.3, -1.0], bd),
        "func": ("func", lambda x: np.sin(math.pi * x[..., 0]) + x[..., 1] ** 2, bd),
        "point": ("point", g[f"{et}/facet_g"], bd),
        "top": ("const", 1.0, top),
    }[case]
    tables = ref_table(et, q) if rule == "reference" else None
    return fem.facet_load(pts, el, et.rstrip("c"), mask, q, kind, val, tables=tables)


@pytest.mark.parametrize("et", MESHES)
@pytest.mark.parametrize("q", [1, 2, 3, 4])
@pytest.mark.parametrize("case", ["const", "vector", "func", "point", "top"])
def test_facet_loads_match_oracle_and_reference(golden_facet, et, q, case):
    g = golden_facet
    mesh = mesh_of(g, et)
    gfield = torch.tensor(g[f"{et}/facet_g"], device=DEV)
    ref = g[f"{et}/facet_{case}/q{q}"]
    got = run_case(mesh, case, q, gfield).cpu().numpy()           # default: the reference's rule
    assert got.shape == ref.shape
    assert rel_err(got, ref) <= 1e-12
    assert rel_err(got, oracle_case(g, et, case, q)) <= 1e-12
    exact = run_case(mesh, case, q, gfield, rule="exact").cpu().numpy()
    assert rel_err(exact, oracle_case(g, et, case, q, rule="exact")) <= 1e-12
    assert rel_err(exact, ref) <= 1e-6


@pytest.mark.parametrize("et", MESHES)
@pytest.mark.parametrize("case", ["const", "vector", "func", "point"])
def test_facet_loads_fp32(golden_facet, et, case):
    g = golden_facet
    mesh = mesh_of(g, et, torch.float32)
    gfield = torch.tensor(g[f"{et}/facet_g"], device=DEV, dtype=torch.float32)
    got = run_case(mesh, case, 2, gfield)
    assert got.dtype == torch.float32
    assert rel_err(got.cpu().numpy(), oracle_case(g, et, case, 2)) <= 1e-5


@pytest.mark.parametrize("etype", ["triangle6", "tetra10"])
def test_facet_loads_larger_curved_mesh(etype):
    """More facets (several thread blocks) with curved P2 facets: every
    midpoint moved, against the oracle."""
    base = tg.Mesh.gen_unit_square(40) if etype == "triangle6" else tg.Mesh.gen_unit_cube(9)
    m = base.to_p2()
    nv = base.n_points
    gen = torch.Generator().manual_seed(3)
    pts = m.points.clone()
    pts[nv:] += 0.1 / 40 * (torch.rand(pts[nv:].shape, generator=gen, dtype=torch.float64) - 0.5)
    el = m.cells[etype]
    bd = m.boundary_mask
    gf = torch.cos(pts[:, 0]) * (1 + pts[:, -1])
    mesh = tg.Mesh(points=pts.to(DEV), cells={etype: el.to(DEV)}, point_data={"is_boundary": bd.to(DEV)})
    for q in (2, 3):
        got = FacetPoint.from_mesh(mesh, quadrature_order=q)(mesh.points, point_data={"g": gf.to(DEV)})
        ref = fem.facet_load(pts.numpy(), el.numpy(), etype, bd.numpy(), q, "point", gf.numpy(),
                             tables=ref_table(etype, q))
        assert rel_err(got.cpu().numpy(), ref) <= 1e-12


def test_facet_selection_and_total_measure():
    """The sum of the constant load is the measure of the selected facets:
    the unit cube's surface plus the interior faces whose nodes are all on
    the boundary, each counted from both sides."""
    mesh = tg.Mesh.gen_unit_cube(6, device=DEV)
    b = FacetOne.from_mesh(mesh, quadrature_order=1)(mesh.points)
    el = mesh.cells["tetra"].cpu().numpy()
    pts = mesh.points.cpu().numpy()
    bd = mesh.boundary_mask.cpu().numpy()
    e, f = fem.facet_select(el, "tetra", bd)
    fn = fem.facet_nodes("tetra")
    tri = pts[el[e][np.arange(len(e))[:, None], fn[f]]]
    area = 0.5 * np.linalg.norm(np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]), axis=1).sum()
    assert abs(float(b.sum()) - area) <= 1e-12 * area
    assert area >= 6.0 - 1e-12


def test_facet_loads_are_bitwise_deterministic():
    mesh = tg.Mesh.gen_unit_cube(10, device=DEV)
    asm = FacetFunc.from_mesh(mesh, quadrature_order=3)
    ref = asm(mesh.points).clone()
    for _ in range(4):
        assert torch.equal(asm(mesh.points), ref)


def test_facet_edge_cases():
    mesh = tg.Mesh.gen_unit_square(4, device=DEV)
    none = torch.zeros(mesh.n_points, dtype=torch.bool, device=DEV)
    z = FacetVector.from_mesh(mesh, boundary_mask=none)(mesh.points)
    assert z.shape == (2 * mesh.n_points,) and not bool(z.any())
    shared = FacetPoint.from_assembler(FacetOne.from_mesh(mesh))
    gf = torch.rand(mesh.n_points, dtype=torch.float64, device=DEV)
    assert torch.equal(shared(mesh.points, point_data={"g": gf}),
                       FacetPoint.from_mesh(mesh)(mesh.points, point_data={"g": gf}))

    class Square(tg.FacetAssembler):
        def forward(self, v):
            return v * v

    with pytest.raises(NotImplementedError):
        Square.from_mesh(mesh)(mesh.points)
    with pytest.raises(NotImplementedError):
        FacetOne.from_mesh(mesh, quadrature_order=5)
    with pytest.raises(NotImplementedError):
        FacetOne.from_mesh(mesh)(mesh.points.clone().requires_grad_(True))
    with pytest.raises(RuntimeError):
        FacetOne.from_mesh(mesh.to("cpu"))(mesh.points.cpu())


@pytest.mark.parametrize("et", ["triangle6c", "tetra10c"])
def test_facet_load_gradient_wrt_point_data(golden_facet, et):
    """dL/dg of L = w . b(g) is M w (M the symmetric facet mass matrix): the
    oracle's point load of w, scaled back per component for vector loads."""
    g = golden_facet
    mesh = mesh_of(g, et)
    pts, el, bd = g[f"{et}/points"], g[f"{et}/elements"], g[f"{et}/boundary"]
    dim = pts.shape[1]
    rng = np.random.default_rng(5)
    g0 = torch.tensor(g[f"{et}/facet_g"], device=DEV)

    field = g0.clone().requires_grad_(True)
    b = FacetPoint.from_mesh(mesh, quadrature_order=3)(mesh.points, point_data={"g": field})
    w = rng.normal(size=b.shape[0])
    (b * torch.tensor(w, device=DEV)).sum().backward()
    ref = fem.facet_load(pts, el, et.rstrip("c"), bd, 3, "point", w, tables=ref_table(et, 3))
    assert rel_err(field.grad.cpu().numpy(), ref) <= 1e-12

    t = [0.5, -1.0] if dim == 2 else [0.0, 0.3, -1.0]

    class PointTraction(tg.FacetAssembler):
        def forward(self, v, p):
            return p * v[:, None] * torch.tensor(t, dtype=v.dtype, device=v.device)

    field = g0.clone().requires_grad_(True)
    b = PointTraction.from_mesh(mesh, quadrature_order=2)(mesh.points, point_data={"p": field})
    assert rel_err(b.detach().cpu().numpy(),
                   fem.facet_load(pts, el, et.rstrip("c"), bd, 2, "point", g0.cpu().numpy()[:, None] * np.array(t),
                                  tables=ref_table(et, 2))) <= 1e-12
    W = rng.normal(size=(pts.shape[0], dim))
    (b * torch.tensor(W.reshape(-1), device=DEV)).sum().backward()
    ref = fem.facet_load(pts, el, et.rstrip("c"), bd, 2, "point", W @ np.array(t), tables=ref_table(et, 2))
    assert rel_err(field.grad.cpu().numpy(), ref) <= 1e-12
