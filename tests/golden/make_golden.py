"""Generate the golden fixtures in this folder by running the reference
TensorMesh package itself (CPU, float64).

Run from the repository root with the reference source tree on the machine:

    python tests/golden/make_golden.py /path/to/TensorMesh

The reference needs two packages that are not installed here (``meshio`` and
``torch_sla``); ``tests/golden/_stubs`` provides the minimal containers the
reference touches on this path (no numerics).  The fixtures written are small
``.npz`` files: every array in them is an input this script built or an
output of the reference's own ``ElementAssembler`` / ``NodeAssembler`` /
``FacetAssembler`` / ``Condenser`` / ``SparseSolveScipy`` calls.  Tests read only the ``.npz``
files, never the reference.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def square_mesh(n, jitter=0.0, seed=0):
    """Unit square, n x n cells, nodes x-fastest, cell (i,j) with corners
    a=(i,j) b=(i+1,j) c=(i+1,j+1) d=(i,j+1) split into (a,b,c), (a,c,d)."""
    xs = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    pts = np.stack([X.ravel(), Y.ravel()], 1)
    bd = (np.isclose(pts[:, 0], 0) | np.isclose(pts[:, 0], 1) | np.isclose(pts[:, 1], 0) | np.isclose(pts[:, 1], 1))
    if jitter:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, pts.shape) / n
        d[bd] = 0.0
        pts = pts + d
    idx = lambda i, j: j * (n + 1) + i  # noqa: E731
    tris = []
    for j in range(n):
        for i in range(n):
            a, b, c, d_ = idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)
            tris += [(a, b, c), (a, c, d_)]
    return pts, np.array(tris, dtype=np.int64), bd


_KUHN = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def cube_mesh(n, jitter=0.0, seed=0):
    """Unit cube, n^3 cells, nodes x-fastest then y then z; each cell split
    into the 6 Kuhn tetrahedra sharing the diagonal v000 -> v111, one per
    axis permutation in lexicographic order."""
    xs = np.linspace(0.0, 1.0, n + 1)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    bd = np.zeros(len(pts), dtype=bool)
    for k in range(3):
        bd |= np.isclose(pts[:, k], 0) | np.isclose(pts[:, k], 1)
    if jitter:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, pts.shape) / n
        d[bd] = 0.0
        pts = pts + d
    idx = lambda i, j, k: (k * (n + 1) + j) * (n + 1) + i  # noqa: E731
    tets = []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                for perm in _KUHN:
                    v = [i, j, k]
                    path = [idx(*v)]
                    for ax in perm:
                        v[ax] += 1
                        path.append(idx(*v))
                    tets.append(tuple(path))
    return pts, np.array(tets, dtype=np.int64), bd


_TRI_EDGES = [(1, 2), (0, 2), (0, 1)]
_TET_EDGES = [(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)]


def to_p2(pts, cells, bd):
    """Insert edge midpoints: unique edges sorted by (min, max) are numbered
    after the vertices; each element lists its midpoints in the reference
    element's edge order."""
    dim = pts.shape[1]
    loc = _TRI_EDGES if dim == 2 else _TET_EDGES
    pairs = np.stack([np.sort(cells[:, [a, b]], axis=1) for a, b in loc], 1)  # [E, ne, 2]
    flat = pairs.reshape(-1, 2)
    key = flat[:, 0] * len(pts) + flat[:, 1]
    uniq, inv = np.unique(key, return_inverse=True)
    u0, u1 = uniq // len(pts), uniq % len(pts)
    mid = 0.5 * (pts[u0] + pts[u1])
    new_pts = np.concatenate([pts, mid], 0)
    new_cells = np.concatenate([cells, len(pts) + inv.reshape(cells.shape[0], len(loc))], 1)
    new_bd = np.concatenate([bd, bd[u0] & bd[u1]])
    return new_pts, new_cells, new_bd


def main(ref_root):
    sys.path.insert(0, os.path.join(HERE, "_stubs"))
    sys.path.insert(0, ref_root)
    import torch
    import meshio
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    import tensormesh as tm
    from tensormesh.functional.elasticity import voigt_shape_grad, voigt_stiffness
    from tensormesh.sparse.solve.scipy_solve import SparseSolveScipy
    from tensormesh.assemble import NeoHookeanModel

    torch.set_num_threads(max(1, os.cpu_count() or 1))

    def mk_mesh(pts, cells, bd, etype):
        p3 = pts if pts.shape[1] == 3 else np.concatenate([pts, np.zeros((len(pts), 1))], 1)
        m = meshio.Mesh(p3, [(etype, cells)], point_data={"is_boundary": bd})
        return tm.Mesh(m)

    def canon(Kmat):
        c = Kmat.to_scipy_coo().tocsr()
        c.sum_duplicates()
        c.sort_indices()
        return c.indptr.astype(np.int64), c.indices.astype(np.int64), c.data.astype(np.float64)

    class KappaLaplace(tm.ElementAssembler):
        def forward(self, gradu, gradv, kappa):
            return kappa * (gradu @ gradv)

    class KappaMass(tm.ElementAssembler):
        def forward(self, u, v, kappa):
            return kappa * u * v

    NU = 0.3

    class EElasticity(tm.ElementAssembler):
        def forward(self, gradu, gradv, E):
            Ba = voigt_shape_grad(gradu)
            Bb = voigt_shape_grad(gradv)
            C = voigt_stiffness(1.0, NU, gradu.shape[0]).to(dtype=gradu.dtype)
            return E * (Ba.T @ C @ Bb)

    out = {}
    # ------------------------------------------------------------------ forms
    meshes = {
        "triangle": square_mesh(4, jitter=0.25, seed=1),
        "tetra": cube_mesh(2, jitter=0.2, seed=2),
    }
    meshes["triangle6"] = to_p2(*meshes["triangle"])
    meshes["tetra10"] = to_p2(*meshes["tetra"])
    rng = np.random.default_rng(7)
    for etype, (pts, cells, bd) in meshes.items():
        mesh = mk_mesh(pts, cells, bd, etype)
        n_el = cells.shape[0]
        coef = np.exp(rng.normal(size=n_el))
        out[f"{etype}/points"] = pts
        out[f"{etype}/elements"] = cells
        out[f"{etype}/boundary"] = bd
        out[f"{etype}/coef"] = coef
        for q in (1, 2, 3):
            cases = {
                "laplace": lambda: tm.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=q)(mesh.points),
                "mass": lambda: tm.MassElementAssembler.from_mesh(mesh, quadrature_order=q)(mesh.points),
                "elasticity": lambda: tm.LinearElasticityElementAssembler.from_mesh(
                    mesh, quadrature_order=q, E=2.5, nu=NU)(mesh.points),
                "laplace_kappa": lambda: KappaLaplace.from_mesh(mesh, quadrature_order=q)(
                    mesh.points, element_data={"kappa": torch.from_numpy(coef)}),
                "mass_kappa": lambda: KappaMass.from_mesh(mesh, quadrature_order=q)(
                    mesh.points, element_data={"kappa": torch.from_numpy(coef)}),
                "elasticity_E": lambda: EElasticity.from_mesh(mesh, quadrature_order=q)(
                    mesh.points, element_data={"E": torch.from_numpy(coef)}),
            }
            for name, fn in cases.items():
                K = fn()
                ip, ix, dv = canon(K)
                out[f"{etype}/{name}/q{q}/indptr"] = ip
                out[f"{etype}/{name}/q{q}/indices"] = ix
                out[f"{etype}/{name}/q{q}/data"] = dv
            # loads
            f_nodes = np.sin(3.0 * pts[:, 0]) + pts[:, 1] ** 2
            loads = {
                "const": lambda: tm.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=q)(mesh.points),
                "func": lambda: tm.func_node_assembler(
                    lambda x: 2 * math.pi ** 2 * torch.sin(math.pi * x[..., 0]) * torch.sin(math.pi * x[..., 1])
                ).from_mesh(mesh, quadrature_order=q)(mesh.points),
                "point": lambda: PointLoad.from_mesh(mesh, quadrature_order=q)(
                    mesh.points, point_data={"f": torch.from_numpy(f_nodes)}),
                "vector": lambda: tm.const_node_assembler(
                    torch.tensor([0.5, -1.0] if pts.shape[1] == 2 else [0.0, 0.3, -1.0], dtype=torch.float64)
                ).from_mesh(mesh, quadrature_order=q)(mesh.points),
            }

            class PointLoad(tm.NodeAssembler):
                def forward(self, v, f):
                    return v * f

            for name, fn in loads.items():
                out[f"{etype}/load_{name}/q{q}"] = fn().detach().numpy().astype(np.float64)
            out[f"{etype}/f_nodes"] = f_nodes
        # the reference's own (unsorted) edges for the scalar pattern claim
        asm = tm.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=1)
        out[f"{etype}/ref_edges"] = asm.edges.numpy().astype(np.int64)

    # -------------------------------------------------- Poisson on the 64 x 64 square
    pts, cells, bd = square_mesh(64)
    mesh = mk_mesh(pts, cells, bd, "triangle")
    K = tm.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=1)(mesh.points)
    fsrc = tm.func_node_assembler(
        lambda x: 2 * math.pi ** 2 * torch.sin(math.pi * x[..., 0]) * torch.sin(math.pi * x[..., 1]))
    b = fsrc.from_mesh(mesh, quadrature_order=1)(mesh.points)
    cond = tm.Condenser(mesh.boundary_mask)
    K_ii, f_i = cond(K, b)
    ip, ix, dv = canon(K)
    c = K_ii.to_scipy_coo().tocsr()
    c.sum_duplicates(); c.sort_indices()
    u_i = spla.spsolve(c.tocsc(), f_i.numpy())
    u = cond.recover(torch.from_numpy(u_i)).numpy()
    out.update({
        "c1/points": pts, "c1/elements": cells, "c1/boundary": bd,
        "c1/K_indptr": ip, "c1/K_indices": ix, "c1/K_data": dv, "c1/b": b.numpy(),
        "c1/Kii_indptr": c.indptr.astype(np.int64), "c1/Kii_indices": c.indices.astype(np.int64),
        "c1/Kii_data": c.data, "c1/f_i": f_i.numpy(), "c1/u": u,
    })

    # --------------------------------------------- adjoint (compliance), 12^2
    pts, cells, bd = square_mesh(12, jitter=0.2, seed=3)
    mesh = mk_mesh(pts, cells, bd, "triangle")
    g = np.random.default_rng(11).normal(size=cells.shape[0])
    kappa = torch.tensor(np.exp(g), requires_grad=True)
    x = torch.tensor(pts, requires_grad=True)
    Kasm = KappaLaplace.from_mesh(mesh, quadrature_order=1)
    Basm = tm.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)
    K = Kasm(x, element_data={"kappa": kappa})
    bvec = Basm(x)
    cond = tm.Condenser(mesh.boundary_mask)
    K_ii, f_i = cond(K, bvec)
    u_i = SparseSolveScipy.apply(K_ii.values, K_ii.row, K_ii.col, K_ii.shape, f_i)
    u = cond.recover(u_i)
    J = (bvec * u).sum()
    J.backward()
    out.update({
        "adj/points": pts, "adj/elements": cells, "adj/boundary": bd, "adj/kappa": np.exp(g),
        "adj/J": np.array(J.item()), "adj/dJ_dkappa": kappa.grad.numpy(), "adj/dJ_dx": x.grad.numpy(),
        "adj/u": u.detach().numpy(),
    })
    # ------------------------------------ Neo-Hookean energy and its u-gradient
    rng = np.random.default_rng(13)
    for etype, (pts, cells, bd) in meshes.items():
        mesh = mk_mesh(pts, cells, bd, etype)
        dim = mesh.points.shape[1]
        u0 = 0.01 * rng.normal(size=(mesh.points.shape[0], dim))
        out[f"{etype}/nh/u"] = u0
        for q in (1, 2):
            model = NeoHookeanModel.from_mesh(mesh, quadrature_order=q, E=2.0, nu=0.3)
            u = torch.tensor(u0, requires_grad=True)
            energy = model.energy(u)
            energy.backward()
            out[f"{etype}/nh/q{q}/energy"] = np.array(energy.item())
            out[f"{etype}/nh/q{q}/grad_u"] = u.grad.numpy().copy()
    np.savez_compressed(os.path.join(HERE, "reference_fem.npz"), **out)
    print("wrote", len(out), "arrays")
    facet_fixtures(tm, torch, meshes, mk_mesh)
    condense_fixtures(tm, torch, mk_mesh, canon, EElasticity)


def condense_fixtures(tm, torch, mk_mesh, canon, EElasticity):
    """Condenser with prescribed (nonzero) Dirichlet values, update_dirichlet
    + condense_rhs, recover; and a small version of the clamped elasticity
    pipeline (all three dofs fixed on x = 0, body force (0, 0, -1),
    per-element E), solved with scipy's direct solver."""
    import scipy.sparse.linalg as spla
    out = {}
    pts, cells, bd = square_mesh(8, jitter=0.2, seed=21)
    mesh = mk_mesh(pts, cells, bd, "triangle")
    K = tm.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=2)(mesh.points)
    b = tm.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=2)(mesh.points)
    g_full = np.sin(2.0 * pts[:, 0]) + pts[:, 1] ** 2
    cond = tm.Condenser(mesh.boundary_mask, torch.from_numpy(g_full))
    K_ii, f_i = cond(K, b)
    c = K_ii.to_scipy_coo().tocsr()
    c.sum_duplicates()
    c.sort_indices()
    u = cond.recover(torch.from_numpy(spla.spsolve(c.tocsc(), f_i.numpy()))).numpy()
    g2 = np.cos(pts[bd, 0]) - pts[bd, 1]
    cond.update_dirichlet(torch.from_numpy(g2))
    f_i2 = cond.condense_rhs(b)
    u2 = cond.recover(torch.from_numpy(spla.spsolve(c.tocsc(), f_i2.numpy()))).numpy()
    out.update({"dir/points": pts, "dir/elements": cells, "dir/boundary": bd, "dir/g_full": g_full,
                "dir/g2_outer": g2, "dir/f_i": f_i.numpy(), "dir/u": u, "dir/f_i2": f_i2.numpy(), "dir/u2": u2})

    pts, cells, bd = cube_mesh(3, jitter=0.15, seed=22)
    mesh = mk_mesh(pts, cells, bd, "tetra")
    E = np.exp(0.5 * np.random.default_rng(23).normal(size=cells.shape[0]))
    K = EElasticity.from_mesh(mesh, quadrature_order=1)(mesh.points, element_data={"E": torch.from_numpy(E)})
    f = tm.const_node_assembler(torch.tensor([0.0, 0.0, -1.0], dtype=torch.float64)).from_mesh(
        mesh, quadrature_order=1)(mesh.points)
    clamp = np.repeat(np.isclose(pts[:, 0], 0.0), 3)
    cond = tm.Condenser(torch.from_numpy(clamp))
    K_ii, f_i = cond(K, f)
    c = K_ii.to_scipy_coo().tocsr()
    c.sum_duplicates()
    c.sort_indices()
    u = cond.recover(torch.from_numpy(spla.spsolve(c.tocsc(), f_i.numpy()))).numpy()
    ip, ix, dv = canon(K)
    out.update({"c2/points": pts, "c2/elements": cells, "c2/E": E, "c2/clamp": clamp, "c2/f": f.numpy(),
                "c2/K_indptr": ip, "c2/K_indices": ix, "c2/K_data": dv,
                "c2/Kii_indptr": c.indptr.astype(np.int64), "c2/Kii_indices": c.indices.astype(np.int64),
                "c2/Kii_data": c.data, "c2/f_i": f_i.numpy(), "c2/u": u})
    np.savez_compressed(os.path.join(HERE, "reference_condense.npz"), **out)
    print("wrote", len(out), "condense arrays")


def facet_fixtures(tm, torch, meshes, mk_mesh):
    """Boundary loads of the reference FacetAssembler on the form meshes, on
    P2 meshes with curved facets (every midpoint moved), with the default
    boundary mask and with a one-side mask; plus the reference's float32
    facet quadrature tables (points in cell coordinates, weights)."""
    from tensormesh.element.element import Tetrahedron, Triangle

    class FacetOne(tm.FacetAssembler):
        def forward(self, v):
            return v

    class FacetVector(tm.FacetAssembler):
        def forward(self, v):
            t = torch.tensor([0.5, -1.0] if v.shape[0] in (3, 6) else [0.0, 0.3, -1.0], dtype=v.dtype)
            return v[:, None] * t

    class FacetFunc(tm.FacetAssembler):
        def forward(self, x, v):
            return (torch.sin(math.pi * x[0]) + x[1] ** 2) * v

    class FacetPoint(tm.FacetAssembler):
        def forward(self, v, g):
            return g * v

    out = {}
    rng = np.random.default_rng(17)
    # "top": the nodes on the side x_{D-1} = 1 (flagged before the midpoints move)
    facet_meshes = {k: (p, c, b, np.isclose(p[:, -1], 1.0)) for k, (p, c, b) in meshes.items()}
    for name, base, amp in (("triangle6c", "triangle", 0.02), ("tetra10c", "tetra", 0.04)):
        pts, cells, bd = to_p2(*meshes[base])
        top = np.isclose(pts[:, -1], 1.0)
        pts = pts.copy()
        nv = meshes[base][0].shape[0]
        pts[nv:] += rng.uniform(-amp, amp, pts[nv:].shape)
        facet_meshes[name] = (pts, cells, bd, top)
    for etype, (pts, cells, bd, top) in facet_meshes.items():
        ref_type = etype.rstrip("c")
        mesh = mk_mesh(pts, cells, bd, ref_type)
        dim = pts.shape[1]
        mesh.register_point_data("is_top", torch.from_numpy(top))
        g = np.cos(2.0 * pts[:, 0]) + 0.5 * pts[:, dim - 1]
        out[f"{etype}/points"] = pts
        out[f"{etype}/elements"] = cells
        out[f"{etype}/boundary"] = bd
        out[f"{etype}/top"] = top
        out[f"{etype}/facet_g"] = g
        for q in (1, 2, 3, 4):
            cases = {
                "const": lambda: FacetOne.from_mesh(mesh, quadrature_order=q)(mesh.points),
                "vector": lambda: FacetVector.from_mesh(mesh, quadrature_order=q)(mesh.points),
                "func": lambda: FacetFunc.from_mesh(mesh, quadrature_order=q)(mesh.points),
                "point": lambda: FacetPoint.from_mesh(mesh, quadrature_order=q)(
                    mesh.points, point_data={"g": torch.from_numpy(g)}),
                "top": lambda: FacetOne.from_mesh(mesh, boundary_mask="is_top", quadrature_order=q)(mesh.points),
            }
            for case, fn in cases.items():
                out[f"{etype}/facet_{case}/q{q}"] = fn().detach().numpy().astype(np.float64)
    for cls, key in ((Triangle, "triangle"), (Tetrahedron, "tetra")):
        for q in (1, 2, 3, 4):
            w, p = cls.get_facet_quadrature(q, transform=True)
            out[f"facet_table/{key}/q{q}/w"] = w.numpy().astype(np.float64)
            out[f"facet_table/{key}/q{q}/p"] = p.numpy().astype(np.float64)
    np.savez_compressed(os.path.join(HERE, "reference_facet.npz"), **out)
    print("wrote", len(out), "facet arrays")
    write_facet_point_module(out)


FACET_MODULE = os.path.join(os.path.dirname(os.path.dirname(HERE)), "tensormesh_gb300", "facet_reference_points.py")


def write_facet_point_module(arrays, path=FACET_MODULE):
    """Write the package's table of the reference's float32 facet quadrature
    points (``facet_table/<family>/q<order>/p`` of the facet fixture), as
    exact float32 hex literals."""
    lines = ['"""Facet quadrature points of the reference facet rule, in cell reference',
             'coordinates, as the reference computes them in float32 (its float32',
             'least-squares facet maps evaluated in float32; element/element.py:1058-1066,',
             'element/quadrature.py:321-410).  A float32 LAPACK solve cannot be restated',
             'bit for bit, so the values are a table: written by tests/golden/make_golden.py',
             'from the reference\'s own output, one float32 per entry (hex literal).',
             '"""', "", "POINTS = {"]
    for fam in ("triangle", "tetra"):
        for q in (1, 2, 3, 4):
            p = np.asarray(arrays[f"facet_table/{fam}/q{q}/p"], dtype=np.float32)
            F, Qf, D = p.shape
            rows = []
            for f in range(F):
                pts = ", ".join("(" + ", ".join(f"float.fromhex('{float(v).hex()}')" for v in p[f, k]) + ",)"
                                for k in range(Qf))
                rows.append(f"        ({pts},),")
            lines.append(f"    ({fam!r}, {q}): (")
            lines += rows
            lines.append("    ),")
    lines.append("}")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the TensorMesh source tree>")
    main(sys.argv[1])
