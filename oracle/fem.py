"""Float64 numpy restatement of TensorMesh's assemble -> CSR -> solve path.

Test infrastructure only (see the package docstring).  Every function names
the reference lines it restates; citations are paths inside the TensorMesh
source tree.

Conventions shared with the reference:
  * element types "triangle", "triangle6", "tetra", "tetra10";
  * P2 node order = vertices, then edge midpoints in the reference element's
    edge order (element/element.py:1684 triangle edges [[1,2],[0,2],[0,1]],
    element/element.py:1949 tetra edges [[2,3],[1,3],[1,2],[0,3],[0,2],[0,1]]);
  * the Jacobian is J[i,j] = sum_b X[b,j] dN[i,b] (element/element.py:962),
    physical gradients dN J^-T (element.py:964-966), JxW = w |det J|
    (element/transformation.py:1289);
  * CSR output in canonical order (rows ascending, columns ascending within a
    row), which is the order of the reference's scalar ``edges``
    (assemble/element_assembler.py:851-856) and of scipy's canonical CSR of
    the reference's block COO (sparse/matrix.py:355-375).
"""
from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np

# ---------------------------------------------------------------------------
# Quadrature rules: element/quadrature.py:68-116 (triangle), 118-166 (tetra).
# Same points and weights as the reference tables (needed for parity); orders
# 1-4 cover every element/form combination the GPU path supports.
# ---------------------------------------------------------------------------
_TRI_W = {
    1: [0.5],
    2: [0.16666666666666666, 0.16666666666666666, 0.16666666666666666],
    3: [-0.28125, 0.260416666666667, 0.260416666666667, 0.260416666666667],
    4: [0.111690794839006, 0.054975871827661, 0.111690794839006,
        0.054975871827661, 0.111690794839006, 0.054975871827661],
}
_TRI_P = {
    1: [[0.3333333333333333, 0.3333333333333333]],
    2: [[0.16666666666666666, 0.16666666666666666], [0.6666666666666666, 0.16666666666666666],
        [0.16666666666666666, 0.6666666666666666]],
    3: [[0.333333333333333, 0.333333333333333], [0.2, 0.6], [0.6, 0.2], [0.2, 0.2]],
    4: [[0.445948490915965, 0.10810301816807], [0.0915762135097699, 0.816847572980459],
        [0.10810301816807, 0.445948490915965], [0.816847572980459, 0.091576213509771],
        [0.445948490915965, 0.445948490915965], [0.091576213509771, 0.0915762135097699]],
}
_TET_W = {
    1: [0.16666666666666666],
    2: [0.041666666666666664] * 4,
    3: [-0.13333333333333333, 0.075, 0.075, 0.075, 0.075],
    4: [-0.01315555555555555] + [0.007622222222222217] * 4 + [0.02488888888888888] * 6,
}
_a, _b = 0.5854101966249685, 0.1381966011250105
_c, _d = 0.7857142857142857, 0.0714285714285714
_e, _f = 0.1005964238332008, 0.3994035761667992
_TET_P = {
    1: [[0.25, 0.25, 0.25]],
    2: [[_a, _b, _b], [_b, _b, _b], [_b, _b, _a], [_b, _a, _b]],
    3: [[0.25, 0.25, 0.25], [0.5, 0.1666666666666667, 0.1666666666666667],
        [0.1666666666666667, 0.1666666666666667, 0.1666666666666667],
        [0.1666666666666667, 0.1666666666666667, 0.5],
        [0.1666666666666667, 0.5, 0.1666666666666667]],
    4: [[0.25, 0.25, 0.25], [_c, _d, _d], [_d, _d, _d], [_d, _d, _c], [_d, _c, _d],
        [_e, _f, _f], [_f, _e, _f], [_f, _f, _e], [_f, _e, _e], [_e, _f, _e], [_e, _e, _f]],
}

ELEMENTS = {
    # name: (dim, n_basis, basis order)
    "triangle": (2, 3, 1),
    "triangle6": (2, 6, 2),
    "tetra": (3, 4, 1),
    "tetra10": (3, 10, 2),
}
_TRI_EDGES = [(1, 2), (0, 2), (0, 1)]
_TET_EDGES = [(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)]


def quadrature(element_type: str, order: int):
    """Weights [Q] and reference points [Q, D] (element/quadrature.py:68-166)."""
    dim = ELEMENTS[element_type][0]
    if dim == 2:
        return np.array(_TRI_W[order], dtype=np.float64), np.array(_TRI_P[order], dtype=np.float64)
    return np.array(_TET_W[order], dtype=np.float64), np.array(_TET_P[order], dtype=np.float64)


def shape_functions(element_type: str, xi: np.ndarray):
    """Lagrange shape values N [Q, B] and reference gradients dN [Q, D, B].

    The reference obtains the same polynomials by inverting a monomial
    Vandermonde matrix at the basis nodes (element/element.py:557-716); for
    P1/P2 simplices the result is the closed-form barycentric basis used
    here: vertex lambda_i (P1), lambda_i (2 lambda_i - 1) and 4 lambda_i
    lambda_j on edge (i, j) (P2).
    """
    dim, nb, p = ELEMENTS[element_type]
    xi = np.asarray(xi, dtype=np.float64)
    q = xi.shape[0]
    lam = np.concatenate([1.0 - xi.sum(1, keepdims=True), xi], axis=1)  # [Q, D+1]
    dlam = np.concatenate([-np.ones((1, dim)), np.eye(dim)], axis=0)    # [D+1, D]
    if p == 1:
        N = lam.copy()
        dN = np.broadcast_to(dlam.T[None], (q, dim, dim + 1)).copy()
        return N, dN
    edges = _TRI_EDGES if dim == 2 else _TET_EDGES
    N = np.zeros((q, nb))
    dN = np.zeros((q, dim, nb))
    for i in range(dim + 1):
        N[:, i] = lam[:, i] * (2.0 * lam[:, i] - 1.0)
        dN[:, :, i] = (4.0 * lam[:, i] - 1.0)[:, None] * dlam[i][None, :]
    for k, (i, j) in enumerate(edges):
        N[:, dim + 1 + k] = 4.0 * lam[:, i] * lam[:, j]
        dN[:, :, dim + 1 + k] = 4.0 * (lam[:, i][:, None] * dlam[j][None, :] + lam[:, j][:, None] * dlam[i][None, :])
    return N, dN


def geometry(points: np.ndarray, elements: np.ndarray, dN: np.ndarray, w: np.ndarray):
    """Physical gradients [E, Q, B, D] and JxW [E, Q].

    element/element.py:962-966 (J = einsum("ebj,qib->eqij"), inverse,
    gradients = einsum("qib,eqji->eqbj")) and element/transformation.py:1289
    (JxW = w |det J|).
    """
    X = points[elements]                                   # [E, B, D]
    J = np.einsum("ebj,qib->eqij", X, dN)                  # [E, Q, D, D]
    Jinv = np.linalg.inv(J)
    grads = np.einsum("qib,eqji->eqbj", dN, Jinv)
    jxw = w[None, :] * np.abs(np.linalg.det(J))
    return grads, jxw


def voigt_elasticity_block(ga: np.ndarray, gb: np.ndarray, E, nu):
    """B_a^T C B_b for all quadrature points / basis pairs.

    functional/elasticity.py:132-200 (voigt_shape_grad: diag rows then the
    shear rows of ``skew``), :202-284 (voigt_stiffness with
    lambda = E nu / ((1+nu)(1-2nu)), mu = E / (2(1+nu))), assemble/builtin.py:
    173-179 (Ba.T @ C @ Bb).  ga [..., D], gb [..., D] -> [..., D, D].
    """
    dim = ga.shape[-1]
    E = np.asarray(E, dtype=np.float64)
    if E.ndim == 0:
        # voigt_stiffness wraps the Python-float constants with torch.tensor
        # (elasticity.py:263-266): they are rounded to float32 (the default
        # dtype) before the cast to float64.
        mu = np.float64(np.float32(float(E) / (2.0 * (1.0 + nu))))
        lam = np.float64(np.float32(float(E) * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))))
    else:
        # per-element modulus times the unit-modulus (rounded) constants
        mu = E * np.float64(np.float32(1.0 / (2.0 * (1.0 + nu))))
        lam = E * np.float64(np.float32(nu / ((1.0 + nu) * (1.0 - 2.0 * nu))))

    def bmat(g):
        if dim == 2:
            z = np.zeros_like(g[..., 0])
            rows = [np.stack([g[..., 0], z], -1), np.stack([z, g[..., 1]], -1),
                    np.stack([g[..., 1], g[..., 0]], -1)]
        else:
            z = np.zeros_like(g[..., 0])
            gx, gy, gz = g[..., 0], g[..., 1], g[..., 2]
            rows = [np.stack([gx, z, z], -1), np.stack([z, gy, z], -1), np.stack([z, z, gz], -1),
                    np.stack([z, gz, gy], -1), np.stack([gz, z, gx], -1), np.stack([gy, gx, z], -1)]
        return np.stack(rows, -2)  # [..., nv, D]

    nv = 3 if dim == 2 else 6
    Ba, Bb = bmat(ga), bmat(gb)
    C = np.zeros(E.shape + (nv, nv))
    nn = dim
    for i in range(nn):
        for j in range(nn):
            C[..., i, j] = lam
        C[..., i, i] = lam + 2.0 * mu
    for i in range(nn, nv):
        C[..., i, i] = mu
    return Ba, Bb, C


def element_matrices(points, elements, element_type, form, quadrature_order,
                     coef=None, nu=0.3):
    """Per-element matrices [E, B, B] (scalar forms) or [E, B, B, D, D].

    Restates ElementAssembler.__call__ (assemble/element_assembler.py:402-464)
    for the built-in forms: Laplace ``gradu @ gradv`` (assemble/builtin.py:
    62-63) optionally times a per-element coefficient passed as element data
    (docs user_guide/differentiability.rst:252-253), mass ``u * v``
    (builtin.py:100-101), and isotropic linear elasticity (builtin.py:
    173-179) with per-element or scalar Young's modulus ``coef``.
    Quadrature sum: einsum("eqij...,eq->eij...") (element_assembler.py:211).
    """
    w, xi = quadrature(element_type, quadrature_order)
    N, dN = shape_functions(element_type, xi)
    grads, jxw = geometry(points, elements, dN, w)
    n_el = elements.shape[0]
    if form == "laplace":
        integrand = np.einsum("eqid,eqjd->eqij", grads, grads)
        if coef is not None:
            integrand = np.asarray(coef, dtype=np.float64).reshape(n_el, 1, 1, 1) * integrand
        return np.einsum("eqij,eq->eij", integrand, jxw)
    if form == "mass":
        integrand = np.einsum("qi,qj->qij", N, N)[None]
        if coef is not None:
            integrand = np.asarray(coef, dtype=np.float64).reshape(n_el, 1, 1, 1) * integrand
        else:
            integrand = np.broadcast_to(integrand, (n_el,) + integrand.shape[1:])
        return np.einsum("eqij,eq->eij", integrand, jxw)
    if form == "elasticity":
        E = 1.0 if coef is None else np.asarray(coef, dtype=np.float64)
        ga = grads[:, :, :, None, :]   # [E, Q, B, 1, D]
        gb = grads[:, :, None, :, :]   # [E, Q, 1, B, D]
        Ba, Bb, _ = voigt_elasticity_block(ga, gb, 1.0, nu)
        _, _, C = voigt_elasticity_block(grads[:, 0, 0], grads[:, 0, 0], E, nu)  # [E or (), nv, nv]
        if C.ndim == 2:
            C = np.broadcast_to(C, (n_el,) + C.shape)
        Ba = np.broadcast_to(Ba, np.broadcast_shapes(Ba.shape, Bb.shape))
        Bb = np.broadcast_to(Bb, Ba.shape)
        blk = np.einsum("eqijvd,evw,eqijwc->eqijdc", Ba, C, Bb)
        return np.einsum("eqijdc,eq->eijdc", blk, jxw)
    raise ValueError(form)


# ---------------------------------------------------------------------------
# Pattern: ElementAssembler.from_mesh (assemble/element_assembler.py:838-866)
# ---------------------------------------------------------------------------
def node_pattern(elements: np.ndarray, n_points: int):
    """Unique node pairs in canonical CSR order plus the slot of every
    element entry (the reference's ``edges`` and ``elem_eids``,
    element_assembler.py:838-866).  Returns indptr [N+1], indices [nnz],
    slots [E, B, B] (int64)."""
    E, B = elements.shape
    u = np.repeat(elements, B, axis=1).reshape(-1).astype(np.int64)
    v = np.tile(elements, (1, B)).reshape(-1).astype(np.int64)
    key = u * n_points + v
    uniq, inv = np.unique(key, return_inverse=True)
    rows = uniq // n_points
    cols = uniq % n_points
    indptr = np.zeros(n_points + 1, dtype=np.int64)
    np.add.at(indptr, rows + 1, 1)
    indptr = np.cumsum(indptr)
    return indptr, cols.astype(np.int64), inv.reshape(E, B, B).astype(np.int64)


def block_pattern(indptr: np.ndarray, indices: np.ndarray, H: int):
    """Dof-level canonical CSR of the block expansion row = H*i + a,
    col = H*j + b (sparse/matrix.py:355-375, then scipy canonical order)."""
    n = indptr.shape[0] - 1
    deg = np.diff(indptr)
    dof_deg = np.repeat(deg * H, H)
    dptr = np.concatenate([[0], np.cumsum(dof_deg)]).astype(np.int64)
    out = np.empty(dptr[-1], dtype=np.int64)
    for i in range(n):
        cols = indices[indptr[i]:indptr[i + 1]]
        blk = (cols[:, None] * H + np.arange(H)[None, :]).reshape(-1)
        for a in range(H):
            r = i * H + a
            out[dptr[r]:dptr[r + 1]] = blk
    return dptr, out


def scatter_csr(elem_mats: np.ndarray, slots: np.ndarray, nnz: int):
    """ReduceProjector: index_add of [E,B,B] entries into [nnz]
    (assemble/projector.py:95-130).  Summation order = element order."""
    vals = np.zeros(nnz)
    np.add.at(vals, slots.reshape(-1), elem_mats.reshape(-1))
    return vals


def scatter_block_csr(elem_blocks: np.ndarray, slots: np.ndarray, indptr, indices, H: int):
    """Scatter [E,B,B,H,H] blocks into dof-level canonical CSR values."""
    nnz_node = indices.shape[0]
    node_vals = np.zeros((nnz_node, H, H))
    np.add.at(node_vals, slots.reshape(-1), elem_blocks.reshape(-1, H, H))
    n = indptr.shape[0] - 1
    deg = np.diff(indptr)
    out = []
    for i in range(n):
        blk = node_vals[indptr[i]:indptr[i + 1]]        # [deg, H, H]
        for a in range(H):
            out.append(blk[:, a, :].reshape(-1))
    return np.concatenate(out) if out else np.zeros(0)


def assemble_csr(points, elements, element_type, form, quadrature_order,
                 coef=None, nu=0.3):
    """Full ElementAssembler.from_mesh(...)(...) in canonical CSR:
    (indptr, indices, values) at dof level."""
    n_points = points.shape[0]
    indptr, indices, slots = node_pattern(elements, n_points)
    Ke = element_matrices(points, elements, element_type, form, quadrature_order, coef, nu)
    if form == "elasticity":
        H = points.shape[1]
        dptr, dind = block_pattern(indptr, indices, H)
        return dptr, dind, scatter_block_csr(Ke, slots, indptr, indices, H)
    return indptr, indices, scatter_csr(Ke, slots, indices.shape[0])


def assemble_values_threaded(points, elements, element_type, form, quadrature_order,
                             slots, nnz, coef=None, nu=0.3, threads=1, chunk=1 << 16):
    """Scalar-form CSR values with element chunks spread over threads (numpy
    releases the GIL inside its kernels).  Used only as the timed CPU
    baseline; the per-chunk math is ``element_matrices`` and the scatter is
    a bincount per chunk summed in chunk order (deterministic)."""
    E = elements.shape[0]
    starts = list(range(0, E, chunk))

    def work(s):
        e = min(E, s + chunk)
        c = None if coef is None else np.asarray(coef)[s:e]
        Ke = element_matrices(points, elements[s:e], element_type, form, quadrature_order, c, nu)
        return np.bincount(slots[s:e].reshape(-1), weights=Ke.reshape(-1), minlength=nnz)

    if threads <= 1:
        parts = [work(s) for s in starts]
    else:
        with ThreadPoolExecutor(threads) as ex:
            parts = list(ex.map(work, starts))
    vals = np.zeros(nnz)
    for p in parts:
        vals += p
    return vals


# ---------------------------------------------------------------------------
# Loads: NodeAssembler (assemble/node_assembler.py:616-698, 242-409) with the
# const / func / point-data forms (assemble/builtin.py:886-969).
# ---------------------------------------------------------------------------
def assemble_load(points, elements, element_type, quadrature_order, kind, value=None):
    """Load vector b_i = sum_e sum_q f(x_q) N_i(x_q) JxW (node_assembler.py
    139-151 integrate, 665-670 scatter by elements.flatten()).

    kind = "const": value is a scalar or a length-H vector -> [N*H] node-major;
    kind = "point": value is point data [N] or [N, H] interpolated at
    quadrature points with einsum("eb...,qb->eq...") (node_assembler.py:389);
    kind = "func": value is a callable f(x) on coordinates [..., D].
    """
    w, xi = quadrature(element_type, quadrature_order)
    N, dN = shape_functions(element_type, xi)
    _, jxw = geometry(points, elements, dN, w)
    n_points = points.shape[0]
    if kind == "const":
        c = np.atleast_1d(np.asarray(value, dtype=np.float64))
        fq = np.broadcast_to(c, (elements.shape[0], xi.shape[0], c.shape[0]))
    elif kind == "point":
        pv = np.asarray(value, dtype=np.float64)
        if pv.ndim == 1:
            pv = pv[:, None]
        fq = np.einsum("ebh,qb->eqh", pv[elements], N)
    elif kind == "func":
        xq = np.einsum("ebd,qb->eqd", points[elements], N)
        f = np.asarray(value(xq), dtype=np.float64)
        fq = f[..., None] if f.ndim == 2 else f
    else:
        raise ValueError(kind)
    be = np.einsum("eqh,qb,eq->ebh", fq, N, jxw)          # [E, B, H]
    H = be.shape[-1]
    out = np.zeros((n_points, H))
    np.add.at(out, elements.reshape(-1), be.reshape(-1, H))
    return out.reshape(-1) if H > 1 else out[:, 0]


# ---------------------------------------------------------------------------
# Facet (boundary) loads: assemble/facet_assembler.py.
# ---------------------------------------------------------------------------
# Facet f of a simplex is the facet opposite vertex f; its nodes are the other
# vertices and, for P2, the midpoints of the edges between them
# (element.py:1411-1440 element_to_facet; Triangle.edge, Tetrahedron.face).
_FACET_VERTICES = {2: [(1, 2), (0, 2), (0, 1)], 3: [(1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)]}


def facet_nodes(element_type: str) -> np.ndarray:
    """Local node ids of each facet [F, nodes per facet]."""
    dim, nb, p = ELEMENTS[element_type]
    out = []
    for vs in _FACET_VERTICES[dim]:
        nodes = list(vs)
        if p == 2:
            edges = _TRI_EDGES if dim == 2 else _TET_EDGES
            nodes += [dim + 1 + k for k, (i, j) in enumerate(edges) if i in vs and j in vs]
        out.append(nodes)
    return np.array(out, dtype=np.int64)


def facet_rule(dim: int, order: int):
    """Facet-local rule (weights [Qf], points [Qf, D-1]): Gauss-Legendre with
    ``order`` points moved to [0, 1] for edges (element/quadrature.py:9-66
    lin_quadrature), the triangle rule for faces (tri_quadrature)."""
    if dim == 2:
        x, w = np.polynomial.legendre.leggauss(order)
        return 0.5 * w, (0.5 * (x + 1.0))[:, None]
    return np.array(_TRI_W[order], dtype=np.float64), np.array(_TRI_P[order], dtype=np.float64)


def facet_quadrature(element_type: str, order: int):
    """Exact float64 facet quadrature in cell reference coordinates.

    Returns (w [F, Qf], xi [F, Qf, D], tangents [F, D-1, D]): facet f is the
    affine image r -> P_a + sum_k r_k (P_{v_k+1} - P_a) of the reference
    segment / triangle, P the reference simplex's vertices and (a, v_1, ...)
    the facet's vertices in order (element.py:993-1066
    get_local_facet_mapping_fns; quadrature.py:321-410 pushes the rule through
    it).  The reference evaluates this table in float32
    (transformation.py:519-531 leaves get_facet_quadrature's float32 default),
    so its float64 facet integrals carry float32 rounding of w and xi; pass its
    table as ``tables`` to facet_load to reproduce it."""
    dim = ELEMENTS[element_type][0]
    P = np.concatenate([np.zeros((1, dim)), np.eye(dim)], 0)
    w, r = facet_rule(dim, order)
    xi, tang = [], []
    for vs in _FACET_VERTICES[dim]:
        T = np.stack([P[v] - P[vs[0]] for v in vs[1:]], 0)       # [D-1, D]
        xi.append(P[vs[0]][None, :] + r @ T)
        tang.append(T)
    F = len(xi)
    return np.broadcast_to(w, (F, w.shape[0])).copy(), np.stack(xi), np.stack(tang)


def facet_select(elements: np.ndarray, element_type: str, boundary_mask: np.ndarray):
    """(element ids, local facet ids) of the facets whose nodes are all
    flagged, element-major (facet_assembler.py:491-508: facet candidates of
    the elements touching the mask, kept when ``mask[facet].all(-1)``,
    ``nonzero`` order)."""
    fn = facet_nodes(element_type)
    sel = np.asarray(boundary_mask, dtype=bool)[elements[:, fn]].all(-1)   # [E, F]
    e, f = np.nonzero(sel)
    return e, f


def facet_load(points, elements, element_type, boundary_mask, quadrature_order, kind, value=None,
               tables=None):
    """Facet load b_i = sum over selected facets, facet quadrature points of
    g(x_q) N_i(xi_q) w_q |F_q| (facet_assembler.py:195-235 same-facet branch:
    integrand, einsum with FxW, ReduceProjector over the whole cell's nodes).

    |F| = sqrt(det(F F^T)) with F = d(gamma)/dr . J, J[i, j] = sum_b
    dN_b/dxi_i X_b[j] evaluated at the float64 facet points
    (transformation.py:993-1003 detF, element.py:1295-1409
    eval_facet_jacobian, 1203-1293 eval_facet_cell_jacobian); the shape values
    and weights come from ``tables`` = (w [F, Qf], xi [F, Qf, D]) when given,
    else from the exact rule (facet_quadrature).

    kind as for assemble_load: "const" (scalar or [H]), "point" (node data
    [N] or [N, H] interpolated with the facet shape values), "func" (callable
    of x [..., D], x interpolated with the facet shape values).
    """
    dim = ELEMENTS[element_type][0]
    w_ex, xi_ex, tang = facet_quadrature(element_type, quadrature_order)
    w_t, xi_t = (w_ex, xi_ex) if tables is None else (np.asarray(tables[0], np.float64),
                                                       np.asarray(tables[1], np.float64))
    F, Qf = xi_t.shape[:2]
    N_t = np.stack([shape_functions(element_type, xi_t[f])[0] for f in range(F)])      # [F, Qf, B]
    dN_ex = np.stack([shape_functions(element_type, xi_ex[f])[1] for f in range(F)])   # [F, Qf, D, B]
    e, f = facet_select(elements, element_type, boundary_mask)
    X = points[elements[e]]                                                            # [S, B, D]
    J = np.einsum("sbj,sqib->sqij", X, dN_ex[f])
    T = np.einsum("ski,sqij->sqkj", tang[f], J)                                        # [S, Qf, D-1, D]
    detF = np.sqrt(np.linalg.det(T @ np.swapaxes(T, -1, -2)))
    fxw = w_t[f] * detF                                                                # [S, Qf]
    Ns = N_t[f]                                                                        # [S, Qf, B]
    if kind == "const":
        c = np.atleast_1d(np.asarray(value, dtype=np.float64))
        fq = np.broadcast_to(c, (len(e), Qf, c.shape[0]))
    elif kind == "point":
        pv = np.asarray(value, dtype=np.float64)
        if pv.ndim == 1:
            pv = pv[:, None]
        fq = np.einsum("sbh,sqb->sqh", pv[elements[e]], Ns)
    elif kind == "func":
        xq = np.einsum("sbd,sqb->sqd", X, Ns)
        fv = np.asarray(value(xq), dtype=np.float64)
        fq = fv[..., None] if fv.ndim == 2 else fv
    else:
        raise ValueError(kind)
    be = np.einsum("sqh,sqb,sq->sbh", fq, Ns, fxw)
    H = be.shape[-1]
    out = np.zeros((points.shape[0], H))
    np.add.at(out, elements[e].reshape(-1), be.reshape(-1, H))
    return out.reshape(-1) if H > 1 else out[:, 0]


# ---------------------------------------------------------------------------
# Condenser (operator/condense.py:182-220 layout, 238-309 call, 429-458
# recover).  Boolean-mask compaction keeps CSR order.
# ---------------------------------------------------------------------------
def condense(indptr, indices, values, dirichlet_mask, dirichlet_value, rhs):
    n = indptr.shape[0] - 1
    mask = np.asarray(dirichlet_mask, dtype=bool)
    inner = ~mask
    rows = np.repeat(np.arange(n), np.diff(indptr))
    is_inner_edge = inner[rows] & inner[indices]
    is_ou2in_edge = inner[rows] & mask[indices]
    local = np.full(n, -1, dtype=np.int64)
    local[inner] = np.arange(inner.sum())
    local[mask] = np.arange(mask.sum())
    ni = int(inner.sum())
    ir, ic = local[rows[is_inner_edge]], local[indices[is_inner_edge]]
    iv = values[is_inner_edge]
    iptr = np.zeros(ni + 1, dtype=np.int64)
    np.add.at(iptr, ir + 1, 1)
    iptr = np.cumsum(iptr)
    uo = np.zeros(int(mask.sum())) if dirichlet_value is None else np.asarray(dirichlet_value, np.float64)
    if uo.shape[0] == n:
        uo = uo[mask]
    orr, occ = local[rows[is_ou2in_edge]], local[indices[is_ou2in_edge]]
    ov = values[is_ou2in_edge]
    minus = np.zeros(ni)
    np.add.at(minus, orr, ov * uo[occ])
    f_i = np.asarray(rhs, np.float64)[inner] - minus
    return iptr, ic, iv, f_i


def recover(u_inner, dirichlet_mask, dirichlet_value=None):
    mask = np.asarray(dirichlet_mask, dtype=bool)
    out = np.zeros(mask.shape[0])
    out[~mask] = u_inner
    if dirichlet_value is not None:
        dv = np.asarray(dirichlet_value, np.float64)
        out[mask] = dv[mask] if dv.shape[0] == mask.shape[0] else dv
    return out


# ---------------------------------------------------------------------------
# Solvers.  Reference: SparseSolveScipy (sparse/solve/scipy_solve.py:21-53)
# for the direct solve and its adjoint; Jacobi preconditioning
# (sparse/solve/torch_solve.py:24-59) inside a textbook PCG.
# ---------------------------------------------------------------------------
def csr_matvec(indptr, indices, values, x):
    rows = np.repeat(np.arange(indptr.shape[0] - 1), np.diff(indptr))
    y = np.zeros(indptr.shape[0] - 1)
    np.add.at(y, rows, values * x[indices])
    return y


def spsolve(indptr, indices, values, b):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n = indptr.shape[0] - 1
    A = sp.csr_matrix((values, indices, indptr), shape=(n, n))
    return spla.spsolve(A.tocsc(), b)


def pcg_jacobi(indptr, indices, values, b, rtol=1e-8, maxiter=100000):
    """Jacobi-preconditioned CG to ||b - A x|| / ||b|| <= rtol.
    Returns (x, iterations, relative residual)."""
    import scipy.sparse as sp
    n = indptr.shape[0] - 1
    A = sp.csr_matrix((values, indices, indptr), shape=(n, n))
    d = A.diagonal().copy()
    d[d == 0] = 1.0
    dinv = 1.0 / d
    x = np.zeros(n)
    r = b.copy()
    z = dinv * r
    p = z.copy()
    rz = r @ z
    bn = math.sqrt(b @ b)
    it = 0
    while it < maxiter and math.sqrt(r @ r) > rtol * bn:
        Ap = A @ p
        alpha = rz / (p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        z = dinv * r
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        it += 1
    res = math.sqrt(np.sum((b - A @ x) ** 2)) / bn
    return x, it, res


def compliance_gradients_kappa(points, elements, element_type, quadrature_order, kappa, u, dJdb=None):
    """Adjoint of J = b^T u with K(kappa) u = b, b independent of kappa:
    dJ/dkappa_e = -u_e^T K0_e u_e (K0_e = unit-coefficient element matrix).
    Restates the chain SparseSolveScipy.backward (scipy_solve.py:42-53:
    grad_b = A^-T g, grad_values = -grad_b[row] u[col]) followed by the
    index_add / einsum backward, for the symmetric Laplace form."""
    K0 = element_matrices(points, elements, element_type, "laplace", quadrature_order, None)
    ue = u[elements]
    lam = u  # symmetric K and J = b^T u  =>  adjoint = u
    return -np.einsum("ei,eij,ej->e", lam[elements], K0, ue)


def neo_hookean(points, elements, element_type, quadrature_order, u, E=1.0, nu=0.3):
    """Neo-Hookean energy and its gradient with respect to the nodal
    displacement u [N, D] (assemble/builtin.py:220-334, NeoHookeanModel;
    ElementAssembler.energy, element_assembler.py:468-680).

    psi(F) = mu/2 (tr F^T F - d) - mu ln J + lam/2 (ln J)^2 with F = I + grad u,
    grad u[i][j] = sum_b u_b[i] dN_b/dx_j ("eb...,eqbd->eq...d"), J = det F,
    mu = E / (2 (1 + nu)), lam = E nu / ((1 + nu)(1 - 2 nu)) (Python floats);
    energy = sum over elements and quadrature points of psi * w |det J_x|.
    The gradient is the first Piola-Kirchhoff stress P = mu F + (lam ln J - mu)
    F^-T contracted with the shape gradients: dE/du_b[i] = sum_q JxW P[i][d]
    dN_b/dx_d, scattered to the nodes (what autograd of the energy returns).
    """
    w, xi = quadrature(element_type, quadrature_order)
    _, dN = shape_functions(element_type, xi)
    grads, jxw = geometry(points, elements, dN, w)          # [E, Q, B, D], [E, Q]
    dim = points.shape[1]
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    ue = u[elements]                                        # [E, B, D]
    gu = np.einsum("ebi,eqbd->eqid", ue, grads)             # [E, Q, D, D]
    F = np.eye(dim)[None, None] + gu
    J = np.linalg.det(F)
    lnJ = np.log(J)
    I1 = (F * F).sum(axis=(-1, -2))
    psi = 0.5 * mu * (I1 - dim) - mu * lnJ + 0.5 * lam * lnJ ** 2
    energy = float((psi * jxw).sum())
    FinvT = np.swapaxes(np.linalg.inv(F), -1, -2)
    P = mu * F + (lam * lnJ - mu)[..., None, None] * FinvT  # [E, Q, D, D]
    fe = np.einsum("eqid,eqbd,eq->ebi", P, grads, jxw)      # [E, B, D]
    g = np.zeros_like(u, dtype=np.float64)
    np.add.at(g, elements.reshape(-1), fe.reshape(-1, dim))
    return energy, g
