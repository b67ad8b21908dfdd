"""Reference elements, quadrature rules and shape-function tables.

Restates, for the simplices on the hot path, TensorMesh's
``element/quadrature.py`` (tri 68-116, tet 118-166) and the Lagrange bases of
``element/element.py`` (Triangle 1673-1800, Tetrahedron 1936-2089).  The
quadrature points and weights are the reference's own numbers (a parity
requirement); the P1/P2 bases are written in closed barycentric form with the
reference's node order: vertices, then edge midpoints in the reference
element's edge order (triangle edges [[1,2],[0,2],[0,1]], tetra edges
[[2,3],[1,3],[1,2],[0,3],[0,2],[0,1]]).
"""
from __future__ import annotations

import functools

import numpy as np
import torch

from ._lib import TM_TET4, TM_TET10, TM_TRI3, TM_TRI6

# name -> (C-ABI id, dim, n_basis, polynomial order)
ELEMENT_TYPES = {
    "triangle": (TM_TRI3, 2, 3, 1),
    "triangle6": (TM_TRI6, 2, 6, 2),
    "tetra": (TM_TET4, 3, 4, 1),
    "tetra10": (TM_TET10, 3, 10, 2),
}

TRI_EDGES = ((1, 2), (0, 2), (0, 1))
TET_EDGES = ((2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1))

_TRI_RULES = {
    1: ([0.5], [[0.3333333333333333, 0.3333333333333333]]),
    2: ([0.16666666666666666] * 3,
        [[0.16666666666666666, 0.16666666666666666], [0.6666666666666666, 0.16666666666666666],
         [0.16666666666666666, 0.6666666666666666]]),
    3: ([-0.28125, 0.260416666666667, 0.260416666666667, 0.260416666666667],
        [[0.333333333333333, 0.333333333333333], [0.2, 0.6], [0.6, 0.2], [0.2, 0.2]]),
    4: ([0.111690794839006, 0.054975871827661, 0.111690794839006, 0.054975871827661,
         0.111690794839006, 0.054975871827661],
        [[0.445948490915965, 0.10810301816807], [0.0915762135097699, 0.816847572980459],
         [0.10810301816807, 0.445948490915965], [0.816847572980459, 0.091576213509771],
         [0.445948490915965, 0.445948490915965], [0.091576213509771, 0.0915762135097699]]),
}
_g1, _g2 = 0.5854101966249685, 0.1381966011250105
_k1, _k2 = 0.7857142857142857, 0.0714285714285714
_k3, _k4 = 0.1005964238332008, 0.3994035761667992
_S = 0.1666666666666667
_TET_RULES = {
    1: ([0.16666666666666666], [[0.25, 0.25, 0.25]]),
    2: ([0.041666666666666664] * 4, [[_g1, _g2, _g2], [_g2, _g2, _g2], [_g2, _g2, _g1], [_g2, _g1, _g2]]),
    3: ([-0.13333333333333333, 0.075, 0.075, 0.075, 0.075],
        [[0.25, 0.25, 0.25], [0.5, _S, _S], [_S, _S, _S], [_S, _S, 0.5], [_S, 0.5, _S]]),
    4: ([-0.01315555555555555] + [0.007622222222222217] * 4 + [0.02488888888888888] * 6,
        [[0.25, 0.25, 0.25], [_k1, _k2, _k2], [_k2, _k2, _k2], [_k2, _k2, _k1], [_k2, _k1, _k2],
         [_k3, _k4, _k4], [_k4, _k3, _k4], [_k4, _k4, _k3], [_k4, _k3, _k3], [_k3, _k4, _k3],
         [_k3, _k3, _k4]]),
}
MAX_QUADRATURE_ORDER = 4


def element_info(element_type: str):
    if element_type not in ELEMENT_TYPES:
        raise NotImplementedError(
            f"element type {element_type!r} is not on the GPU path; supported: {sorted(ELEMENT_TYPES)}")
    return ELEMENT_TYPES[element_type]


def quadrature(element_type: str, order: int):
    """(weights [Q], points [Q, D]) as float64 numpy arrays."""
    _, dim, _, _ = element_info(element_type)
    rules = _TRI_RULES if dim == 2 else _TET_RULES
    if order not in rules:
        raise NotImplementedError(f"quadrature order {order} (supported 1..{MAX_QUADRATURE_ORDER})")
    w, p = rules[order]
    return np.asarray(w, dtype=np.float64), np.asarray(p, dtype=np.float64)


def shape_tables(element_type: str, xi: np.ndarray):
    """N [Q, B] and reference gradients dN [Q, B, D] at points xi [Q, D]."""
    _, dim, nb, order = element_info(element_type)
    q = xi.shape[0]
    lam = np.concatenate([1.0 - xi.sum(1, keepdims=True), xi], axis=1)
    dlam = np.concatenate([-np.ones((1, dim)), np.eye(dim)], axis=0)
    N = np.zeros((q, nb))
    dN = np.zeros((q, nb, dim))
    if order == 1:
        N[:] = lam
        dN[:] = dlam[None]
        return N, dN
    for i in range(dim + 1):
        N[:, i] = lam[:, i] * (2.0 * lam[:, i] - 1.0)
        dN[:, i, :] = (4.0 * lam[:, i] - 1.0)[:, None] * dlam[i][None]
    edges = TRI_EDGES if dim == 2 else TET_EDGES
    for k, (i, j) in enumerate(edges):
        N[:, dim + 1 + k] = 4.0 * lam[:, i] * lam[:, j]
        dN[:, dim + 1 + k, :] = 4.0 * (lam[:, i][:, None] * dlam[j][None] + lam[:, j][:, None] * dlam[i][None])
    return N, dN


@functools.lru_cache(maxsize=None)
def _table_numpy(element_type: str, order: int):
    w, xi = quadrature(element_type, order)
    N, dN = shape_tables(element_type, xi)
    return w, N, dN


_DEVICE_TABLES = {}


def kernel_tables(element_type: str, order: int, device) -> torch.Tensor:
    """Flat float64 table [w(Q), N(Q*B), dN(Q*B*D)] as read by the kernels
    (uploaded once per device and cached)."""
    key = (element_type, order, str(torch.device(device)))
    t = _DEVICE_TABLES.get(key)
    if t is None:
        w, N, dN = _table_numpy(element_type, order)
        flat = np.concatenate([w.ravel(), N.ravel(), dN.ravel()])
        t = _DEVICE_TABLES[key] = torch.from_numpy(flat).to(device=device, dtype=torch.float64)
    return t


def n_quadrature(element_type: str, order: int) -> int:
    return _table_numpy(element_type, order)[0].shape[0]


def shape_values(element_type: str, order: int):
    """(w [Q], N [Q, B]) as float64 numpy arrays."""
    w, N, _ = _table_numpy(element_type, order)
    return w, N
