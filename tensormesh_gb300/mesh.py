"""Mesh container with the reference's accessors, plus structured generators.

Mirrors the parts of TensorMesh's ``Mesh`` (mesh/mesh.py:86-145 constructor,
403-486 ``elements``, 633-652 ``boundary_mask``) that the assembly path
reads: ``points [N, D]``, ``cells {type: [E, B]}``, ``point_data``,
``default_element_type``, ``elements()``, ``boundary_mask``, ``dtype``,
``device`` and ``.to``.  A meshio-like object (``.points``, ``.cells`` with
``.type``/``.data``, ``.point_data``) is accepted directly.

The generators build the structured meshes of the benchmark configurations
without gmsh: split unit squares (2 triangles per cell) and Kuhn cubes (6
tetrahedra per cell sharing the v000-v111 diagonal), node ids x-fastest,
and P2 versions by edge-midpoint insertion.
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np
import torch

from .element import TET_EDGES, TRI_EDGES, element_info

_DIM_OF = {"triangle": 2, "triangle6": 2, "tetra": 3, "tetra10": 3}
# Kuhn tetrahedra: one per permutation of the axes (x=0, y=1, z=2).
KUHN_PERMUTATIONS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))


class Mesh:
    def __init__(self, mesh=None, *, points=None, cells: Optional[Dict[str, torch.Tensor]] = None,
                 point_data: Optional[Dict[str, torch.Tensor]] = None):
        if mesh is not None:
            pts = np.asarray(mesh.points)
            cells = {}
            for c in mesh.cells:
                cells[c.type] = torch.as_tensor(np.asarray(c.data)).long()
            point_data = {k: torch.as_tensor(np.asarray(v)) for k, v in getattr(mesh, "point_data", {}).items()}
            dim = max(_DIM_OF.get(k, 0) for k in cells)
            points = torch.as_tensor(pts[:, :dim])
        if points is None or cells is None:
            raise ValueError("Mesh needs a meshio-like object or points= and cells=")
        self.points = torch.as_tensor(points)
        self.cells = {k: torch.as_tensor(v).long() for k, v in cells.items()}
        self.point_data = {}
        for k, v in (point_data or {}).items():
            v = torch.as_tensor(v)
            if k.startswith("is_") or k.endswith("_mask"):  # mesh.py:104-107
                v = v.bool()
            self.point_data[k] = v
        for k in self.cells:
            element_info(k)  # raises for element types off the GPU path

    # -- reference accessors ---------------------------------------------------
    @property
    def default_element_type(self) -> str:
        dim = max(_DIM_OF[k] for k in self.cells)
        types = [k for k in self.cells if _DIM_OF[k] == dim]
        return types[0] if len(types) == 1 else types

    def elements(self, element_type=None):
        if element_type is None:
            t = self.default_element_type
            return self.cells[t] if isinstance(t, str) else {k: self.cells[k] for k in t}
        if element_type == "all":
            return dict(self.cells)
        return self.cells[element_type]

    @property
    def boundary_mask(self) -> torch.Tensor:
        if "is_boundary" in self.point_data:
            return self.point_data["is_boundary"]
        if "boundary_mask" in self.point_data:
            return self.point_data["boundary_mask"]
        raise KeyError("'boundary_mask' or 'is_boundary' is not found in point_data")

    @property
    def dim(self) -> int:
        return int(self.points.shape[1])

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    @property
    def n_elements(self) -> int:
        return sum(int(v.shape[0]) for v in self.cells.values())

    @property
    def dtype(self) -> torch.dtype:
        return self.points.dtype

    @property
    def device(self) -> torch.device:
        return self.points.device

    def to(self, device=None, dtype=None) -> "Mesh":
        pts = self.points.to(device=device) if device is not None else self.points
        if dtype is not None:
            pts = pts.to(dtype)
        m = Mesh(points=pts, cells={k: v.to(pts.device) for k, v in self.cells.items()},
                 point_data={k: v.to(pts.device) for k, v in self.point_data.items()})
        return m

    def double(self) -> "Mesh":
        return self.to(dtype=torch.float64)

    def float(self) -> "Mesh":
        return self.to(dtype=torch.float32)

    # -- structured generators ---------------------------------------------------
    @staticmethod
    def gen_unit_square(n: int, device="cpu", dtype=torch.float64) -> "Mesh":
        """n x n cells on [0,1]^2; cell (i,j) corners a=(i,j) b=(i+1,j)
        c=(i+1,j+1) d=(i,j+1) split into (a,b,c) and (a,c,d)."""
        dev = torch.device(device)
        xs = torch.linspace(0.0, 1.0, n + 1, dtype=torch.float64, device=dev)
        Y, X = torch.meshgrid(xs, xs, indexing="ij")
        pts = torch.stack([X.reshape(-1), Y.reshape(-1)], 1)
        j, i = torch.meshgrid(torch.arange(n, device=dev), torch.arange(n, device=dev), indexing="ij")
        a = (j * (n + 1) + i).reshape(-1)
        b, c, d = a + 1, a + n + 2, a + n + 1
        tris = torch.stack([torch.stack([a, b, c], 1), torch.stack([a, c, d], 1)], 1).reshape(-1, 3)
        ii = torch.arange(n + 1, device=dev)
        jj, iii = torch.meshgrid(ii, ii, indexing="ij")
        bd = ((iii == 0) | (iii == n) | (jj == 0) | (jj == n)).reshape(-1)
        return Mesh(points=pts.to(dtype), cells={"triangle": tris}, point_data={"is_boundary": bd})

    @staticmethod
    def gen_unit_cube(n: int, device="cpu", dtype=torch.float64) -> "Mesh":
        """n^3 cells on [0,1]^3, node (i,j,k) -> (k(n+1)+j)(n+1)+i; each cell
        split into the 6 Kuhn tetrahedra v000 -> +e_p0 -> +e_p1 -> v111, one per
        axis permutation in lexicographic order."""
        dev = torch.device(device)
        m = n + 1
        xs = torch.linspace(0.0, 1.0, m, dtype=torch.float64, device=dev)
        Z, Y, X = torch.meshgrid(xs, xs, xs, indexing="ij")
        pts = torch.stack([X.reshape(-1), Y.reshape(-1), Z.reshape(-1)], 1)
        k, j, i = torch.meshgrid(torch.arange(n, device=dev), torch.arange(n, device=dev),
                                 torch.arange(n, device=dev), indexing="ij")
        base = ((k * m + j) * m + i).reshape(-1)
        off = (1, m, m * m)
        tets = []
        for perm in KUHN_PERMUTATIONS:
            v1 = base + off[perm[0]]
            v2 = v1 + off[perm[1]]
            v3 = v2 + off[perm[2]]
            tets.append(torch.stack([base, v1, v2, v3], 1))
        tets = torch.stack(tets, 1).reshape(-1, 4)
        kk, jj, ii = torch.meshgrid(torch.arange(m, device=dev), torch.arange(m, device=dev),
                                    torch.arange(m, device=dev), indexing="ij")
        bd = ((ii == 0) | (ii == n) | (jj == 0) | (jj == n) | (kk == 0) | (kk == n)).reshape(-1)
        return Mesh(points=pts.to(dtype), cells={"tetra": tets}, point_data={"is_boundary": bd})

    def to_p2(self) -> "Mesh":
        """Quadratic version: unique edges sorted by (min, max) node id become
        new nodes N.., placed at edge midpoints; each element lists them in the
        reference element's edge order."""
        t = self.default_element_type
        if t not in ("triangle", "tetra"):
            raise ValueError("to_p2 needs a linear simplex mesh")
        cells = self.cells[t]
        N = self.n_points
        loc = TRI_EDGES if t == "triangle" else TET_EDGES
        pairs = torch.stack([torch.sort(cells[:, [a, b]], dim=1).values for a, b in loc], 1)
        key = (pairs[..., 0] * N + pairs[..., 1]).reshape(-1)
        uniq, inv = torch.unique(key, sorted=True, return_inverse=True)
        u0 = torch.div(uniq, N, rounding_mode="floor")
        u1 = uniq - u0 * N
        mid = 0.5 * (self.points[u0] + self.points[u1])
        pts = torch.cat([self.points, mid], 0)
        new_cells = torch.cat([cells, N + inv.view(cells.shape[0], len(loc))], 1)
        pd = {}
        for k, v in self.point_data.items():
            if v.dtype == torch.bool:
                pd[k] = torch.cat([v, v[u0] & v[u1]])
        return Mesh(points=pts, cells={t + ("6" if t == "triangle" else "10"): new_cells}, point_data=pd)
