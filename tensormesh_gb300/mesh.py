"""Mesh container with the reference's accessors, plus structured generators.

Mirrors TensorMesh's ``Mesh`` (mesh/mesh.py:86-145 constructor, 227-323
``to_meshio``/``save``, 403-486 ``elements``, 617-652 ``n_elements`` and
``boundary_mask``, 654-669 ``default_element_type``, 693-740
``from_meshio``/``read``): ``points [N, D]``, ``cells {type: [E, B]}``,
``point_data``, ``cell_data {key: {type: [E, ...]}}``, ``field_data``,
``default_element_type``, ``elements()``, ``boundary_mask``, ``dtype``,
``device`` and ``.to``.

A meshio mesh (any object with ``.points``, ``.cells`` holding
``.type``/``.data`` blocks, and optionally ``.point_data``, ``.cell_data``,
``.field_data``, ``.cell_sets``) is accepted as it comes from a file: every
cell block is kept (blocks of one type are concatenated in block order, as
``meshio.Mesh.cells_dict`` does), so a gmsh volume mesh with its line and
boundary-triangle blocks loads; the default element type is the
highest-dimensional one and the points keep that many coordinates.  Element
types the GPU kernels do not cover are stored and raise only when an
assembler is built on them.  ``reorder=True`` converts P2 connectivity from
the Gmsh/VTK node order to the internal one (element.py:108-136).

The generators build the structured meshes of the benchmark configurations
without gmsh: split unit squares (2 triangles per cell) and Kuhn cubes (6
tetrahedra per cell sharing the v000-v111 diagonal), node ids x-fastest,
and P2 versions by edge-midpoint insertion.
"""
from __future__ import annotations

import re
from typing import Dict, Iterable, Optional

import numpy as np
import torch

from .element import TET_EDGES, TRI_EDGES

# Spatial dimension by element-name prefix (element/element_type2dimension.py:
# every entry there is its prefix's dimension; the trailing digits give the
# node count).
_DIM_OF_PREFIX = {"vertex": 0, "line": 1, "polygon": 2, "triangle": 2, "quad": 2,
                  "tetra": 3, "hexahedron": 3, "wedge": 3, "pyramid": 3}
# Kuhn tetrahedra: one per permutation of the axes (x=0, y=1, z=2).
KUHN_PERMUTATIONS = ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0))
# Midside nodes in the Gmsh/VTK (meshio) order: triangle6 nodes 3-5 sit on
# edges 01, 12, 20; tetra10 nodes 4-9 on edges 01, 12, 02, 03, 13, 23.
_VTK_EDGES = {"triangle6": ((0, 1), (1, 2), (0, 2)),
              "tetra10": ((0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3))}


def element_dimension(element_type: str) -> int:
    m = re.match(r"[a-zA-Z]+", element_type)
    if m is None or m.group(0) not in _DIM_OF_PREFIX:
        raise ValueError(f"unknown element type {element_type!r}")
    return _DIM_OF_PREFIX[m.group(0)]


def gmsh_permutation(element_type: str, n_nodes: int) -> torch.Tensor:
    """perm with ``internal = gmsh[..., perm]`` (the reference's
    ``get_gmsh_permutation``, element.py:139-152, 1767-1800, 2020-2080).

    Vertices come first in both orders.  The internal P2 order lists the
    midside node of edge TRI_EDGES[k] / TET_EDGES[k] at position d+1+k; its
    Gmsh/VTK position is that edge's index in the VTK edge list.  Linear
    simplices, lines and vertices keep their order."""
    prefix = re.match(r"[a-zA-Z]+", element_type).group(0)
    if prefix in ("vertex", "line") or element_type in ("triangle", "tetra"):
        return torch.arange(n_nodes)
    if element_type in _VTK_EDGES:
        vtk, local = _VTK_EDGES[element_type], (TRI_EDGES if prefix == "triangle" else TET_EDGES)
        nv = 3 if prefix == "triangle" else 4
        mid = [nv + vtk.index(tuple(sorted(e))) for e in local]
        return torch.tensor(list(range(nv)) + mid)
    raise NotImplementedError(f"reordering {element_type} connectivity is not provided")


def reorder_connectivity(element_type: str, elements: torch.Tensor, to_gmsh: bool = True) -> torch.Tensor:
    """Connectivity between the internal and the Gmsh/VTK node order
    (``Element.reorder``, element.py:108-136)."""
    perm = gmsh_permutation(element_type, elements.shape[-1]).to(elements.device)
    if to_gmsh:
        perm = torch.argsort(perm)
    return elements.index_select(-1, perm)


def _meshio():
    try:
        import meshio
    except ImportError as e:
        raise ImportError("reading, writing and exporting meshes needs the meshio package") from e
    return meshio


def _flag_to_bool(key, v):
    if key.startswith("is_") or key.endswith("_mask"):  # mesh.py:104-114
        return v.bool()
    return v


class Mesh:
    def __init__(self, mesh=None, reorder: bool = False, *, points=None,
                 cells: Optional[Dict[str, torch.Tensor]] = None,
                 point_data: Optional[Dict[str, torch.Tensor]] = None,
                 cell_data: Optional[Dict[str, Dict[str, torch.Tensor]]] = None,
                 field_data: Optional[Dict[str, torch.Tensor]] = None, cell_sets=None):
        if mesh is not None:
            blocks = {}
            data_blocks = {}
            for i, c in enumerate(mesh.cells):
                blocks.setdefault(c.type, []).append(np.asarray(c.data))
                for key, per_block in getattr(mesh, "cell_data", {}).items():
                    data_blocks.setdefault(key, {}).setdefault(c.type, []).append(np.asarray(per_block[i]))
            cells = {k: torch.from_numpy(np.concatenate(v)).long() for k, v in blocks.items()}
            if reorder:
                cells = {k: reorder_connectivity(k, v, to_gmsh=False) for k, v in cells.items()}
            cell_data = {key: {t: torch.from_numpy(np.concatenate(v)) for t, v in per_type.items()}
                         for key, per_type in data_blocks.items()}
            point_data = {k: torch.from_numpy(np.asarray(v)) for k, v in getattr(mesh, "point_data", {}).items()}
            field_data = {k: torch.from_numpy(np.asarray(v)) for k, v in getattr(mesh, "field_data", {}).items()}
            cell_sets = dict(getattr(mesh, "cell_sets", {}) or {})
            dim = max(element_dimension(k) for k in cells)
            points = torch.from_numpy(np.asarray(mesh.points)[:, :dim])
        if points is None or cells is None:
            raise ValueError("Mesh needs a meshio-like object or points= and cells=")
        if len(cells) == 0:
            raise ValueError("Mesh needs at least one cell block")
        self.points = torch.as_tensor(points)
        self.cells = {k: torch.as_tensor(v).long() for k, v in cells.items()}
        self.dim2eletyp: Dict[int, list] = {}
        for k in self.cells:
            self.dim2eletyp.setdefault(element_dimension(k), []).append(k)
        self.point_data = {k: _flag_to_bool(k, torch.as_tensor(v)) for k, v in (point_data or {}).items()}
        self.cell_data = {k: {t: _flag_to_bool(k, torch.as_tensor(v)) for t, v in d.items()}
                          for k, d in (cell_data or {}).items()}
        self.field_data = {k: _flag_to_bool(k, torch.as_tensor(v)) for k, v in (field_data or {}).items()}
        self.cell_sets = dict(cell_sets or {})

    # -- reference accessors ---------------------------------------------------
    @property
    def default_element_type(self):
        """The highest-dimensional element type, or the list of them when
        several share that dimension (mesh.py:133-137)."""
        types = self.dim2eletyp[max(self.dim2eletyp)]
        return types[0] if len(types) == 1 else list(types)

    def elements(self, element_type=None):
        """mesh.py:403-486: None -> the default type (a tensor, or a dict for
        several), "all" -> every block, an int -> the blocks of that dimension
        (-1: the mesh's), a str -> that block, an iterable -> those blocks."""
        if element_type is None:
            t = self.default_element_type
            return self.cells[t] if isinstance(t, str) else {k: self.cells[k] for k in t}
        if isinstance(element_type, str):
            if element_type == "all":
                return dict(self.cells)
            return self.cells[element_type]
        if isinstance(element_type, int):
            d = self.dim if element_type == -1 else element_type
            return {k: self.cells[k] for k in self.dim2eletyp.get(d, [])}
        if isinstance(element_type, Iterable):
            return {k: self.cells[k] for k in element_type}
        raise TypeError(f"element_type must be str, int or Iterable[str], got {element_type!r}")

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
        """Elements of the default type(s) (mesh.py:617-631)."""
        t = self.default_element_type
        return sum(int(self.cells[k].shape[0]) for k in ([t] if isinstance(t, str) else t))

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
        d = pts.device
        return Mesh(points=pts, cells={k: v.to(d) for k, v in self.cells.items()},
                    point_data={k: v.to(d) for k, v in self.point_data.items()},
                    cell_data={k: {t: v.to(d) for t, v in per.items()} for k, per in self.cell_data.items()},
                    field_data={k: v.to(d) for k, v in self.field_data.items()}, cell_sets=self.cell_sets)

    def double(self) -> "Mesh":
        return self.to(dtype=torch.float64)

    def float(self) -> "Mesh":
        return self.to(dtype=torch.float32)

    # -- fields and graph helpers -------------------------------------------------
    def register_point_data(self, key: str, value: torch.Tensor) -> "Mesh":
        """Add a per-point field (mesh.py:147-170)."""
        assert key not in self.point_data, f"the key {key} already exists in point_data"
        assert value.shape[0] == self.points.shape[0], \
            f"the first dimension of value should be {self.points.shape[0]}, but got {value.shape[0]}"
        self.point_data[key] = value
        return self

    def register_element_data(self, key: str, value) -> "Mesh":
        """Add a per-element field (mesh.py:172-199): a tensor for a mesh with
        one default element type, else a dict with one tensor per default type.
        Stored as ``cell_data[key][element_type]``, the layout the constructor
        reads from meshio."""
        t = self.default_element_type
        if isinstance(value, torch.Tensor):
            assert isinstance(t, str), "only for homogeneous elements can value be a tensor; pass a dict per type"
            assert value.shape[0] == self.cells[t].shape[0], \
                f"the first dimension of value should be {self.cells[t].shape[0]}, but got {value.shape[0]}"
            value = {t: value}
        else:
            assert isinstance(value, dict), "value should be a tensor or a dict of tensors per element type"
            types = [t] if isinstance(t, str) else t
            assert set(types) == set(value), f"the keys of value should be {types}, got {list(value)}"
            for k, v in value.items():
                assert v.shape[0] == self.cells[k].shape[0], \
                    f"the first dimension of value should be {self.cells[k].shape[0]}, but got {v.shape[0]}"
        self.cell_data.setdefault(key, {}).update(value)
        return self

    def clone(self) -> "Mesh":
        """A copy whose tensors are clones (the autograd graph through the
        points and fields is kept; mesh.py:488-502)."""
        return Mesh(points=self.points.clone(), cells={k: v.clone() for k, v in self.cells.items()},
                    point_data={k: v.clone() for k, v in self.point_data.items()},
                    cell_data={k: {t: v.clone() for t, v in per.items()} for k, per in self.cell_data.items()},
                    field_data={k: v.clone() for k, v in self.field_data.items()}, cell_sets=dict(self.cell_sets))

    def node_adjacency(self, element_type=None):
        """Node adjacency with ones where two nodes share an element, the
        diagonal included, as a canonical-CSR ``SparseMatrix`` [N, N]
        (mesh.py:327-345, adjacency.py:111-145)."""
        from .plan import node_pattern
        from .sparse import SparseMatrix
        els = self.elements(element_type)
        if isinstance(els, dict):
            els = list(els.values())
        else:
            els = [els]
        n = self.n_points
        if len(els) == 1:
            pat = node_pattern(els[0], n)
            indptr, indices = pat.indptr, pat.indices
        else:
            keys = []
            for el in els:
                e = el.long()
                B = e.shape[1]
                keys.append((e.unsqueeze(2).expand(-1, B, B) * n + e.unsqueeze(1).expand(-1, B, B)).reshape(-1))
            uniq = torch.unique(torch.cat(keys), sorted=True)
            rows = torch.div(uniq, n, rounding_mode="floor")
            indices = (uniq - rows * n).to(torch.int32)
            indptr = torch.zeros(n + 1, dtype=torch.int64, device=uniq.device)
            indptr[1:] = torch.cumsum(torch.bincount(rows, minlength=n), 0)
        ones = torch.ones(indices.shape[0], dtype=torch.get_default_dtype(), device=indices.device)
        return SparseMatrix(ones, indptr=indptr, indices=indices, shape=(n, n))

    # -- meshio round trip -------------------------------------------------------
    @classmethod
    def from_meshio(cls, mesh, reorder: bool = False) -> "Mesh":
        return cls(mesh, reorder)

    @classmethod
    def read(cls, file_name: str, file_format: Optional[str] = None, reorder: bool = False) -> "Mesh":
        return cls(_meshio().read(file_name, file_format), reorder)

    from_file = read

    def to_meshio(self, reorder: bool = False):
        """An in-memory ``meshio.Mesh`` (mesh.py:227-260); ``reorder=True``
        writes connectivity in the Gmsh/VTK order."""
        meshio = _meshio()
        cells = {}
        for k, v in self.cells.items():
            conn = v.detach().cpu()
            cells[k] = (reorder_connectivity(k, conn, to_gmsh=True) if reorder else conn).numpy()
        order = list(cells)
        return meshio.Mesh(
            points=self.points.detach().cpu().numpy(), cells=cells,
            point_data={k: v.detach().cpu().numpy() for k, v in self.point_data.items()},
            cell_data={k: [per[t].detach().cpu().numpy() for t in order if t in per]
                       for k, per in self.cell_data.items()},
            field_data={k: v.detach().cpu().numpy() for k, v in self.field_data.items()},
            cell_sets=self.cell_sets)

    def save(self, file_name: str, file_format: Optional[str] = None) -> "Mesh":
        """``meshio.write`` (mesh.py:267-323): flag arrays become floats; a
        .vtk/.vtu file gets Gmsh/VTK connectivity, 3-D points, a zero ``u``
        point field when there is none, and no cell sets."""
        vtk = file_name.endswith((".vtk", ".vtu"))
        m = self.to_meshio(reorder=vtk)
        flag = lambda k: k.startswith("is_") or k.endswith("_mask")
        m.point_data = {k: (v.astype(float) if flag(k) else v) for k, v in m.point_data.items()}
        m.cell_data = {k: [(b.astype(float) if flag(k) else b) for b in v] for k, v in m.cell_data.items()}
        m.field_data = {k: (v.astype(float) if flag(k) else v) for k, v in m.field_data.items()}
        if vtk:
            if m.points.shape[1] == 2:
                m.points = np.concatenate([m.points, np.zeros((m.points.shape[0], 1))], -1)
            m.point_data.setdefault("u", np.zeros((m.points.shape[0],)))
            m.cell_sets = {}
        _meshio().write(file_name, m, file_format)
        return self

    to_file = save

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
