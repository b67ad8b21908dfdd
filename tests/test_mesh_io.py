"""Mesh container against meshio-style input: every cell block kept, the
default element type and the point dimension taken from the highest-dimensional
block, Gmsh/VTK node order converted on request, and the meshio round trip
(the reference's mesh/mesh.py:86-145, 227-323, 403-486, 617-669)."""
import sys
import types

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300 import mesh as M


class Block:
    def __init__(self, type, data):
        self.type, self.data = type, np.asarray(data)


class FakeMeshio(types.ModuleType):
    """Records what ``save`` hands to ``meshio.write``; ``Mesh`` holds the
    constructor's arguments as attributes, as meshio's does."""

    def __init__(self):
        super().__init__("meshio")
        self.written = None

        class Mesh:
            def __init__(self, points, cells, point_data=None, cell_data=None, field_data=None, cell_sets=None):
                self.points = np.asarray(points)
                self.cells = [Block(k, v) for k, v in cells.items()]
                self.point_data = dict(point_data or {})
                self.cell_data = dict(cell_data or {})
                self.field_data = dict(field_data or {})
                self.cell_sets = dict(cell_sets or {})

        self.Mesh = Mesh

    def write(self, name, mesh, fmt=None):
        self.written = (name, mesh, fmt)

    def read(self, name, fmt=None):
        return self.written[1]


def gmsh_like_cube(n=2):
    """A tetra volume with the extra blocks a gmsh file carries: boundary
    triangles, a line and a vertex, split over two tetra blocks; points in 3-D."""
    cube = tg.Mesh.gen_unit_cube(n)
    tets = cube.cells["tetra"].numpy()
    h = len(tets) // 2
    tri = np.array([[0, 1, 2], [1, 2, 3]])
    blocks = [Block("vertex", [[0]]), Block("line", [[0, 1], [1, 2]]), Block("triangle", tri),
              Block("tetra", tets[:h]), Block("tetra", tets[h:])]
    src = types.SimpleNamespace(
        points=cube.points.numpy(), cells=blocks,
        point_data={"is_boundary": cube.boundary_mask.numpy().astype(np.uint8), "T": np.arange(cube.n_points)},
        cell_data={"region": [np.array([7]), np.array([1, 2]), np.array([3, 4]),
                              np.full(h, 5), np.full(len(tets) - h, 6)]},
        field_data={"is_fixed": np.array([1, 0])}, cell_sets={})
    return cube, src


def test_meshio_blocks_kept_and_default_type():
    cube, src = gmsh_like_cube()
    m = tg.Mesh(src)
    assert sorted(m.cells) == ["line", "tetra", "triangle", "vertex"]
    assert m.default_element_type == "tetra"
    assert m.dim == 3 and m.n_elements == cube.n_elements
    assert torch.equal(m.elements(), cube.cells["tetra"])
    assert set(m.elements("all")) == set(m.cells)
    assert list(m.elements(2)) == ["triangle"] and list(m.elements(-1)) == ["tetra"]
    assert list(m.elements(["line", "vertex"])) == ["line", "vertex"]
    assert m.boundary_mask.dtype == torch.bool and torch.equal(m.boundary_mask, cube.boundary_mask)
    assert m.field_data["is_fixed"].dtype == torch.bool
    assert m.point_data["T"].dtype != torch.bool
    assert torch.equal(m.cell_data["region"]["tetra"],
                       torch.cat([torch.full((cube.n_elements // 2,), 5),
                                  torch.full((cube.n_elements - cube.n_elements // 2,), 6)]))


def test_surface_mesh_points_cut_to_two_coordinates():
    sq = tg.Mesh.gen_unit_square(3)
    pts3 = np.concatenate([sq.points.numpy(), np.zeros((sq.n_points, 1))], 1)
    src = types.SimpleNamespace(points=pts3, cells=[Block("line", [[0, 1]]), Block("triangle", sq.cells["triangle"])])
    m = tg.Mesh(src)
    assert m.dim == 2 and m.default_element_type == "triangle"
    assert torch.equal(m.points, sq.points)


def test_mixed_same_dimension_types_listed():
    src = types.SimpleNamespace(points=np.zeros((8, 3)),
                                cells=[Block("triangle", [[0, 1, 2]]), Block("quad", [[0, 1, 2, 3]])])
    m = tg.Mesh(src)
    assert m.default_element_type == ["triangle", "quad"]
    assert m.n_elements == 2
    with pytest.raises(NotImplementedError):
        tg.LaplaceElementAssembler.from_mesh(m)


def test_unknown_element_type_raises():
    src = types.SimpleNamespace(points=np.zeros((3, 2)), cells=[Block("blob", [[0, 1, 2]])])
    with pytest.raises(ValueError):
        tg.Mesh(src)


def test_gmsh_permutations_match_reference():
    """The reference's get_gmsh_permutation for the simplices (element.py:
    1767-1800 triangles, 2020-2080 tetrahedra), as it returns them."""
    assert M.gmsh_permutation("tetra10", 10).tolist() == [0, 1, 2, 3, 9, 8, 5, 7, 6, 4]
    assert M.gmsh_permutation("triangle6", 6).tolist() == [0, 1, 2, 4, 5, 3]
    assert M.gmsh_permutation("tetra", 4).tolist() == [0, 1, 2, 3]
    assert M.gmsh_permutation("triangle", 3).tolist() == [0, 1, 2]
    assert M.gmsh_permutation("line3", 3).tolist() == [0, 1, 2]
    with pytest.raises(NotImplementedError):
        M.gmsh_permutation("quad", 4)


@pytest.mark.parametrize("base", ["square", "cube"])
def test_reorder_round_trip_and_vtk_midpoints(base, monkeypatch):
    fake = FakeMeshio()
    monkeypatch.setitem(sys.modules, "meshio", fake)
    p2 = (tg.Mesh.gen_unit_square(3) if base == "square" else tg.Mesh.gen_unit_cube(2)).to_p2()
    t = p2.default_element_type
    vm = p2.to_meshio(reorder=True)
    (blk,) = vm.cells
    conn = blk.data
    pts = vm.points
    nv = 3 if t == "triangle6" else 4
    for k, (a, b) in enumerate(M._VTK_EDGES[t]):
        np.testing.assert_allclose(pts[conn[:, nv + k]], 0.5 * (pts[conn[:, a]] + pts[conn[:, b]]), atol=0)
    back = tg.Mesh.from_meshio(vm, reorder=True)
    assert torch.equal(back.cells[t], p2.cells[t])
    assert torch.equal(back.points, p2.points)
    same = tg.Mesh(vm)
    assert not torch.equal(same.cells[t], p2.cells[t])


def test_save_vtk_pads_and_casts(monkeypatch):
    fake = FakeMeshio()
    monkeypatch.setitem(sys.modules, "meshio", fake)
    sq = tg.Mesh.gen_unit_square(2).to_p2()
    sq.save("out.vtu")
    name, m, fmt = fake.written
    assert name == "out.vtu" and fmt is None
    assert m.points.shape[1] == 3 and np.all(m.points[:, 2] == 0)
    assert m.point_data["is_boundary"].dtype == np.float64
    assert "u" in m.point_data and m.cell_sets == {}
    assert m.cells[0].data.tolist() == M.reorder_connectivity(
        "triangle6", sq.cells["triangle6"], to_gmsh=True).tolist()
    sq.save("out.msh")
    _, m2, _ = fake.written
    assert m2.points.shape[1] == 2 and "u" not in m2.point_data
    assert torch.equal(torch.from_numpy(m2.cells[0].data), sq.cells["triangle6"])
    r = tg.Mesh.read("out.msh")
    assert torch.equal(r.cells["triangle6"], sq.cells["triangle6"]) and r.boundary_mask.dtype == torch.bool


def test_to_keeps_all_fields():
    _, src = gmsh_like_cube()
    m = tg.Mesh(src).to(dtype=torch.float32)
    assert m.dtype == torch.float32 and sorted(m.cells) == ["line", "tetra", "triangle", "vertex"]
    assert "region" in m.cell_data and "is_fixed" in m.field_data


@pytest.mark.gpu
def test_gmsh_like_mesh_assembles_its_volume_block():
    from oracle import fem
    cube, src = gmsh_like_cube(3)
    m = tg.Mesh(src).to("cuda")
    K = tg.LaplaceElementAssembler.from_mesh(m, quadrature_order=1)(m.points)
    ip, ix, dv = fem.assemble_csr(cube.points.numpy(), cube.cells["tetra"].numpy(), "tetra", "laplace", 1)
    np.testing.assert_array_equal(K.indptr.cpu().numpy(), ip)
    np.testing.assert_array_equal(K.indices.cpu().numpy(), ix)
    assert np.max(np.abs(K.values.cpu().numpy() - dv)) <= 1e-12 * np.max(np.abs(dv))


def test_register_fields_clone_and_node_adjacency():
    cube, src = gmsh_like_cube()
    m = tg.Mesh(src)
    t = torch.arange(m.n_points, dtype=torch.float64)
    assert m.register_point_data("temp", t) is m and torch.equal(m.point_data["temp"], t)
    with pytest.raises(AssertionError):
        m.register_point_data("temp", t)
    with pytest.raises(AssertionError):
        m.register_point_data("short", t[:-1])
    k = torch.rand(m.n_elements, dtype=torch.float64)
    m.register_element_data("kappa", k)
    assert torch.equal(m.cell_data["kappa"]["tetra"], k)
    with pytest.raises(AssertionError):
        m.register_element_data("bad", k[:-1])
    pts = m.points.clone().requires_grad_(True)
    m2 = tg.Mesh(points=pts, cells=m.cells, point_data=m.point_data).clone()
    m2.points.sum().backward()
    assert torch.equal(pts.grad, torch.ones_like(pts))
    # node adjacency: all pairs inside each tetra, diagonal included, canonical order
    A = m.node_adjacency()
    el = m.cells["tetra"].numpy()
    pairs = {(int(a), int(b)) for e in el for a in e for b in e}
    rows = np.repeat(np.arange(m.n_points), np.diff(A.indptr.numpy()))
    got = list(zip(rows.tolist(), A.indices.numpy().tolist()))
    assert got == sorted(pairs)
    assert A.values.dtype == torch.get_default_dtype() and bool((A.values == 1).all())
    # several types of one dimension are merged
    two = tg.Mesh(points=torch.zeros(5, 2), cells={"triangle": torch.tensor([[0, 1, 2]]),
                                                   "quad": torch.tensor([[1, 2, 3, 4]])})
    A2 = two.node_adjacency()
    rows = np.repeat(np.arange(5), np.diff(A2.indptr.numpy()))
    assert set(zip(rows.tolist(), A2.indices.numpy().tolist())) == (
        {(a, b) for a in (0, 1, 2) for b in (0, 1, 2)} | {(a, b) for a in (1, 2, 3, 4) for b in (1, 2, 3, 4)})
