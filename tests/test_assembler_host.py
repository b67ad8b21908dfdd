"""Assembler objects on the host (no kernels run): the reference's device /
dtype / type(dtype) accessors, and from_assembler sharing the topology."""
import pytest
import torch

import tensormesh_gb300 as tg


def test_device_dtype_and_type():
    mesh = tg.Mesh.gen_unit_square(3)
    for asm in (tg.LaplaceElementAssembler.from_mesh(mesh), tg.const_node_assembler(1.0).from_mesh(mesh),
                tg.NeoHookeanModel.from_mesh(mesh, E=2.0, nu=0.3)):
        assert asm.device == torch.device("cpu") and asm.dtype == torch.float64
        assert asm.type(torch.float32) is asm and asm.dtype == torch.float32 and asm.points.dtype == torch.float32
        with pytest.raises(TypeError):
            asm.type(torch.int32)


def test_from_assembler_shares_topology_and_calls_post_init():
    mesh = tg.Mesh.gen_unit_cube(2)
    a = tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=1)
    b = tg.LinearElasticityElementAssembler.from_assembler(a, E=3.0, nu=0.25)
    assert b.topology is a.topology and b.quadrature_order == 1
    assert (b.E, b.nu) == (3.0, 0.25)
    with pytest.raises(AssertionError):
        tg.LaplaceElementAssembler.from_assembler(object())


def test_facet_topology_groups_pairs_by_node_in_order():
    """The (selected facet, cell node) pairs of a FacetTopology are grouped by
    node, in pair order inside a node (the fixed order of the reduction)."""
    from tensormesh_gb300.facet import FacetTopology
    from oracle import fem
    mesh = tg.Mesh.gen_unit_cube(3).to_p2()
    el = mesh.cells["tetra10"]
    topo = FacetTopology(el, mesh.n_points, "tetra10", mesh.boundary_mask)
    e, f = fem.facet_select(el.numpy(), "tetra10", mesh.boundary_mask.numpy())
    assert torch.equal(topo.sel, torch.from_numpy(e * 4 + f))
    nodes = el[torch.from_numpy(e)].reshape(-1)
    for n in range(mesh.n_points):
        group = topo.perm[topo.ptr[n]:topo.ptr[n + 1]]
        assert bool((nodes[group] == n).all())
        assert bool((group[1:] > group[:-1]).all())
    assert int(topo.ptr[-1]) == nodes.numel()
