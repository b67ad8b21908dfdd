"""Host-side failure handling (no kernels run): bad connectivity and
non-finite inputs are rejected with a clear error before any launch; the
Condenser's prescribed-value contract; the reference's NodeAssembler fast-mode
switches exist and return the assembler."""
import pytest
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300.validate import check_connectivity, check_finite, input_checks_enabled


class _MeshWith:
    """A mesh whose single cell block is replaced (for bad connectivity)."""

    def __init__(self, mesh, cells):
        self.points = mesh.points
        self._cells = cells
        self.default_element_type = mesh.default_element_type

    def elements(self):
        return {self.default_element_type: self._cells}


def test_connectivity_out_of_range_is_an_index_error():
    mesh = tg.Mesh.gen_unit_square(3)
    el = mesh.cells["triangle"].clone()
    el[5, 1] = mesh.n_points           # one past the last node
    with pytest.raises(IndexError, match="element 5 refers to node 16"):
        tg.LaplaceElementAssembler.from_mesh(_MeshWith(mesh, el))
    el = mesh.cells["triangle"].clone()
    el[2, 0] = -1
    with pytest.raises(IndexError, match="element 2 refers to node -1"):
        tg.const_node_assembler(1.0).from_mesh(_MeshWith(mesh, el))
    check_connectivity(mesh.cells["triangle"], mesh.n_points)  # a valid mesh passes


def test_connectivity_shape_asserts_like_the_reference():
    mesh = tg.Mesh.gen_unit_square(2)
    with pytest.raises(AssertionError, match="triangle elements have 3 nodes"):
        tg.LaplaceElementAssembler.from_mesh(_MeshWith(mesh, mesh.cells["triangle"][:, :2].contiguous()))


def test_non_finite_inputs_are_rejected_by_name():
    good = torch.ones(10, dtype=torch.float64)
    check_finite((("points", good), ("kappa", good), ("unused", None)))
    for bad_value in (float("nan"), float("inf"), -float("inf")):
        bad = good.clone()
        bad[7] = bad_value
        with pytest.raises(ValueError, match="kappa holds a non-finite value"):
            check_finite((("points", good), ("kappa", bad)))
    # integer tensors are not coefficients and are not checked
    check_finite((("ids", torch.arange(3)),))


def test_input_checks_can_be_switched_off():
    bad = torch.tensor([1.0, float("nan")])
    assert input_checks_enabled()
    try:
        tg.set_input_checks(False)
        check_finite((("kappa", bad),))
    finally:
        tg.set_input_checks(True)
    with pytest.raises(ValueError):
        check_finite((("kappa", bad),))


def test_condenser_prescribed_value_layouts():
    mask = torch.tensor([True, False, True, False, False])
    full = torch.arange(5, dtype=torch.float64)
    c = tg.Condenser(mask, full)
    assert torch.equal(c.dirichlet_value, torch.tensor([0.0, 2.0], dtype=torch.float64))
    c = tg.Condenser(mask, torch.tensor([7.0, 8.0]))
    assert torch.equal(c.dirichlet_value, torch.tensor([7.0, 8.0]))
    assert torch.equal(tg.Condenser(mask).dirichlet_value, torch.zeros(2))
    with pytest.raises(AssertionError, match="expected 5 .* or 2"):
        tg.Condenser(mask, torch.zeros(3))
    with pytest.raises(AssertionError, match="1-D"):
        tg.Condenser(mask, torch.zeros(5, 1))
    with pytest.raises(AssertionError):
        tg.Condenser(mask.long())


def test_node_assembler_fast_mode_switches_return_self():
    mesh = tg.Mesh.gen_unit_square(2)
    asm = tg.const_node_assembler(1.0).from_mesh(mesh)
    assert not asm.is_compiled()
    assert asm.compile() is asm and asm.is_compiled()
    assert asm.compile(mode="default", fullgraph=True) is asm
    assert asm.reset_compile() is asm and not asm.is_compiled()
    assert asm.flat_mode() is asm and asm.is_compiled()
