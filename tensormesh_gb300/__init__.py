"""tensormesh_gb300: GB300-native (sm_103a) drop-in for TensorMesh's
tensorised finite-element hot path -- assemble (map-reduce) -> CSR scatter ->
SpMV / Jacobi-PCG -- behind the reference's own Python API.

Exports mirror ``tensormesh/__init__.py``: Mesh, Condenser, ElementAssembler,
NodeAssembler, LaplaceElementAssembler, MassElementAssembler,
LinearElasticityElementAssembler, const_node_assembler, func_node_assembler,
FacetAssembler, plus SparseMatrix.
"""
from .mesh import Mesh
from .sparse import SparseMatrix
from .assemble import (ElementAssembler, NodeAssembler, LaplaceElementAssembler, MassElementAssembler,
                       LinearElasticityElementAssembler, const_node_assembler, func_node_assembler)
from .condense import Condenser
from .energy import NeoHookeanModel
from .facet import FacetAssembler
from .validate import set_input_checks

__all__ = ["Mesh", "SparseMatrix", "ElementAssembler", "NodeAssembler", "LaplaceElementAssembler",
           "MassElementAssembler", "LinearElasticityElementAssembler", "const_node_assembler",
           "func_node_assembler", "Condenser", "NeoHookeanModel", "FacetAssembler", "set_input_checks"]
