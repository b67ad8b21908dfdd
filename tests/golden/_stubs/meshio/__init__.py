"""Minimal stand-in for the ``meshio`` package, used only to import the
reference TensorMesh package when generating golden fixtures.

The reference's ``Mesh.__init__`` reads ``.cells`` (objects with ``.type``
and ``.data``), ``.cells_dict``, ``.point_data``, ``.cell_data``,
``.cell_data_dict``, ``.field_data``, ``.cell_sets`` and ``.points``
(tensormesh/mesh/mesh.py:86-145).  Nothing else is provided.
"""
import numpy as np


class CellBlock:
    def __init__(self, type, data):
        self.type = type
        self.data = np.asarray(data)


class Mesh:
    def __init__(self, points, cells, point_data=None, cell_data=None,
                 field_data=None, cell_sets=None):
        self.points = np.asarray(points)
        if isinstance(cells, dict):
            cells = list(cells.items())
        self.cells = [c if isinstance(c, CellBlock) else CellBlock(c[0], c[1])
                      for c in cells]
        self.point_data = dict(point_data or {})
        self.cell_data = dict(cell_data or {})
        self.field_data = dict(field_data or {})
        self.cell_sets = dict(cell_sets or {})

    @property
    def cells_dict(self):
        out = {}
        for c in self.cells:
            out[c.type] = c.data if c.type not in out else np.concatenate([out[c.type], c.data])
        return out

    @property
    def cell_data_dict(self):
        return {k: {c.type: v[i] for i, c in enumerate(self.cells)}
                for k, v in self.cell_data.items()}


def read(*a, **k):
    raise RuntimeError("meshio stub: file IO is not available")


def write(*a, **k):
    raise RuntimeError("meshio stub: file IO is not available")
