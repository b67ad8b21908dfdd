"""CPU oracle for the tensorised finite-element hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the ``tensormesh_gb300`` package imports
this package; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and only
as the checker or as the timed CPU baseline -- never as the product path.

``oracle.fem`` is a float64 numpy restatement of the reference algorithm
(TensorMesh ``assemble/element_assembler.py``, ``assemble/node_assembler.py``,
``element/transformation.py``, ``element/element.py``,
``operator/condense.py``, ``sparse/solve/*``); every function cites the
reference lines it follows.  It is pinned against golden fixtures generated
by running the reference package itself (``tests/golden/make_golden.py``),
see ``tests/test_oracle_golden.py``.
"""
from . import fem  # noqa: F401
