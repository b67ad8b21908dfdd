"""The timed CPU baseline (oracle.torch_ref: the reference's own torch
operation sequence for ElementAssembler.__call__) against the reference.

* parity: its CSR values equal the reference's own outputs (golden
  fixtures) to rounding, for P1/P2 triangles and tetrahedra;
* speed: where the reference source tree is available on this machine, the
  two take the same time on the same cores (within +-25%) on a 40^3 Kuhn
  cube, so the CPU baseline stands for the reference's CPU path.  The tree is
  looked up in $TENSORMESH_SRC, then beside this repository; without it the
  timing test is skipped.
"""
import os
import sys
import time

import numpy as np
import pytest
import torch

from oracle import fem
from oracle.torch_ref import ReferenceOps

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def rel_err(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


@pytest.mark.parametrize("etype", ["triangle", "triangle6", "tetra", "tetra10"])
@pytest.mark.parametrize("q", [1, 2, 3])
def test_torch_reference_ops_match_reference_outputs(golden, etype, q):
    pts, el = golden[f"{etype}/points"], golden[f"{etype}/elements"]
    coef = golden[f"{etype}/coef"]
    ops = ReferenceOps(pts, el, etype, q)
    got = ops.values(torch.from_numpy(pts), torch.from_numpy(coef)).numpy()
    ref = golden[f"{etype}/laplace_kappa/q{q}/data"]
    assert got.shape == ref.shape
    assert rel_err(got, ref) <= 1e-12


def _reference_tree():
    cands = [os.environ.get("TENSORMESH_SRC"), os.path.join(os.path.dirname(ROOT), "reference")]
    for c in cands:
        if c and os.path.isfile(os.path.join(c, "tensormesh", "__init__.py")):
            return c
    return None


def _kuhn(n):
    xs = np.linspace(0.0, 1.0, n + 1)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    m = n + 1
    idx = lambda i, j, k: (k * m + j) * m + i  # noqa: E731
    cells = []
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    I, J, K = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = np.stack([I.ravel(), J.ravel(), K.ravel()], 1)
    for p in perms:
        v = base.copy()
        tet = [idx(*v.T)]
        for ax in p:
            v = v.copy()
            v[:, ax] += 1
            tet.append(idx(*v.T))
        cells.append(np.stack(tet, 1))
    return pts, np.stack(cells, 1).reshape(-1, 4)


def _median_time(fn, reps=5):
    fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts))


def test_torch_reference_ops_time_like_the_reference():
    tree = _reference_tree()
    if tree is None:
        pytest.skip("the reference source tree is not on this machine")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden", "_stubs"))
    sys.path.insert(0, tree)
    try:
        import meshio
        import tensormesh as tm
    finally:
        sys.path.remove(tree)
    torch.set_num_threads(os.cpu_count() or 1)
    pts, el = _kuhn(40)
    kappa = np.exp(np.random.default_rng(0).normal(size=el.shape[0]))

    class KappaLaplace(tm.ElementAssembler):
        def forward(self, gradu, gradv, kappa):
            return kappa * (gradu @ gradv)

    mesh = tm.Mesh(meshio.Mesh(pts, [("tetra", el)]))
    asm = KappaLaplace.from_mesh(mesh, quadrature_order=1)
    pts_t = torch.from_numpy(pts)
    kap_t = torch.from_numpy(kappa)
    ops = ReferenceOps(pts, el, "tetra", 1)
    t_ref = _median_time(lambda: asm(pts_t, element_data={"kappa": kap_t}))
    t_ops = _median_time(lambda: ops.values(pts_t, kap_t))
    ratio = t_ops / t_ref
    print(f"reference __call__ {t_ref * 1e3:.1f} ms, torch restatement {t_ops * 1e3:.1f} ms, ratio {ratio:.2f}")
    assert 0.75 <= ratio <= 1.25, ratio


def test_reference_jacobi_pcg_sequence_matches_the_oracle_solver():
    """The timed CPU solve baseline (the reference's CG loop with its Jacobi
    preconditioner, in torch) runs the oracle's Jacobi-PCG iteration."""
    import warnings
    import scipy.sparse as sp
    from oracle import fem
    from oracle.torch_ref import ReferenceJacobiPCG
    n = 300
    A = sp.random(n, n, density=0.03, random_state=3)
    A = (A + A.T + 25.0 * sp.eye(n)).tocsr()
    A.sort_indices()
    b = np.random.default_rng(4).normal(size=n)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ref = ReferenceJacobiPCG(A.indptr, A.indices, A.data)
        x = ref.iterate(torch.from_numpy(b), 40).numpy()
    xo, _, _ = fem.pcg_jacobi(A.indptr, A.indices.astype(np.int64), A.data, b, rtol=1e-14)
    assert np.max(np.abs(x - xo)) <= 1e-10 * np.max(np.abs(xo))
