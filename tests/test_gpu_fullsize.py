"""Size-independent properties at the benchmark's full sizes, where the
oracle cannot assemble the whole matrix in seconds:

* 128^3 Kuhn cube (12,582,912 tetrahedra), FP64 kappa-Laplace with kappa
  piecewise constant on 8^3 blocks (log kappa ~ N(0, 2^2)): linear fields
  are integrated exactly (u^T K u = |a|^2 sum_e kappa_e vol_e for u = a.x),
  rows sum to zero, K is symmetric, a seeded sample of rows equals the
  oracle's, the result is bitwise repeatable, and Jacobi-PCG on the
  condensed system reaches its FP64 true residual;
* 64^3 Kuhn cube elasticity with per-element E: the six rigid-body modes lie
  in the null space and K is symmetric."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem

pytestmark = pytest.mark.gpu
DEV = "cuda"


class KappaLaplace(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * (gradu @ gradv)


class EElasticity(tg.ElementAssembler):
    def forward(self, gradu, gradv, E):
        lam, mu = tg.forms.reference_lame(1.0, 0.3)
        return E * tg.forms.elasticity_block(gradu, gradv, lam, mu)


def block_kappa(n, blocks=8, seed=2024):
    g = np.random.default_rng(seed).normal(0.0, 2.0, size=(blocks,) * 3)
    c = np.arange(n ** 3)
    s = n // blocks
    i, j, k = c % n, (c // n) % n, c // (n * n)
    return np.repeat(np.exp(g[k // s, j // s, i // s]), 6)


def volumes(points, elements):
    X = points[elements.long()]
    d = X[:, 1:] - X[:, :1]
    return torch.linalg.det(d).abs() / 6.0


def transpose_perm(K):
    """Permutation p with (row, col)[p] = (col, row): K symmetric in values
    iff values[p] == values."""
    n = K.shape[0]
    row, col = K.row.long(), K.col.long()
    key = row * n + col
    keyT = col * n + row
    order = torch.argsort(key)
    pos = torch.searchsorted(key[order], keyT)
    assert torch.equal(key[order][pos], keyT), "pattern is not symmetric"
    return order[pos]


@pytest.fixture(scope="module")
def c5():
    mesh = tg.Mesh.gen_unit_cube(128, device=DEV)
    kappa = torch.from_numpy(block_kappa(128)).to(DEV)
    asm = KappaLaplace.from_mesh(mesh, quadrature_order=1)
    K = asm(mesh.points, element_data={"kappa": kappa})
    return mesh, kappa, asm, K


def test_c5_sizes(c5):
    mesh, _, _, K = c5
    assert mesh.n_elements == 12_582_912 and mesh.n_points == 2_146_689
    assert K.nnz == 31_802_497


def test_c5_linear_fields_integrate_exactly(c5):
    mesh, kappa, _, K = c5
    vol_sum = float((kappa * volumes(mesh.points, mesh.cells["tetra"])).sum())
    for a in ((1.0, 0.0, 0.0), (0.3, -0.7, 0.5)):
        av = torch.tensor(a, dtype=torch.float64, device=DEV)
        u = mesh.points @ av
        energy = float(u @ (K @ u))
        assert abs(energy - float(av @ av) * vol_sum) <= 1e-9 * float(av @ av) * vol_sum


def test_c5_rows_sum_to_zero_and_symmetric(c5):
    mesh, _, _, K = c5
    ones = torch.ones(mesh.n_points, dtype=torch.float64, device=DEV)
    absK = K.with_values(K.values.abs())
    r = (K @ ones).abs() / (absK @ ones)
    assert float(r.max()) <= 1e-12
    p = transpose_perm(K)
    assert float((K.values - K.values[p]).abs().max()) <= 2e-13 * float(K.values.abs().max())


def test_c5_sampled_rows_match_oracle(c5):
    mesh, kappa, _, K = c5
    N = mesh.n_points
    el = mesh.cells["tetra"].cpu().numpy()
    pts = mesh.points.cpu().numpy()
    kap = kappa.cpu().numpy()
    rows = np.random.default_rng(11).choice(N, 400, replace=False)
    sampled = np.zeros(N, dtype=bool)
    sampled[rows] = True
    touch = np.nonzero(sampled[el].any(1))[0]
    Ke = fem.element_matrices(pts, el[touch], "tetra", "laplace", 1, coef=kap[touch])   # [m, 4, 4]
    et = el[touch]
    a_idx, b_idx = np.meshgrid(np.arange(4), np.arange(4), indexing="ij")
    r_all = et[:, a_idx].reshape(-1)
    c_all = et[:, b_idx].reshape(-1)
    v_all = Ke.reshape(-1)
    keep = sampled[r_all]
    key, inv = np.unique(r_all[keep] * N + c_all[keep], return_inverse=True)
    ref = np.zeros(key.shape[0])
    np.add.at(ref, inv, v_all[keep])
    ip = K.indptr.cpu().numpy()
    ix = K.indices.cpu().numpy().astype(np.int64)
    vals = K.values.cpu().numpy()
    got_keys, got_vals = [], []
    for r in np.sort(rows):
        s, e = ip[r], ip[r + 1]
        got_keys.append(r * N + ix[s:e])
        got_vals.append(vals[s:e])
    got_keys = np.concatenate(got_keys)
    got_vals = np.concatenate(got_vals)
    np.testing.assert_array_equal(got_keys, key)
    assert np.max(np.abs(got_vals - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_c5_bitwise_repeatable(c5):
    mesh, kappa, asm, K = c5
    ref = K.values.clone()
    again = asm(mesh.points, element_data={"kappa": kappa}).values
    assert torch.equal(again, ref)


def test_c5_pcg_reaches_true_residual(c5):
    mesh, _, _, K = c5
    b = torch.ones(mesh.n_points, dtype=torch.float64, device=DEV)
    cond = tg.Condenser(mesh.boundary_mask)
    K_ii, f_i = cond(K, b)
    u_i = K_ii.solve(f_i, rtol=1e-8)
    res = float(torch.linalg.vector_norm(f_i - K_ii @ u_i) / torch.linalg.vector_norm(f_i))
    assert res <= 1e-8 * 1.0000001
    assert K_ii.last_solve_info.status == 0


def test_c2_rigid_body_modes_and_symmetry():
    mesh = tg.Mesh.gen_unit_cube(64, device=DEV)
    E = torch.from_numpy(np.exp(0.5 * np.random.default_rng(2025).normal(size=mesh.n_elements))).to(DEV)
    K = EElasticity.from_mesh(mesh, quadrature_order=1)(mesh.points, element_data={"E": E})
    assert K.shape == (3 * mesh.n_points, 3 * mesh.n_points)
    x, y, z = mesh.points.unbind(1)
    one, zero = torch.ones_like(x), torch.zeros_like(x)
    modes = [(one, zero, zero), (zero, one, zero), (zero, zero, one),
             (-y, x, zero), (zero, -z, y), (z, zero, -x)]
    absK = K.with_values(K.values.abs())
    for m in modes:
        r = torch.stack(m, 1).reshape(-1).contiguous()
        scale = absK @ r.abs()
        assert float(((K @ r).abs() / scale.clamp_min(1e-300)).max()) <= 1e-12
    p = transpose_perm(K)
    assert float((K.values - K.values[p]).abs().max()) <= 2e-13 * float(K.values.abs().max())
