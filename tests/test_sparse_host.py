"""SparseMatrix container operations that run on the values and the
pattern only (no kernels): sums and differences (same or different
patterns), scalar and elementwise products, transpose, degree, from_dense,
eye, and autograd through the values (the reference's sparse/matrix.py:
133-243, 309-324, 439-459)."""
import numpy as np
import scipy.sparse as sp
import torch

import tensormesh_gb300 as tg
from oracle import fem


def oracle_matrix(form, n=4, seed=0):
    mesh = tg.Mesh.gen_unit_square(n)
    pts = mesh.points.numpy() + 0.02 * np.random.default_rng(seed).normal(size=mesh.points.shape)
    ip, ix, dv = fem.assemble_csr(pts, mesh.cells["triangle"].numpy(), "triangle", form, 2)
    K = tg.SparseMatrix(torch.from_numpy(dv), shape=(len(ip) - 1,) * 2, indptr=torch.from_numpy(ip),
                        indices=torch.from_numpy(ix).to(torch.int32))
    return K, sp.csr_matrix((dv, ix, ip), shape=(len(ip) - 1,) * 2)


def dense(A):
    return A.to_dense().detach().numpy()


def test_sums_products_and_transpose_match_scipy():
    K, Ks = oracle_matrix("laplace")
    M, Ms = oracle_matrix("mass", seed=1)
    dt = 0.25
    np.testing.assert_allclose(dense(K + dt * M), (Ks + dt * Ms).toarray(), rtol=0, atol=1e-15)
    np.testing.assert_allclose(dense(M - K / 2), (Ms - Ks / 2).toarray(), rtol=0, atol=1e-15)
    np.testing.assert_allclose(dense(K * M), Ks.multiply(Ms).toarray(), rtol=0, atol=1e-15)
    assert (K + 0) is K and sum([K, M]).nnz == K.nnz
    # different patterns: union, canonical order
    n = K.shape[0]
    D = tg.SparseMatrix.eye(n, 3.0, dtype=torch.float64)
    R = tg.SparseMatrix(torch.ones(2, dtype=torch.float64), torch.tensor([0, n - 1]), torch.tensor([n - 1, 0]), (n, n))
    S = K + D + R
    ref = (Ks + 3 * sp.eye(n) + sp.coo_matrix(([1.0, 1.0], ([0, n - 1], [n - 1, 0])), shape=(n, n))).tocsr()
    ref.sort_indices()
    np.testing.assert_array_equal(S.indptr.numpy(), ref.indptr)
    np.testing.assert_array_equal(S.indices.numpy(), ref.indices)
    np.testing.assert_allclose(S.values.numpy(), ref.data, rtol=0, atol=1e-15)
    # transpose of a non-symmetric matrix
    A = S + R * 4.0
    At = A.T
    np.testing.assert_array_equal(dense(At), dense(A).T)
    assert At.shape == (n, n) and torch.equal(A.degree(0), At.degree(1))
    assert torch.equal(A.degree(0), torch.from_numpy(np.diff(A.indptr.numpy())))


def test_from_dense_eye_and_autograd_through_values():
    d = torch.tensor([[2.0, 0.0, -1.0], [0.0, 0.0, 0.0], [4.0, 5.0, 0.0]], dtype=torch.float64)
    A = tg.SparseMatrix.from_dense(d)
    assert A.nnz == 4 and torch.equal(A.to_dense(), d)
    I = tg.SparseMatrix.eye(3, dtype=torch.float64)
    assert torch.equal(I.to_dense(), torch.eye(3, dtype=torch.float64))
    v = A.values.clone().requires_grad_(True)
    B = A.with_values(v)
    C = (2.0 * B + I).T
    C.values.sum().backward()
    assert torch.equal(v.grad, torch.full_like(v, 2.0))
    assert B.grad is not None and torch.equal(B.grad.values, v.grad)
    assert not B.detach().values.requires_grad
