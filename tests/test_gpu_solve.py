"""SpMV, Condenser and Jacobi-PCG on the GPU against the reference pipeline
(golden: 64x64 Poisson, reference assembler + Condenser + scipy direct
solve) and the oracle."""
import math

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem

pytestmark = pytest.mark.gpu
DEV = "cuda"


def rel_err(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def test_c1_poisson_pipeline_matches_reference(golden):
    mesh = tg.Mesh.gen_unit_square(64, device=DEV)
    K = tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=1)(mesh.points)
    f = tg.func_node_assembler(
        lambda x: 2 * math.pi ** 2 * torch.sin(math.pi * x[..., 0]) * torch.sin(math.pi * x[..., 1]))
    b = f.from_mesh(mesh, quadrature_order=1)(mesh.points)
    assert rel_err(K.values.cpu(), golden["c1/K_data"]) <= 1e-12
    assert rel_err(b.cpu(), golden["c1/b"]) <= 1e-12
    cond = tg.Condenser(mesh.boundary_mask)
    K_ii, f_i = cond(K, b)
    np.testing.assert_array_equal(K_ii.indptr.cpu().numpy(), golden["c1/Kii_indptr"])
    np.testing.assert_array_equal(K_ii.indices.cpu().numpy(), golden["c1/Kii_indices"])
    assert rel_err(K_ii.values.cpu(), golden["c1/Kii_data"]) <= 1e-12
    assert rel_err(f_i.cpu(), golden["c1/f_i"]) <= 1e-12
    u_i = K_ii.solve(f_i, rtol=1e-12)
    info = K_ii.last_solve_info
    assert info.residual <= 1e-12
    u = cond.recover(u_i)
    assert rel_err(u.cpu(), golden["c1/u"]) <= 1e-9
    # same Condenser reused on a second matrix from the same assembler
    K2 = tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=1)(mesh.points)
    K2_ii, _ = cond(K2, b)
    assert torch.equal(K2_ii.values, K_ii.values)


def test_spmv_matches_scipy():
    mesh = tg.Mesh.gen_unit_cube(10, device=DEV)
    K = tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=1)(mesh.points)
    x = torch.randn(K.shape[0], dtype=torch.float64, device=DEV)
    y = (K @ x).cpu().numpy()
    ref = K.to_scipy_csr() @ x.cpu().numpy()
    assert rel_err(y, ref) <= 1e-14


@pytest.mark.parametrize("dtype,rtol", [(torch.float64, 1e-8), (torch.float32, 1e-5)])
def test_pcg_reaches_tolerance(dtype, rtol):
    mesh = tg.Mesh.gen_unit_cube(16, device=DEV, dtype=dtype)
    kappa = torch.exp(torch.randn(mesh.n_elements, device=DEV, dtype=dtype))

    class KL(tg.ElementAssembler):
        def forward(self, gradu, gradv, kappa):
            return kappa * (gradu @ gradv)
    K = KL.from_mesh(mesh, quadrature_order=1)(mesh.points, element_data={"kappa": kappa})
    b = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)(mesh.points)
    cond = tg.Condenser(mesh.boundary_mask)
    K_ii, f_i = cond(K, b)
    u = K_ii.solve(f_i, rtol=rtol)
    info = K_ii.last_solve_info
    assert info.status == 0
    res = np.linalg.norm(K_ii.to_scipy_csr().astype(np.float64) @ u.double().cpu().numpy()
                         - f_i.double().cpu().numpy()) / np.linalg.norm(f_i.double().cpu().numpy())
    assert res <= rtol * 1.01
    # oracle PCG agrees on the solution
    if dtype == torch.float64:
        x, it, r = fem.pcg_jacobi(K_ii.indptr.cpu().numpy(), K_ii.indices.cpu().numpy().astype(np.int64),
                                  K_ii.values.cpu().numpy(), f_i.cpu().numpy(), rtol=1e-10)
        assert rel_err(u.cpu().numpy(), x) <= 1e-6


def test_pcg_iteration_cap_reports_status():
    mesh = tg.Mesh.gen_unit_square(32, device=DEV)
    K = tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=1)(mesh.points)
    b = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)(mesh.points)
    K_ii, f_i = tg.Condenser(mesh.boundary_mask)(K, b)
    with pytest.warns(UserWarning):
        K_ii.solve(f_i, rtol=1e-12, maxiter=3)
    assert K_ii.last_solve_info.status == 3  # TM_ERR_MAXITER
    assert K_ii.last_solve_info.iterations == 3
