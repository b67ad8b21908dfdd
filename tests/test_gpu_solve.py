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


def test_condenser_with_prescribed_values_matches_reference(golden_condense):
    """Nonzero Dirichlet values through the GPU Condenser: f_i, the recovered
    solution, then update_dirichlet + condense_rhs with new values."""
    g = golden_condense
    pts = torch.tensor(g["dir/points"], device=DEV)
    bd = torch.tensor(g["dir/boundary"], device=DEV)
    mesh = tg.Mesh(points=pts, cells={"triangle": torch.tensor(g["dir/elements"], device=DEV)},
                   point_data={"is_boundary": bd})
    K = tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=2)(mesh.points)
    b = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=2)(mesh.points)
    cond = tg.Condenser(mesh.boundary_mask, torch.tensor(g["dir/g_full"], device=DEV))
    K_ii, f_i = cond(K, b)
    assert rel_err(f_i.cpu(), g["dir/f_i"]) <= 1e-12
    u = cond.recover(K_ii.solve(f_i, rtol=1e-13))
    assert rel_err(u.cpu(), g["dir/u"]) <= 1e-10
    cond.update_dirichlet(torch.tensor(g["dir/g2_outer"], device=DEV))
    f_i2 = cond.condense_rhs(b)
    assert rel_err(f_i2.cpu(), g["dir/f_i2"]) <= 1e-12
    u2 = cond.recover(K_ii.solve(f_i2, rtol=1e-13))
    assert rel_err(u2.cpu(), g["dir/u2"]) <= 1e-10


def test_clamped_elasticity_pipeline_matches_reference(golden_condense):
    """Per-element-E elasticity clamped on x = 0 under a body force (the C2
    configuration at a size the reference solves directly)."""
    g = golden_condense
    mesh = tg.Mesh(points=torch.tensor(g["c2/points"], device=DEV),
                   cells={"tetra": torch.tensor(g["c2/elements"], device=DEV)})

    class EElasticity(tg.ElementAssembler):
        def forward(self, gradu, gradv, E):
            lam, mu = tg.forms.reference_lame(1.0, 0.3)
            return E * tg.forms.elasticity_block(gradu, gradv, lam, mu)

    K = EElasticity.from_mesh(mesh, quadrature_order=1)(mesh.points,
                                                       element_data={"E": torch.tensor(g["c2/E"], device=DEV)})
    np.testing.assert_array_equal(K.indptr.cpu().numpy(), g["c2/K_indptr"])
    np.testing.assert_array_equal(K.indices.cpu().numpy(), g["c2/K_indices"])
    assert rel_err(K.values.cpu(), g["c2/K_data"]) <= 1e-12
    f = tg.const_node_assembler(torch.tensor([0.0, 0.0, -1.0], dtype=torch.float64)).from_mesh(
        mesh, quadrature_order=1)(mesh.points)
    assert rel_err(f.cpu(), g["c2/f"]) <= 1e-12
    cond = tg.Condenser(torch.tensor(g["c2/clamp"], device=DEV))
    K_ii, f_i = cond(K, f)
    np.testing.assert_array_equal(K_ii.indptr.cpu().numpy(), g["c2/Kii_indptr"])
    np.testing.assert_array_equal(K_ii.indices.cpu().numpy(), g["c2/Kii_indices"])
    assert rel_err(K_ii.values.cpu(), g["c2/Kii_data"]) <= 1e-12
    assert rel_err(f_i.cpu(), g["c2/f_i"]) <= 1e-12
    u = cond.recover(K_ii.solve(f_i, rtol=1e-13))
    assert rel_err(u.cpu(), g["c2/u"]) <= 1e-9


def test_bounded_grid_barrier_times_out_and_context_survives():
    """The PCG kernels' grid barrier gives up instead of spinning: a
    cooperative launch in which one CTA never arrives returns TM_ERR_TIMEOUT
    (here after 2^20 polls), and the next solve on the same context works."""
    import ctypes
    from tensormesh_gb300 import _lib
    lib = _lib.load()
    work = torch.zeros(4096, dtype=torch.uint8, device=DEV)
    status = ctypes.c_int32(-1)
    st = lib.tm_selftest_barrier_timeout(8, 1 << 20, ctypes.byref(status), ctypes.c_void_p(work.data_ptr()),
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _lib.TM_OK
    assert status.value == _lib.TM_ERR_TIMEOUT
    # a single CTA cannot wait on anyone: rejected before any launch
    assert lib.tm_selftest_barrier_timeout(1, 1 << 20, ctypes.byref(status), ctypes.c_void_p(work.data_ptr()),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == _lib.TM_ERR_INVALID
    mesh = tg.Mesh.gen_unit_square(16, device=DEV)
    K = tg.LaplaceElementAssembler.from_mesh(mesh, quadrature_order=1)(mesh.points)
    b = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)(mesh.points)
    K_ii, f_i = tg.Condenser(mesh.boundary_mask)(K, b)
    K_ii.solve(f_i, rtol=1e-10)
    assert K_ii.last_solve_info.status == 0 and K_ii.last_solve_info.residual <= 1e-10
