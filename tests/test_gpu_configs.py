"""The benchmark configurations at their stated sizes (the other GPU tests use
small cases of the same code paths):

* C2: 3D isotropic elasticity, P1 tets on a 64^3 Kuhn cube (1,572,864 tets,
  823,875 dofs), per-element E = exp(0.5 g), nu = 0.3, x = 0 face clamped,
  body force (0, 0, -1): Jacobi-PCG to a 1e-8 FP64 relative residual, checked
  with an independent FP64 product;
* C3: 256 unit-square P1 meshes, N ~ U{32..256} (seeded), kappa = exp(g):
  the batched persistent launch, 8 instances (the largest, the smallest and
  six more) against the FP64 oracle: K within 1e-5 (FP32 assembly), u
  against the FP64 direct solve;
* C4: 2D P1 Poisson on a 256 x 256 grid, kappa = exp(g): dJ/dkappa and
  dJ/d(interior xy) of the compliance against central differences (h = 1e-6)
  on 64 seeded directions each.
"""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem

pytestmark = pytest.mark.gpu
DEV = "cuda"


class EElasticity(tg.ElementAssembler):
    def forward(self, gradu, gradv, E):
        lam, mu = tg.forms.reference_lame(1.0, 0.3)
        return E * tg.forms.elasticity_block(gradu, gradv, lam, mu)


class KappaLaplace(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * (gradu @ gradv)


def test_c2_elasticity_pcg_64cube():
    mesh = tg.Mesh.gen_unit_cube(64, device=DEV)
    rng = np.random.default_rng(2026)
    E = torch.from_numpy(np.exp(0.5 * rng.normal(size=mesh.n_elements))).to(DEV)
    K = EElasticity.from_mesh(mesh, quadrature_order=1)(mesh.points, element_data={"E": E})
    f = tg.const_node_assembler(torch.tensor([0.0, 0.0, -1.0], dtype=torch.float64)).from_mesh(mesh, quadrature_order=1)(mesh.points)
    clamp = (mesh.points[:, 0] == 0.0).repeat_interleave(3)
    cond = tg.Condenser(clamp)
    K_ii, f_i = cond(K, f)
    assert K_ii.shape[0] == 3 * (mesh.n_points - 65 * 65)
    u_i = K_ii.solve(f_i, rtol=1e-8)
    info = K_ii.last_solve_info
    assert info.status == 0 and info.residual <= 1e-8, info
    # independent FP64 product (torch sparse CSR)
    A = torch.sparse_csr_tensor(K_ii.indptr, K_ii.indices.long(), K_ii.values, size=K_ii.shape)
    r = f_i - torch.mv(A, u_i)
    true_res = float(torch.linalg.norm(r) / torch.linalg.norm(f_i))
    assert true_res <= 1e-8 * 1.0001, true_res
    u = cond.recover(u_i).view(-1, 3)
    assert float(u[:, 2].min()) < 0.0 and torch.all(u[clamp.view(-1, 3)[:, 0]] == 0)


def c3_batch():
    rng = np.random.default_rng(2024 + 3)
    sizes = rng.integers(32, 257, size=256)
    meshes = [tg.Mesh.gen_unit_square(int(k), device=DEV) for k in sizes]
    kap = np.exp(rng.normal(size=sum(m.n_elements for m in meshes)))
    return sizes, meshes, kap


def test_c3_batched_full_size(tmp_path, monkeypatch):
    monkeypatch.setenv("TM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    from tensormesh_gb300.batched import BatchedPoisson
    sizes, meshes, kap = c3_batch()
    bp = BatchedPoisson(meshes)
    u, info = bp(torch.from_numpy(kap).to(DEV), rtol=1e-6, graph=True)
    torch.cuda.synchronize()
    assert int((info.status.cpu() == 0).sum()) == 256
    vals = bp.values.double().cpu().numpy()
    ip = bp.pattern.indptr.cpu().numpy()
    eoff = np.concatenate([[0], np.cumsum([m.n_elements for m in meshes])])
    order = np.argsort(sizes)
    picks = sorted({int(order[-1]), int(order[0])} | set(np.random.default_rng(5).choice(256, 6, replace=False).tolist()))
    for i in picks:
        m = meshes[i]
        pts, el = m.points.cpu().numpy(), m.cells["triangle"].cpu().numpy()
        ki = kap[eoff[i]:eoff[i + 1]]
        oip, oix, odv = fem.assemble_csr(pts, el, "triangle", "laplace", 1, coef=ki)
        r0, r1 = bp.node_ptr[i], bp.node_ptr[i + 1]
        got = vals[ip[r0]:ip[r1]]
        assert np.max(np.abs(got - odv)) <= 1e-5 * np.max(np.abs(odv)), i
        bref = fem.assemble_load(pts, el, "triangle", 1, "const", 1.0)
        bd = m.boundary_mask.cpu().numpy()
        iptr, iind, ival, fi = fem.condense(oip, oix, odv, bd, None, bref)
        uref = fem.recover(fem.spsolve(iptr, iind, ival, fi), bd)
        uu = u[r0:r1].double().cpu().numpy()
        err = np.max(np.abs(uu - uref)) / np.max(np.abs(uref))
        assert err <= 1e-3, (i, int(sizes[i]), err)


def compliance(asm, basm, cond, x, kappa):
    K = asm(x, element_data={"kappa": kappa})
    b = basm(x)
    K_ii, f_i = cond(K, b)
    # 3e-12: near the FP64 floor of this system's residual (|K| |u| / |b| ~ 1e4),
    # far below what the h = 1e-6 central differences resolve
    u = cond.recover(K_ii.solve(f_i, rtol=3e-12))
    return (b * u).sum()


def test_c4_adjoint_256_square():
    mesh = tg.Mesh.gen_unit_square(256, device=DEV)
    g = torch.Generator().manual_seed(11)
    kappa0 = torch.exp(torch.randn(mesh.n_elements, generator=g, dtype=torch.float64)).to(DEV)
    asm = KappaLaplace.from_mesh(mesh, quadrature_order=1)
    basm = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)
    cond = tg.Condenser(mesh.boundary_mask)
    x0 = mesh.points.clone()
    x = x0.clone().requires_grad_(True)
    kappa = kappa0.clone().requires_grad_(True)
    compliance(asm, basm, cond, x, kappa).backward()
    gk, gx = kappa.grad, x.grad
    interior = ~mesh.boundary_mask
    h = 1e-6
    errs_k, errs_x = [], []
    with torch.no_grad():
        for _ in range(64):
            d = torch.randn(mesh.n_elements, generator=g, dtype=torch.float64).to(DEV)
            fd = (compliance(asm, basm, cond, x0, kappa0 + h * d) - compliance(asm, basm, cond, x0, kappa0 - h * d)) / (2 * h)
            errs_k.append(abs(float(fd - (gk * d).sum())) / float((gk * d).abs().sum()))
            dx = torch.randn(x0.shape, generator=g, dtype=torch.float64).to(DEV) * interior[:, None]
            fd = (compliance(asm, basm, cond, x0 + h * dx, kappa0) - compliance(asm, basm, cond, x0 - h * dx, kappa0)) / (2 * h)
            errs_x.append(abs(float(fd - (gx * dx).sum())) / float((gx * dx).abs().sum()))
    assert max(errs_k) <= 1e-5, max(errs_k)
    assert max(errs_x) <= 1e-5, max(errs_x)
