"""Learned preconditioner: the MPNN's hand-written BF16 tensor-core forward
and backward kernels against a plain PyTorch float32 reference of the same
network on the CPU (same bf16 rounding points), and what the trained network
gains inside flexible PCG over the same method without it."""
import math

import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300.learned import MPNN, Graph, LearnedPreconditioner, generate_pairs, train

pytestmark = pytest.mark.gpu
DEV = "cuda"


def poisson_system(n, seed, device=DEV, blocks=4):
    mesh = tg.Mesh.gen_unit_cube(n, device=device)
    g = torch.Generator().manual_seed(seed)
    logk = torch.randn(blocks, blocks, blocks, generator=g, dtype=torch.float64) * 2.0
    c = torch.arange(n ** 3)
    i, j, k = c % n, (c // n) % n, c // (n * n)
    s = n // blocks
    kappa = torch.exp(logk[k // s, j // s, i // s]).repeat_interleave(6).to(device)

    class KL(tg.ElementAssembler):
        def forward(self, gradu, gradv, kappa):
            return kappa * (gradu @ gradv)
    K = KL.from_mesh(mesh, quadrature_order=1)(mesh.points, element_data={"kappa": kappa})
    b = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)(mesh.points)
    cond = tg.Condenser(mesh.boundary_mask)
    K_ii, f_i = cond(K, b)
    coords = mesh.points[~mesh.boundary_mask]
    return K_ii, f_i, coords


def bf(t):
    return t.to(torch.bfloat16).float()


def reference_forward(params, G, x):
    """float32 torch restatement of the network with the kernels' bf16
    rounding points (features and weights in bf16, accumulation in fp32)."""
    n = G.n
    A = torch.sparse_csr_tensor(G.indptr.cpu(), G.indices.cpu().long(), G.aoff.cpu(), (n, n))
    w = params["w_in"].cpu()
    ax = A @ x
    H = bf(torch.relu(x[:, None] * w[0] + ax[:, None] * w[1] + w[2]))
    L = sum(1 for k in params if k.startswith("W"))
    for l in range(L):
        AH = bf(A @ H)
        Z = torch.cat([H, AH], 1) @ bf(params[f"W{l}"].cpu()) + params[f"b{l}"].cpu()
        H = bf(torch.relu(Z))
    wr = params["wr"].cpu()
    return H @ wr[:64] + A @ (H @ wr[64:])


def test_mpnn_forward_matches_torch_reference():
    K, f, coords = poisson_system(8, 0)
    G = Graph(K.indptr, K.indices, K.values)
    model = MPNN(DEV, seed=1)
    x = torch.randn(G.n, generator=torch.Generator().manual_seed(2)).to(DEV)
    y = model.forward(G, x).cpu()
    ref = reference_forward(model.params, G, x.cpu())
    rel = float((y - ref).norm() / ref.norm())
    assert rel <= 2e-2, rel


def test_mpnn_backward_matches_torch_autograd():
    K, f, coords = poisson_system(8, 1)
    G = Graph(K.indptr, K.indices, K.values)
    model = MPNN(DEV, seed=3)
    x = torch.randn(G.n, generator=torch.Generator().manual_seed(4)).to(DEV)
    gy = torch.randn(G.n, generator=torch.Generator().manual_seed(5)).to(DEV)
    y, saved = model.forward(G, x, keep=True)
    grads = model.backward(G, saved, gy)
    params = {k: v.detach().cpu().clone().requires_grad_(True) for k, v in model.params.items()}
    ref = reference_forward(params, G, x.cpu())
    (ref * gy.cpu()).sum().backward()
    for k, p in params.items():
        got = grads[k].cpu().reshape(p.shape)
        want = p.grad
        cos = float(torch.nn.functional.cosine_similarity(got.reshape(1, -1), want.reshape(1, -1)))
        rel = float((got - want).norm() / want.norm())
        assert cos >= 0.999 and rel <= 5e-2, (k, cos, rel)


def test_two_level_preconditioner_is_symmetric_positive():
    K, f, coords = poisson_system(12, 7)
    pre = LearnedPreconditioner(MPNN(DEV, seed=2), coarse_target=64)
    pre.setup(K, coords)
    g = torch.Generator().manual_seed(8)
    u = torch.randn(f.shape[0], generator=g, dtype=torch.float64).to(DEV)
    v = torch.randn(f.shape[0], generator=g, dtype=torch.float64).to(DEV)
    uMv, vMu = float(torch.dot(u, pre(v))), float(torch.dot(v, pre(u)))
    assert abs(uMv - vMu) <= 1e-5 * (abs(uMv) + abs(vMu)), (uMv, vMu)
    assert float(torch.dot(u, pre(u))) > 0


def test_two_level_apply_matches_a_torch_restatement():
    """tm_twolevel_apply against the same operator written in torch float32,
    with the coarse inverse as the kernels hold it (D H D, H in half
    precision): y_c = K_c^-1 P^T r, s = S (r - K P y_c),
    y_c2 = K_c^-1 P^T K s, z = P (y_c - y_c2) + s."""
    K, f, coords = poisson_system(12, 4)
    pre = LearnedPreconditioner(MPNN(DEV, seed=3), coarse_target=64)
    pre.setup(K, coords)
    C = pre.coarse
    n = f.shape[0]
    g = torch.Generator().manual_seed(11)
    r = torch.randn(n, generator=g, dtype=torch.float64).to(DEV)
    z = pre(r)
    Kc = C.kc_scale[:, None] * C.kc_half.float() * C.kc_scale[None, :]

    def coarse(v):
        return Kc @ torch.zeros(C.nc, dtype=torch.float32, device=DEV).index_add_(0, C.agg, v.float())
    kp = torch.sparse_csr_tensor(C.kp_indptr, C.kp_indices.long(), C.kp_values32, (n, C.nc))
    Kf = torch.sparse_csr_tensor(K.indptr, K.indices.long(), K.values.float(), (n, n))
    yc = coarse(r)
    s1 = pre.sw.float() * (r.float() - kp @ yc)
    yc2 = coarse(Kf @ s1)
    ref = (yc - yc2)[C.agg] + s1
    assert float((z.float() - ref).abs().max() / ref.abs().max()) <= 1e-4
    # the half-precision H is the symmetric unit-diagonal form of the float32 inverse
    H = C.kc_half.float()
    assert torch.equal(H, H.T)
    assert float((torch.diagonal(H) - 1).abs().max()) <= 1e-3
    assert float((Kc - C.Kc_inv).abs().max() / C.Kc_inv.abs().max()) <= 1e-3


def test_graph_replay_matches_eager_iterations():
    K, f, coords = poisson_system(12, 3)
    pre = LearnedPreconditioner(MPNN(DEV, seed=1), coarse_target=64)
    xs = []
    for graph in (False, True):
        x = torch.zeros_like(f)
        info = pre.solve(K, f, x, rtol=1e-8, coords=coords, check_every=4, graph=graph)
        assert info.status == 0 and info.residual <= 1e-8 and not info.fallback
        xs.append((x, info.iterations))
    assert xs[0][1] == xs[1][1]
    assert torch.equal(xs[0][0], xs[1][0])


def test_training_and_two_level_solve_against_jacobi_pcg():
    torch.manual_seed(0)
    systems = generate_pairs([poisson_system(12, s) for s in range(6)], iterations=(1, 3, 8), coarse_target=64)
    model = MPNN(DEV, seed=0)
    model.params["wr"].zero_()
    pre = LearnedPreconditioner(model, coarse_target=64)
    losses = train(pre, systems, epochs=3, lr=3e-3)
    assert len(losses) == 3 * len(systems) and all(math.isfinite(v) for v in losses)
    # the proxy is log(lambda_max / lambda_min) up to the sampling: positive
    assert all(v > 0.0 for v in losses)
    K, f, coords = poisson_system(16, 99)
    K.solve(f, rtol=1e-8)
    jac_its = K.last_solve_info.iterations
    for use in (True, False):
        x = torch.zeros_like(f)
        info = LearnedPreconditioner(pre.model, coarse_target=64, use_network=use).solve(K, f, x, rtol=1e-8,
                                                                                       coords=coords)
        assert info.status == 0 and info.residual <= 1e-8 and not info.fallback
        assert info.iterations < jac_its, (use, info.iterations, jac_its)


def test_solve_hook_and_adjoint_with_two_level_preconditioner():
    """K.solve(..., preconditioner=pre) in the forward and the adjoint solve:
    the compliance and its kappa-gradient agree with the Jacobi-PCG ones."""
    mesh = tg.Mesh.gen_unit_square(48, device=DEV)
    g = torch.Generator().manual_seed(4)
    kappa0 = torch.exp(torch.randn(mesh.n_elements, generator=g, dtype=torch.float64)).to(DEV)

    class KL(tg.ElementAssembler):
        def forward(self, gradu, gradv, kappa):
            return kappa * (gradu @ gradv)
    asm = KL.from_mesh(mesh, quadrature_order=1)
    load = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)
    cond = tg.Condenser(mesh.boundary_mask)
    pre = LearnedPreconditioner(None, coarse_target=64, use_network=False,
                                coords=mesh.points[~mesh.boundary_mask].contiguous())
    out = []
    for kw in ({}, {"preconditioner": pre}):
        kappa = kappa0.clone().requires_grad_(True)
        K = asm(mesh.points, element_data={"kappa": kappa})
        b = load(mesh.points)
        K_ii, f_i = cond(K, b)
        J = (b * cond.recover(K_ii.solve(f_i, rtol=1e-12, **kw))).sum()
        J.backward()
        out.append((float(J.detach()), kappa.grad.clone()))
    assert abs(out[0][0] - out[1][0]) <= 1e-10 * abs(out[0][0])
    assert float((out[0][1] - out[1][1]).abs().max()) <= 1e-8 * float(out[0][1].abs().max())


def test_fused_flexible_cg_matches_the_torch_iteration():
    """tm_fcg_twolevel_iterations (fused vector updates, device scalars)
    against a torch restatement of the same iteration: q = K p,
    alpha = rz / (p, q), x += alpha p, r -= alpha q, z = M r,
    beta = max(0, -alpha (z, q) / rz), rz = (r, z), p = z + beta p."""
    K, f, coords = poisson_system(12, 5)
    pre = LearnedPreconditioner(MPNN(DEV, seed=1), coarse_target=64)
    pre.setup(K, coords)
    x = torch.zeros_like(f)
    r = f.clone()
    z = pre(r)
    p = z.clone()
    rz = torch.dot(r, z)
    xr, rr, pr, rzr = x.clone(), r.clone(), p.clone(), rz.clone()
    pre._iterate(x, r, p, rz, 6)
    for _ in range(6):
        q = pre._K(pr)
        alpha = rzr / torch.dot(pr, q)
        xr += alpha * pr
        rr -= alpha * q
        zr = pre(rr)
        beta = torch.clamp(-alpha * torch.dot(zr, q) / rzr, min=0.0)
        rzr = torch.dot(rr, zr)
        pr = zr + beta * pr
    assert float((x - xr).abs().max() / xr.abs().max()) <= 1e-10
    assert float((r - rr).abs().max() / rr.abs().max()) <= 1e-8
    assert abs(float(rz) - float(rzr)) <= 1e-9 * abs(float(rzr))


def test_kp_kernels_match_a_sorted_torch_construction():
    """tm_kp_count / tm_kp_fill give K P exactly as the sort-based
    construction: per row, aggregates ascending, each sum in CSR order."""
    from tensormesh_gb300.learned import CoarseSpace
    K, f, coords = poisson_system(12, 2)
    C = CoarseSpace(K.indptr, K.indices, K.values, coords, target=32)
    n = K.shape[0]
    rows = torch.repeat_interleave(torch.arange(n, device=DEV), K.indptr[1:] - K.indptr[:-1])
    key = rows * C.nc + C.agg[K.indices.long()]
    order = torch.argsort(key, stable=True)
    uniq, counts = torch.unique_consecutive(key[order], return_counts=True)
    vals = K.values.double()[order].cpu().numpy()
    ends = np.cumsum(counts.cpu().numpy())
    starts = ends - counts.cpu().numpy()
    ref = np.array([np.sum(vals[a:b]) if b - a == 1 else float(np.add.reduce(vals[a:b])) for a, b in zip(starts, ends)])
    kp_rows = torch.div(uniq, C.nc, rounding_mode="floor")
    np.testing.assert_array_equal(C.kp_indices.cpu().numpy(), (uniq - kp_rows * C.nc).cpu().numpy())
    ip = torch.zeros(n + 1, dtype=torch.int64, device=DEV)
    ip[1:] = torch.cumsum(torch.bincount(kp_rows, minlength=n), 0)
    assert torch.equal(C.kp_indptr, ip)
    assert np.max(np.abs(C.kp_values.cpu().numpy() - ref)) <= 1e-14 * np.max(np.abs(ref))
