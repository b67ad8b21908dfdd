"""Batched persistent launch: many uneven 2D P1 Poisson meshes assembled
(float32) and Jacobi-PCG-solved in one launch, replayed from a CUDA graph;
checked per instance against the float64 oracle."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from oracle import fem
from tensormesh_gb300.batched import BatchedPoisson

pytestmark = pytest.mark.gpu
DEV = "cuda"


def make_batch(sizes, seed=0):
    meshes = [tg.Mesh.gen_unit_square(int(n), device=DEV) for n in sizes]
    g = torch.Generator().manual_seed(seed)
    kappas = [torch.exp(torch.randn(m.n_elements, generator=g, dtype=torch.float64)) for m in meshes]
    return meshes, kappas


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("cluster,big", [(1, None), (4, None), (2, (8, 2)), (2, (16, 1))])
def test_batched_matches_fp64_oracle(graph, cluster, big, tmp_path, monkeypatch):
    """big = (cluster_big, n_big): the largest instances run in a second,
    concurrent launch on larger clusters."""
    monkeypatch.setenv("TM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    sizes = [5, 17, 32, 9, 24, 3]
    meshes, kappas = make_batch(sizes)
    cb, nbig = big if big else (None, 0)
    bp = BatchedPoisson(meshes, cluster=cluster, cluster_big=cb, n_big=nbig)
    assert bp.config["n_big"] == nbig
    k = torch.cat(kappas).to(DEV)
    u, info = bp(k, rtol=1e-6, graph=graph)
    torch.cuda.synchronize()
    assert info.status.cpu().tolist() == [0] * len(sizes)
    vals = bp.values.double().cpu().numpy()
    ip = bp.pattern.indptr.cpu().numpy()
    for i, m in enumerate(meshes):
        pts, el = m.points.cpu().numpy(), m.cells["triangle"].cpu().numpy()
        oip, oix, odv = fem.assemble_csr(pts, el, "triangle", "laplace", 1, coef=kappas[i].numpy())
        r0, r1 = bp.node_ptr[i], bp.node_ptr[i + 1]
        got = vals[ip[r0]:ip[r1]]
        assert np.max(np.abs(got - odv)) <= 1e-5 * np.max(np.abs(odv))
        bref = fem.assemble_load(pts, el, "triangle", 1, "const", 1.0)
        bd = m.boundary_mask.cpu().numpy()
        iptr, iind, ival, fi = fem.condense(oip, oix, odv, bd, None, bref)
        if iptr.shape[0] > 1:
            uref = fem.recover(fem.spsolve(iptr, iind, ival, fi), bd)
            uu = u[r0:r1].double().cpu().numpy()
            assert np.max(np.abs(uu - uref)) <= 5e-4 * np.max(np.abs(uref))


@pytest.mark.parametrize("big", [None, (8, 1)])
def test_batched_graph_replay_is_deterministic(big, tmp_path, monkeypatch):
    monkeypatch.setenv("TM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    meshes, kappas = make_batch([12, 30, 7, 20], seed=1)
    cb, nbig = big if big else (None, 0)
    bp = BatchedPoisson(meshes, cluster=2, cluster_big=cb, n_big=nbig)
    k = torch.cat(kappas).to(DEV)
    u1, _ = bp(k)
    a = u1.clone()
    for _ in range(3):
        u2, _ = bp(k)
        assert torch.equal(u2, a)


def test_autotuner_picks_and_caches(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("TM_AUTOTUNE_CACHE", str(path))
    meshes, kappas = make_batch([10, 40, 25], seed=2)
    bp = BatchedPoisson(meshes)
    k = torch.cat(kappas).to(DEV)
    best = bp.autotune(k, clusters=(1, 2, 4), budgets=(512, 2048), reps=2, big=((None, 0), (8, 1)))
    assert best["cluster"] in (1, 2, 4) and best["slot_budget"] in (512, 2048)
    assert len(best["candidates"]) == 12
    assert path.exists()
    bp2 = BatchedPoisson(meshes)
    again = bp2.autotune(k, clusters=(1, 2, 4), budgets=(512, 2048), big=((None, 0), (8, 1)))
    assert again["cluster"] == best["cluster"] and bp2.config["slot_budget"] == best["slot_budget"]
    assert bp2.config["n_big"] == best["n_big"]
    u, info = bp2(k)
    assert int(info.status.max()) == 0
