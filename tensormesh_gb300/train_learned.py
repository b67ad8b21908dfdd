"""Train the learned preconditioner's message-passing network on the GPU.

    python -m tensormesh_gb300.train_learned --systems 500 --epochs 4 --lr 5e-4 --n 32 --out weights.npz

Each training system is a 3D P1 Poisson problem on an n^3 Kuhn cube, with
log kappa piecewise constant on 8^3 blocks, each block N(0, 2^2), zero
Dirichlet on all faces and f = 1: the generator of the 128^3 benchmark
configuration at a smaller size, with fresh seeds.  Residual/error pairs come
from the preconditioner's own flexible-PCG iterates (two-level method with
unit smoother weights) on each system (``learned.generate_pairs``), and the
network that sets the smoother weights is trained with the project's own
forward/backward kernels (``learned.train``).  After every epoch the network
is scored by the mean flexible-PCG iteration count on held-out systems of the
same generator; the best checkpoint is kept, the untrained network (weights
w = 1, the method without learning) being checkpoint 0.  The weights are
written as an .npz of float32 arrays, the selection record in its metadata.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300.learned import MPNN, LearnedPreconditioner, generate_pairs, train


class _KappaLaplace(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * (gradu @ gradv)


def block_log_kappa(n: int, blocks: int, rng: np.random.Generator) -> np.ndarray:
    g = rng.normal(0.0, 2.0, size=(blocks, blocks, blocks))
    c = np.arange(n ** 3)
    i, j, k = c % n, (c // n) % n, c // (n * n)
    s = max(1, n // blocks)
    return np.repeat(g[np.minimum(k // s, blocks - 1), np.minimum(j // s, blocks - 1),
                       np.minimum(i // s, blocks - 1)], 6)


class PoissonFamily:
    """Systems of the benchmark generator on one mesh (one topology, new kappa)."""

    def __init__(self, n: int, device="cuda", blocks: int = 8):
        self.mesh = tg.Mesh.gen_unit_cube(n, device=device)
        self.asm = _KappaLaplace.from_mesh(self.mesh, quadrature_order=1)
        self.b = tg.const_node_assembler(1.0).from_mesh(self.mesh, quadrature_order=1)(self.mesh.points)
        self.cond = tg.Condenser(self.mesh.boundary_mask)
        self.coords = self.mesh.points[~self.mesh.boundary_mask].contiguous()
        self.n, self.blocks, self.device = n, blocks, device

    def system(self, seed: int):
        rng = np.random.default_rng(seed)
        kappa = torch.from_numpy(np.exp(block_log_kappa(self.n, self.blocks, rng))).to(self.device)
        K = self.asm(self.mesh.points, element_data={"kappa": kappa})
        K_ii, f_i = self.cond(K, self.b)
        return K_ii, f_i, self.coords


def save_weights(model: MPNN, path: str, meta: dict):
    arrays = {k: v.detach().float().cpu().numpy() for k, v in model.params.items()}
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez(path, **arrays)


def load_weights(path: str, device="cuda") -> MPNN:
    z = np.load(path)
    model = MPNN(device)
    model.load_state_dict({k: torch.from_numpy(z[k]) for k in z.files if k != "meta"})
    return model


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=2000)
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--epochs", type=int, default=2)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--coarse", type=int, default=512, help="dofs per coarse aggregate")
    ap.add_argument("--iterations", default="1,3,8,20", help="flexible-PCG iteration counts of the pairs")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--val", type=int, default=4, help="held-out systems for checkpoint selection")
    ap.add_argument("--out", required=True)
    args = ap.parse_args()
    torch.cuda.set_device(0)
    fam = PoissonFamily(args.n)
    t0 = time.perf_counter()
    its = tuple(int(c) for c in args.iterations.split(","))
    systems = []
    for s in range(args.systems):
        systems += generate_pairs([fam.system(10_000 + s)], iterations=its, coarse_target=args.coarse)
    t_data = time.perf_counter() - t0
    model = MPNN("cuda", seed=args.seed)
    model.params["wr"].zero_()          # start from w = 1 (the method without the network)
    pre = LearnedPreconditioner(model, coarse_target=args.coarse)
    val = [fam.system(90_000 + s) for s in range(args.val)]

    def val_iterations() -> float:
        its = []
        for A, b, coords in val:
            p = LearnedPreconditioner(model, coarse_target=args.coarse)
            its.append(p.solve(A, b, torch.zeros_like(b), rtol=1e-8, coords=coords, check_every=1).iterations)
        return float(np.mean(its))

    # checkpoint selection on the solver's own metric: flexible-PCG iterations
    # on held-out systems; the initial network (w = 1) is checkpoint 0
    history = [(0, val_iterations(), None)]
    best = (history[0][1], {k: v.clone() for k, v in model.params.items()})
    log = []
    for ep in range(args.epochs):
        train(pre, systems, epochs=1, lr=args.lr, seed=args.seed + ep,
              log=lambda _, l: log.append((ep, l)) or print(f"epoch {ep}: mean loss {l:.4f}", flush=True))
        v = val_iterations()
        history.append((ep + 1, v, log[-1][1] if log else None))
        print(f"epoch {ep}: validation iterations {v:.1f}", flush=True)
        if v < best[0]:
            best = (v, {k: t.clone() for k, t in model.params.items()})
    for k, t in best[1].items():
        model.params[k].copy_(t)
    model.invalidate()
    t_train = time.perf_counter() - t0 - t_data
    n_pairs = sum(len(pr) for _, _, pr in systems)
    meta = dict(systems=args.systems, n=args.n, epochs=args.epochs, lr=args.lr, coarse=args.coarse,
                iterations=list(its), pairs=n_pairs, data_seconds=t_data, train_seconds=t_train,
                validation=[dict(checkpoint=c, mean_iterations=v, train_loss=l) for c, v, l in history],
                selected_validation_iterations=best[0])
    save_weights(pre.model, args.out, meta)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
