"""Train the learned preconditioner's message-passing network on the GPU.

    python -m tensormesh_gb300.train_learned --systems 2000 --n 32 --out weights.npz

Each training system is a 3D P1 Poisson problem on an n^3 Kuhn cube, with
log kappa piecewise constant on 8^3 blocks, each block N(0, 2^2), zero
Dirichlet on all faces and f = 1: the generator of the 128^3 benchmark
configuration at a smaller size, with fresh seeds.  Residual/error pairs come
from the preconditioner's own flexible-PCG iterates (two-level method with
unit smoother weights) on each system (``learned.generate_pairs``), and the
network that sets the smoother weights is trained with the project's own
forward/backward kernels (``learned.train``).  The weights are written as an
.npz of float32 arrays.
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
    log = []
    losses = train(pre, systems, epochs=args.epochs, lr=args.lr,
                   log=lambda ep, l: log.append((ep, l)) or print(f"epoch {ep}: mean loss {l:.4f}", flush=True))
    t_train = time.perf_counter() - t0 - t_data
    n_pairs = sum(len(pr) for _, _, pr in systems)
    meta = dict(systems=args.systems, n=args.n, epochs=args.epochs, lr=args.lr, coarse=args.coarse,
                iterations=list(its), pairs=n_pairs, data_seconds=t_data, train_seconds=t_train,
                first_epoch_loss=log[0][1] if log else None, last_epoch_loss=log[-1][1] if log else None)
    save_weights(pre.model, args.out, meta)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
