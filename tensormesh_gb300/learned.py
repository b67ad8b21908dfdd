"""Learned preconditioner: a mesh-graph message-passing network (MPNN) used
inside flexible PCG, with Jacobi-PCG as fallback and judge.

Architecture (hidden width 64, BF16 weights and activations on the tensor
cores, FP32 accumulation -- kernels in csrc/mpnn.cu):
  * graph = the condensed stiffness K_ii; edge weights a_ij =
    K_ij / sqrt(K_ii K_jj) (off-diagonal, symmetric);
  * input  x = D^-1/2 r / s, s = ||D^-1/2 r|| / sqrt(n)  (scale-equivariant);
  * 4 message-passing layers: a lift H0 = relu(x w0 + (A x) w1 + b0) and
    three hidden layers H = relu(H W_s + (A H) W_n + b);
  * a message-passing readout y = H wr0 + A (H wr1); the correction is
    z = s D^-1/2 y.

The network is the smoother of a two-level preconditioner: a coarse
correction on node aggregates (piecewise-constant prolongation P over an
RCB partition of the dofs, K_c = P^T K P inverted once) removes the smooth
error a local network cannot see, then the MPNN corrects the rest:
    z_c = P K_c^-1 P^T r ;  z = z_c + MPNN(r - K z_c) ;  z += P K_c^-1 P^T (r - K z).
It is trained on residual/error pairs (r_k, e_k) of the plain Jacobi-PCG
iterates x_k of method-generated systems, minimising the energy norm
||z(r_k) - e_k||_K^2 / ||e_k||_K^2, with the hand-written forward and
backward kernels and Adam.  Flexible CG (Polak-Ribiere beta) tolerates the
nonlinear preconditioner; the true FP64 residual ||b - K x|| / ||b|| from
the plain SpMV decides convergence, and a stagnating solve falls back to
Jacobi-PCG.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass
from typing import Dict, List, Optional

import torch

from . import _lib
from .plan import rcb_partition_grouped
from .solve import SolveInfo, pcg_jacobi_raw, spmv_raw, true_relative_residual

F = 64


def _s(dev):
    return _lib.stream_handle(dev)


class Graph:
    """Normalised operator of one SPD CSR matrix (float32)."""

    def __init__(self, indptr, indices, values):
        self.indptr, self.indices = indptr, indices
        n = indptr.shape[0] - 1
        self.n = n
        dev = values.device
        rows = torch.repeat_interleave(torch.arange(n, device=dev), indptr[1:] - indptr[:-1])
        diag = torch.zeros(n, dtype=torch.float64, device=dev).index_put_(
            (rows[rows == indices.long()],), values.double()[rows == indices.long()])
        diag = torch.where(diag > 0, diag, torch.ones_like(diag))
        self.dinv_sqrt = (1.0 / diag.sqrt()).float().contiguous()
        a = values.double() * (1.0 / diag.sqrt())[rows] * (1.0 / diag.sqrt())[indices.long()]
        a = torch.where(rows == indices.long(), torch.zeros_like(a), a)
        self.aoff = a.float().contiguous()
        self.values32 = values.float().contiguous()


class MPNN:
    """Weights (FP32 master copies) and the kernel-driven forward/backward."""

    def __init__(self, device="cuda", seed: int = 0, n_hidden: int = 3):
        g = torch.Generator().manual_seed(seed)
        dev = torch.device(device)
        self.device = dev
        self.params: Dict[str, torch.Tensor] = {
            "w_in": torch.cat([torch.randn(2, F, generator=g) * 0.5, torch.zeros(1, F)]).to(dev),
            "wr": (torch.randn(2 * F, generator=g) * (0.1 / math.sqrt(F))).to(dev),
        }
        for l in range(n_hidden):
            self.params[f"W{l}"] = (torch.randn(2 * F, F, generator=g) * math.sqrt(1.0 / F)).to(dev)
            self.params[f"b{l}"] = torch.zeros(F, device=dev)
        self.n_hidden = n_hidden
        self._bf = None

    # BF16 copies of the weights for the kernels
    def _bf16(self):
        if self._bf is None:
            self._bf = {}
            for l in range(self.n_hidden):
                W = self.params[f"W{l}"]
                self._bf[f"Wt{l}"] = W.t().contiguous().to(torch.bfloat16)   # [64 out][128 in]
                self._bf[f"W{l}"] = W.contiguous().to(torch.bfloat16)       # [128 in][64 out]
        return self._bf

    def invalidate(self):
        self._bf = None

    def forward(self, G: Graph, x: torch.Tensor, keep: bool = False):
        """y = MPNN(x) (float32 [n]); with keep=True also returns the
        activations needed by backward."""
        n, dev = G.n, x.device
        bf = self._bf16()
        s = _s(dev)
        H = torch.empty(n, F, dtype=torch.bfloat16, device=dev)
        ax = torch.empty(n, dtype=torch.float32, device=dev)
        _lib.call("tm_mpnn_input_fwd", n, G.indptr.data_ptr(), G.indices.data_ptr(), G.aoff.data_ptr(),
                  x.data_ptr(), self.params["w_in"].data_ptr(), H.data_ptr(), ax.data_ptr(), s)
        acts = [H]
        for l in range(self.n_hidden):
            Hn = torch.empty(n, F, dtype=torch.bfloat16, device=dev)
            _lib.call("tm_mpnn_layer_fwd", n, G.indptr.data_ptr(), G.indices.data_ptr(), G.aoff.data_ptr(),
                      acts[-1].data_ptr(), bf[f"Wt{l}"].data_ptr(), self.params[f"b{l}"].data_ptr(), Hn.data_ptr(),
                      1, s)
            acts.append(Hn)
            if not keep and len(acts) > 2:
                acts[-2] = None
        u = torch.empty(n, dtype=torch.float32, device=dev)
        t = torch.empty(n, dtype=torch.float32, device=dev)
        y = torch.empty(n, dtype=torch.float32, device=dev)
        _lib.call("tm_mpnn_readout_fwd", n, G.indptr.data_ptr(), G.indices.data_ptr(), G.aoff.data_ptr(),
                  acts[-1].data_ptr(), self.params["wr"].data_ptr(), 0, u.data_ptr(), t.data_ptr(), y.data_ptr(), s)
        if keep:
            return y, (x, ax, acts)
        return y

    def backward(self, G: Graph, saved, gy: torch.Tensor) -> Dict[str, torch.Tensor]:
        x, ax, acts = saved
        n, dev = G.n, gy.device
        bf = self._bf16()
        s = _s(dev)
        tiles = (n + 63) // 64
        grads = {}
        dH = torch.empty(n, F, dtype=torch.float32, device=dev)
        part = torch.empty(tiles * 3 * F, dtype=torch.float32, device=dev)
        dwr = torch.empty(2 * F, dtype=torch.float32, device=dev)
        gy = gy.float().contiguous()
        _lib.call("tm_mpnn_readout_bwd", n, G.indptr.data_ptr(), G.indices.data_ptr(), G.aoff.data_ptr(),
                  acts[-1].data_ptr(), gy.data_ptr(), self.params["wr"].data_ptr(), dH.data_ptr(), part.data_ptr(),
                  dwr.data_ptr(), s)
        grads["wr"] = dwr
        part_dW = torch.empty(tiles * 2 * F * F, dtype=torch.float32, device=dev)
        part_db = torch.empty(tiles * F, dtype=torch.float32, device=dev)
        U = torch.empty(n, F, dtype=torch.float32, device=dev)
        T = torch.empty(n, F, dtype=torch.float32, device=dev)
        for l in reversed(range(self.n_hidden)):
            dW = torch.empty(2 * F, F, dtype=torch.float32, device=dev)
            db = torch.empty(F, dtype=torch.float32, device=dev)
            dHin = torch.empty(n, F, dtype=torch.float32, device=dev)
            _lib.call("tm_mpnn_layer_bwd", n, G.indptr.data_ptr(), G.indices.data_ptr(), G.aoff.data_ptr(),
                      acts[l].data_ptr(), acts[l + 1].data_ptr(), dH.data_ptr(), bf[f"W{l}"].data_ptr(), 1,
                      part_dW.data_ptr(), part_db.data_ptr(), U.data_ptr(), T.data_ptr(), dHin.data_ptr(),
                      dW.data_ptr(), db.data_ptr(), s)
            grads[f"W{l}"], grads[f"b{l}"] = dW, db
            dH = dHin
        dw = torch.empty(3 * F, dtype=torch.float32, device=dev)
        _lib.call("tm_mpnn_input_bwd", n, x.data_ptr(), ax.data_ptr(), acts[0].data_ptr(), dH.data_ptr(),
                  part.data_ptr(), dw.data_ptr(), s)
        grads["w_in"] = dw.view(3, F)
        return grads

    def state_dict(self):
        return {k: v.detach().cpu().clone() for k, v in self.params.items()}

    def load_state_dict(self, sd):
        for k, v in sd.items():
            self.params[k] = v.to(self.device).float().contiguous()
        self.invalidate()


class CoarseSpace:
    """Piecewise-constant aggregation of the dofs into RCB parts; K_c =
    P^T K P is formed once (deterministic segmented sums) and inverted once."""

    def __init__(self, indptr, indices, values, coords, target: int = 512):
        dev = values.device
        n = indptr.shape[0] - 1
        deg = torch.ones(n, dtype=torch.int64, device=dev)
        agg = rcb_partition_grouped(coords, torch.zeros(n, dtype=torch.int64, device=dev), deg, float(target), target)
        self.agg = agg
        nc = int(agg.max()) + 1
        self.nc = nc
        rows = torch.repeat_interleave(torch.arange(n, device=dev), indptr[1:] - indptr[:-1])
        key = agg[rows] * nc + agg[indices.long()]
        order = torch.argsort(key, stable=True)
        k_sorted = key[order]
        uniq, counts = torch.unique_consecutive(k_sorted, return_counts=True)
        ptr = torch.zeros(uniq.shape[0] + 1, dtype=torch.int64, device=dev)
        ptr[1:] = torch.cumsum(counts, 0)
        from .adjoint import segment_sum
        vals = segment_sum(ptr, order.contiguous(), values.double().contiguous(), 1)
        Kc = torch.zeros(nc * nc, dtype=torch.float64, device=dev)
        Kc[uniq] = vals
        Kc = Kc.view(nc, nc)
        self.Kc_inv = torch.linalg.inv(Kc).contiguous()
        self.agg_order = torch.argsort(agg, stable=True)
        self.agg_ptr = torch.zeros(nc + 1, dtype=torch.int64, device=dev)
        self.agg_ptr[1:] = torch.cumsum(torch.bincount(agg, minlength=nc), 0)

    def apply(self, r: torch.Tensor) -> torch.Tensor:
        """P K_c^-1 P^T r."""
        from .adjoint import segment_sum
        rc = segment_sum(self.agg_ptr, self.agg_order, r.double().contiguous(), 1)
        zc = self.Kc_inv @ rc
        return zc[self.agg].to(r.dtype)


@dataclass
class LearnedSolveInfo(SolveInfo):
    preconditioner: str = "learned"
    fallback: bool = False
    seconds: float = 0.0


class LearnedPreconditioner:
    """Two-level preconditioner with an MPNN smoother, for flexible PCG."""

    def __init__(self, model: Optional[MPNN] = None, device="cuda", coarse_target: int = 512,
                 use_network: bool = True):
        self.model = model or MPNN(device)
        self.coarse_target = coarse_target
        self.use_network = use_network
        self._setup_key = None

    def setup(self, A, coords):
        key = (A.values.data_ptr(), A.values._version, A.nnz)
        if key == self._setup_key:
            return
        self.A = A
        self.G = Graph(A.indptr, A.indices, A.values.detach())
        self.coarse = CoarseSpace(A.indptr, A.indices, A.values.detach(), coords, self.coarse_target)
        self._setup_key = key

    def _K(self, v):
        return spmv_raw(self.A.indptr, self.A.indices, self.A.values, v.to(self.A.dtype).contiguous())

    def smoother(self, r: torch.Tensor) -> torch.Tensor:
        G = self.G
        if not self.use_network:
            return (G.dinv_sqrt.to(r.dtype) ** 2) * r
        xs = G.dinv_sqrt * r.float()
        sc = float(torch.linalg.vector_norm(xs)) / math.sqrt(max(1, G.n))
        if sc == 0.0:
            return torch.zeros_like(r)
        y = self.model.forward(G, (xs / sc).contiguous())
        return (sc * G.dinv_sqrt * y).to(r.dtype)

    def __call__(self, r: torch.Tensor) -> torch.Tensor:
        zc = self.coarse.apply(r)
        z = zc + self.smoother(r - self._K(zc))
        return z + self.coarse.apply(r - self._K(z))

    # -- flexible PCG ------------------------------------------------------------
    def solve(self, A, b, x, rtol=1e-8, atol=0.0, maxiter=10000, coords=None, check_every: int = 1):
        """Flexible CG (Polak-Ribiere) with this preconditioner; falls back to
        Jacobi-PCG if the residual stagnates.  x is updated in place."""
        if coords is None:
            raise ValueError("the learned preconditioner needs dof coordinates (coords=) for its coarse space")
        t0 = time.perf_counter()
        self.setup(A, coords)
        bn = float(torch.linalg.vector_norm(b.double()))
        tol = max(rtol * bn, atol)
        r = b - self._K(x)
        z = self(r)
        p = z.clone()
        rz = float(torch.dot(r.double(), z.double()))
        it = 0
        best = float("inf")
        stall = 0
        status = _lib.TM_ERR_MAXITER
        while it < maxiter:
            rn = float(torch.linalg.vector_norm(r.double()))
            if rn <= tol:
                status = _lib.TM_OK
                break
            best, stall = (rn, 0) if rn < 0.999 * best else (best, stall + 1)
            if stall > 50:
                break
            q = self._K(p)
            pq = float(torch.dot(p.double(), q.double()))
            if not pq > 0:
                status = _lib.TM_ERR_BREAKDOWN
                break
            alpha = rz / pq
            x += alpha * p
            r_old = r
            r = r - alpha * q
            z_new = self(r)
            beta = float(torch.dot(z_new.double(), (r - r_old).double())) / rz
            rz = float(torch.dot(r.double(), z_new.double()))
            p = z_new + max(beta, 0.0) * p
            it += 1
        true_res = true_relative_residual(A.indptr, A.indices, A.values, b, x, bn)
        fallback = False
        if status != _lib.TM_OK or true_res > rtol * 1.0000001:
            fb = pcg_jacobi_raw(A.indptr, A.indices, A.values.contiguous(), b, x, rtol, atol, maxiter)
            it += fb.iterations
            status, true_res, fallback = fb.status, fb.residual, True
        return LearnedSolveInfo(status, it, true_res, true_res, 0, "learned", fallback, time.perf_counter() - t0)


# -- training --------------------------------------------------------------------
def generate_pairs(systems, checkpoints=(1, 4, 16, 64), rtol=1e-10):
    """Residual/error pairs of plain Jacobi-PCG iterates.

    systems: iterable of (A, b, coords).  For each, the converged solution x*
    comes from Jacobi-PCG to ``rtol``; then the solver is re-run with an
    iteration cap k for each checkpoint, giving x_k, e_k = x* - x_k and
    r_k = b - A x_k."""
    pairs = []
    for A, b, coords in systems:
        xs = torch.zeros_like(b)
        pcg_jacobi_raw(A.indptr, A.indices, A.values, b, xs, rtol, 0.0, 100000)
        for k in checkpoints:
            xk = torch.zeros_like(b)
            pcg_jacobi_raw(A.indptr, A.indices, A.values, b, xk, 1e-30, 0.0, k, max_restarts=0)
            e = (xs - xk).float()
            r = (b - spmv_raw(A.indptr, A.indices, A.values, xk)).float()
            pairs.append((A, coords, r, e))
    return pairs


class Adam:
    def __init__(self, params: Dict[str, torch.Tensor], lr=2e-3, betas=(0.9, 0.999), eps=1e-8):
        self.p, self.lr, self.b1, self.b2, self.eps = params, lr, betas[0], betas[1], eps
        self.m = {k: torch.zeros_like(v) for k, v in params.items()}
        self.v = {k: torch.zeros_like(v) for k, v in params.items()}
        self.t = 0

    def step(self, grads):
        self.t += 1
        for k, g in grads.items():
            g = g.view_as(self.p[k])
            self.m[k].mul_(self.b1).add_(g, alpha=1 - self.b1)
            self.v[k].mul_(self.b2).addcmul_(g, g, value=1 - self.b2)
            mh = self.m[k] / (1 - self.b1 ** self.t)
            vh = self.v[k] / (1 - self.b2 ** self.t)
            self.p[k] -= self.lr * mh / (vh.sqrt() + self.eps)


def train(precond: LearnedPreconditioner, pairs, epochs: int = 2, lr: float = 2e-3, log=None) -> List[float]:
    """Minimise E ||z(r) - e||_K^2 / ||e||_K^2 over the pairs, where z is the
    two-level preconditioner's output and only the network is trained."""
    model = precond.model
    opt = Adam(model.params, lr=lr)
    losses = []
    for ep in range(epochs):
        for (A, coords, r, e) in pairs:
            precond.setup(A, coords)
            G = precond.G
            A32 = G.values32
            K = lambda v: spmv_raw(A.indptr, A.indices, A32, v.contiguous())  # noqa: E731
            zc = precond.coarse.apply(r)
            r1 = r - K(zc)
            xs = G.dinv_sqrt * r1
            sc = float(torch.linalg.vector_norm(xs)) / math.sqrt(G.n)
            if sc == 0.0:
                continue
            y, saved = model.forward(G, (xs / sc).contiguous(), keep=True)
            zs = sc * G.dinv_sqrt * y
            z1 = zc + zs
            z = z1 + precond.coarse.apply(r - K(z1))
            err = z - e
            Ke = K(e)
            enorm = float(torch.dot(e, Ke))
            Kerr = K(err)
            loss = float(torch.dot(err, Kerr)) / enorm
            losses.append(loss)
            # d loss / d z = 2 K err / enorm ; z = z1 + C (r - K z1) => dz1 = (I - K C) dz (C, K symmetric)
            gz = 2.0 * Kerr / enorm
            gz1 = gz - K(precond.coarse.apply(gz))
            gy = sc * G.dinv_sqrt * gz1
            grads = model.backward(G, saved, gy)
            opt.step(grads)
            model.invalidate()
        if log is not None:
            log(ep, sum(losses[-len(pairs):]) / max(1, len(pairs)))
    return losses
