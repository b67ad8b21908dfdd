"""Learned preconditioner: a mesh-graph message-passing network (MPNN) sets
the smoother of a two-level preconditioner used inside flexible PCG, with
Jacobi-PCG as fallback; the true residual decides convergence.

Network (hidden width 64, BF16 weights and activations on the tensor cores,
FP32 accumulation -- kernels in csrc/mpnn.cu):
  * graph = the condensed stiffness K_ii; edge weights a_ij =
    K_ij / sqrt(K_ii K_jj) (off-diagonal, symmetric);
  * input: the feature 1 on every node, so the lift sees the row sums of A;
  * 4 message-passing layers: a lift H0 = relu(x w0 + (A x) w1 + b0) and
    three hidden layers H = relu(H W_s + (A H) W_n + b);
  * a message-passing readout y = H wr0 + A (H wr1).

Preconditioner: coarse correction C = P K_c^-1 P^T on node aggregates
(piecewise-constant P over Morton-curve parts of the dofs, K_c = P^T K P
inverted once) and the damped Jacobi smoother S = diag(w) D^-1 with
w = 1/2 + sigmoid(y):
    z = C r + (I - C K) S (I - K C) r.
The network runs once per matrix, at set-up; an iteration costs two SpMVs
(K and the thin K P), two coarse solves and vector updates, all on the device
without host synchronisation.  Training minimises a proxy of the condition
number of the preconditioned operator (Rayleigh quotients of errors taken
from the preconditioner's own flexible-PCG iterates against those of random
errors, see ``train``) on generated systems, with the hand-written forward
and backward kernels and Adam.  The true FP64 residual
||b - K x|| / ||b|| decides convergence, and a stagnating solve falls back to
Jacobi-PCG.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass
from typing import Dict, List, Optional

import torch

from . import _lib
from .plan import morton_parts
from .solve import SolveInfo, pcg_jacobi_raw, spmv_raw, true_relative_residual

F = 64


def _s(dev):
    return _lib.stream_handle(dev)


class Graph:
    """Normalised operator of one SPD CSR matrix (float32): D^-1 for the
    smoother and, formed on first use (the network's edge weights only),
    the off-diagonal part of D^-1/2 A D^-1/2."""

    def __init__(self, indptr, indices, values):
        self.indptr, self.indices = indptr, indices
        n = indptr.shape[0] - 1
        self.n = n
        self.device = values.device
        self._values = values
        dev = values.device
        rows = torch.repeat_interleave(torch.arange(n, device=dev), indptr[1:] - indptr[:-1])
        on_diag = rows == indices.long()
        diag = torch.zeros(n, dtype=torch.float64, device=dev).index_put_((rows[on_diag],), values.double()[on_diag])
        self._diag = torch.where(diag > 0, diag, torch.ones_like(diag))
        self.dinv = (1.0 / self._diag).contiguous()                    # FP64
        self.values32 = values.float().contiguous()
        self._aoff = None

    @property
    def aoff(self):
        if self._aoff is None:
            n, dev = self.n, self.device
            rows = torch.repeat_interleave(torch.arange(n, device=dev), self.indptr[1:] - self.indptr[:-1])
            cols = self.indices.long()
            ds = 1.0 / self._diag.sqrt()
            a = self._values.double() * ds[rows] * ds[cols]
            self._aoff = torch.where(rows == cols, torch.zeros_like(a), a).float().contiguous()
        return self._aoff


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
    """Piecewise-constant aggregation of the dofs into parts of about
    ``target`` dofs, consecutive along a Morton curve of their coordinates.  Stores P (the aggregate of each dof), K P as a CSR
    (n x n_c, a few entries per row: only rows next to an aggregate border
    have more than one), and K_c^-1 = (P^T K P)^-1, inverted once after a
    symmetric diagonal scaling (Cholesky in float32, in FP64 if float32 is not
    positive definite) and kept in float32 (the torch path) and as a
    half-precision unit-diagonal matrix with a float32 diagonal scale (the
    kernels' matvecs); the preconditioner only needs it approximately."""

    def __init__(self, indptr, indices, values, coords, target: int = 512):
        from .adjoint import segment_sum
        dev = values.device
        n = indptr.shape[0] - 1
        agg = morton_parts(coords, target)
        self.agg = agg
        nc = int(agg.max()) + 1
        self.nc = nc
        # K P: entry (i, c) = sum of K_ij over j in aggregate c, per row in
        # ascending aggregate order, each sum in CSR order (tm_kp_count /
        # tm_kp_fill: one thread per row, no global sort)
        agg32 = agg.to(torch.int32).contiguous()
        vals64 = values.double().contiguous()
        s = _s(dev)
        cnt = torch.empty(n, dtype=torch.int64, device=dev)
        _lib.call("tm_kp_count", n, indptr.data_ptr(), indices.data_ptr(), agg32.data_ptr(), cnt.data_ptr(), s)
        self.kp_indptr = torch.zeros(n + 1, dtype=torch.int64, device=dev)
        self.kp_indptr[1:] = torch.cumsum(cnt, 0)
        kp_nnz = int(self.kp_indptr[-1])
        self.kp_indices = torch.empty(kp_nnz, dtype=torch.int32, device=dev)
        kp_vals = torch.empty(kp_nnz, dtype=torch.float64, device=dev)
        _lib.call("tm_kp_fill", n, indptr.data_ptr(), indices.data_ptr(), vals64.data_ptr(), agg32.data_ptr(),
                  self.kp_indptr.data_ptr(), self.kp_indices.data_ptr(), kp_vals.data_ptr(), s)
        kp_rows = torch.repeat_interleave(torch.arange(n, device=dev), cnt)
        self.kp_values = kp_vals
        # K_c = P^T (K P): sum the rows of K P by aggregate
        key2 = agg[kp_rows] * nc + self.kp_indices.long()
        order2 = torch.argsort(key2, stable=True)
        uniq2, counts2 = torch.unique_consecutive(key2[order2], return_counts=True)
        ptr2 = torch.zeros(uniq2.shape[0] + 1, dtype=torch.int64, device=dev)
        ptr2[1:] = torch.cumsum(counts2, 0)
        kc_vals = segment_sum(ptr2, order2.contiguous(), kp_vals, 1)
        Kc = torch.zeros(nc * nc, dtype=torch.float64, device=dev)
        Kc[uniq2] = kc_vals
        Kc = Kc.view(nc, nc)
        s = 1.0 / torch.sqrt(torch.clamp(torch.diagonal(Kc), min=torch.finfo(torch.float64).tiny))
        Ks = Kc * s[:, None] * s[None, :]                  # unit diagonal
        L, info = torch.linalg.cholesky_ex(Ks.float())
        if int(info) == 0:
            Kinv = torch.cholesky_inverse(L).double()
        else:                                             # float32 not enough: factor in FP64
            Kinv = torch.cholesky_inverse(torch.linalg.cholesky(Ks))
        self.Kc_inv = (Kinv * s[:, None] * s[None, :]).float().contiguous()
        # half-precision copy for the coarse matvecs of tm_twolevel_apply:
        # H = D^-1 K_c^-1 D^-1 (symmetrised, unit diagonal, |H_ij| <= 1) with
        # D = diag(sqrt(K_c^-1_ii)), half the bytes of the float32 matrix
        d = torch.sqrt(torch.clamp(torch.diagonal(self.Kc_inv), min=torch.finfo(torch.float32).tiny))
        H = 0.5 * (self.Kc_inv + self.Kc_inv.T) / (d[:, None] * d[None, :])   # exactly symmetric
        self.kc_half = H.half().contiguous()
        self.kc_scale = d.float().contiguous()
        self.agg_order = torch.argsort(agg, stable=True)
        self.agg_ptr = torch.zeros(nc + 1, dtype=torch.int64, device=dev)
        self.agg_ptr[1:] = torch.cumsum(torch.bincount(agg, minlength=nc), 0)
        self.agg32 = agg32
        self.agg_order32 = self.agg_order.to(torch.int32).contiguous()
        self.kp_values32 = self.kp_values.float().contiguous()

    def restrict_solve(self, r: torch.Tensor) -> torch.Tensor:
        """y_c = K_c^-1 P^T r (coarse values, FP64)."""
        from .adjoint import segment_sum
        rc = segment_sum(self.agg_ptr, self.agg_order, r.double().contiguous(), 1)
        return (self.Kc_inv @ rc.float()).double()

    def apply(self, r: torch.Tensor) -> torch.Tensor:
        """P K_c^-1 P^T r."""
        return self.restrict_solve(r)[self.agg].to(r.dtype)

    def kp(self, yc: torch.Tensor) -> torch.Tensor:
        """K P y_c."""
        return spmv_raw(self.kp_indptr, self.kp_indices, self.kp_values, yc.double().contiguous())


@dataclass
class LearnedSolveInfo(SolveInfo):
    preconditioner: str = "learned"
    fallback: bool = False
    seconds: float = 0.0


class LearnedPreconditioner:
    """Two-level preconditioner whose smoother weights come from the MPNN.

    At set-up the network reads the normalised operator (edge weights a_ij,
    input feature 1 on every node, so its first layer sees the row sums of A)
    and returns one value y_i per dof; the smoother is the damped Jacobi step
    S = diag(w) D^-1 with w_i = 1/2 + sigmoid(y_i) in (1/2, 3/2) (w = 1 when
    the network outputs 0).  With the coarse correction C = P K_c^-1 P^T the
    preconditioner is
        z = C r + (I - C K) S (I - K C) r,
    symmetric positive definite, applied with one SpMV by K and one by the
    thin K P.  ``use_network=False`` gives the same method with w = 1."""

    def __init__(self, model: Optional[MPNN] = None, device="cuda", coarse_target: int = 512,
                 use_network: bool = True, coords: Optional[torch.Tensor] = None):
        self.model = model or MPNN(device)
        self.coarse_target = coarse_target
        self.use_network = use_network
        self.coords = coords          # dof coordinates, used when solve() gets none
        self._setup_key = None

    def setup(self, A, coords):
        key = (A.values.data_ptr(), A.values._version, A.nnz, self.use_network)
        if key == self._setup_key:
            return
        self.A = A
        self.G = Graph(A.indptr, A.indices, A.values.detach())
        self.coarse = CoarseSpace(A.indptr, A.indices, A.values.detach(), coords, self.coarse_target)
        self.w = self.weights()
        self.sw = (self.w.double() * self.G.dinv).to(A.dtype).contiguous()
        self._sell = self._sell_copy() if A.dtype == torch.float64 else None
        self._fused = self._fused_struct() if A.dtype == torch.float64 else None
        self._setup_key = key

    def _sell_copy(self):
        """SELL-32 copy of K (FP64 values, 16-bit column offsets where they
        fit) for the flexible CG's products (tm_sell_fill / tm_spmv_sell)."""
        from .solve import sell_plan
        A = self.A
        sp, n_pad, narrow = sell_plan(A.indptr, A.indices)
        dev = A.values.device
        scol = torch.empty(n_pad, dtype=torch.int16 if narrow else torch.int32, device=dev)
        sval = torch.empty(n_pad, dtype=torch.float64, device=dev)
        bad = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("tm_sell_fill", _lib.TM_F64, A.shape[0], A.indptr.data_ptr(), A.indices.data_ptr(),
                  A.values.detach().contiguous().data_ptr(), sp.data_ptr(), n_pad, int(narrow), scol.data_ptr(),
                  sval.data_ptr(), bad.data_ptr(), _s(dev))
        if int(bad.item()) != 0:
            return None    # a pattern the copy cannot hold: the products stay on the CSR arrays
        # the float32 copy for the smoother's product shares the column array
        sval32 = sval.float()
        return sp, int(narrow), scol, sval, sval32

    def _fused_struct(self):
        """ctypes view of the operator for tm_twolevel_apply (the tensors it
        points to are kept on self)."""
        C, G, A = self.coarse, self.G, self.A
        n = G.n
        self._sw32 = self.sw.float().contiguous()
        self._work = torch.empty(2 * n + 4 * C.nc, dtype=torch.float32, device=A.values.device)
        t = _lib.TwoLevel()
        t.n, t.nc, t.pad0 = n, C.nc, 0
        t.agg, t.agg_ptr, t.agg_perm = C.agg32.data_ptr(), C.agg_ptr.data_ptr(), C.agg_order32.data_ptr()
        t.kc_inv = C.Kc_inv.data_ptr()
        t.kc_half, t.kc_scale = C.kc_half.data_ptr(), C.kc_scale.data_ptr()
        t.kp_indptr, t.kp_indices, t.kp_values = (C.kp_indptr.data_ptr(), C.kp_indices.data_ptr(),
                                                  C.kp_values32.data_ptr())
        t.k_nnz = int(G.values32.shape[0])
        t.k_indptr, t.k_indices, t.k_values = A.indptr.data_ptr(), A.indices.data_ptr(), G.values32.data_ptr()
        t.sw, t.work = self._sw32.data_ptr(), self._work.data_ptr()
        sell = getattr(self, "_sell", None)
        if sell is not None:
            t.k_slice_ptr, t.k_scol, t.k_sval, t.k_narrow = (sell[0].data_ptr(), sell[2].data_ptr(),
                                                             sell[4].data_ptr(), sell[1])
        return t

    def weights(self, keep: bool = False):
        """Smoother weights w (float32 [n]); with keep=True also (y, saved)."""
        G = self.G
        if not self.use_network:
            return torch.ones(G.n, dtype=torch.float32, device=G.device)
        x = torch.ones(G.n, dtype=torch.float32, device=G.device)
        if keep:
            y, saved = self.model.forward(G, x, keep=True)
            return 0.5 + torch.sigmoid(y), (y, saved)
        return 0.5 + torch.sigmoid(self.model.forward(G, x))

    def _K(self, v):
        return spmv_raw(self.A.indptr, self.A.indices, self.A.values, v.to(self.A.dtype).contiguous())

    def __call__(self, r: torch.Tensor) -> torch.Tensor:
        if self._fused is not None and r.dtype == torch.float64:
            z = torch.empty_like(r)
            _lib.call("tm_twolevel_apply", self._fused, r.contiguous().data_ptr(), z.data_ptr(),
                      _lib.stream_handle(r.device))
            return z
        C = self.coarse
        yc = C.restrict_solve(r)
        r1 = r - C.kp(yc).to(r.dtype)                 # r - K C r
        s1 = self.sw * r1                            # S (I - K C) r
        r2 = self._K(s1)
        yc2 = C.restrict_solve(r2)
        return (yc - yc2).to(r.dtype)[C.agg] + s1    # C r + (I - C K) s1

    def _iterate(self, x, r, p, rz, k: int):
        """k flexible-PCG iterations; x, r, p and rz (0-dim) are updated in
        place, so the sequence can be captured once and replayed.  FP64
        systems with the fused operator run them as one C call
        (tm_fcg_twolevel_iterations: the vector updates and dot products in a
        few fused kernels, every scalar kept on the device)."""
        if self._fused is not None and x.dtype == torch.float64:
            n = x.shape[0]
            bufs = getattr(self, "_fcg_bufs", None)
            if bufs is None or bufs[0].shape[0] != n or bufs[0].device != x.device:
                nd = int(_lib.load().tm_fcg_workspace_doubles())
                bufs = (torch.empty(n, dtype=torch.float64, device=x.device),
                        torch.empty(n, dtype=torch.float64, device=x.device),
                        torch.zeros(8, dtype=torch.float64, device=x.device),
                        torch.empty(nd, dtype=torch.float64, device=x.device))
                self._fcg_bufs = bufs
            q, z, sc, part = bufs
            A = self.A
            sc[:1].copy_(rz.reshape(1))
            sell = getattr(self, "_sell", None)
            sp, narrow, scol, sval = sell[:4] if sell is not None else (None, 0, None, None)
            _lib.call("tm_fcg_twolevel_iterations", self._fused, A.nnz, A.indptr.data_ptr(), A.indices.data_ptr(),
                      A.values.data_ptr(), _lib.ptr(sp), narrow, _lib.ptr(scol), _lib.ptr(sval), x.data_ptr(),
                      r.data_ptr(), p.data_ptr(), q.data_ptr(), z.data_ptr(), sc.data_ptr(), part.data_ptr(), int(k),
                      _lib.stream_handle(x.device))
            rz.copy_(sc[0])
            return
        rr, pp, rzz = r, p, rz
        for _ in range(k):
            q = self._K(pp)
            alpha = rzz / torch.dot(pp, q)
            x.add_(alpha * pp)
            r_new = rr - alpha * q
            z_new = self(r_new)
            # Polak-Ribiere (z, r_new - r_old) with r_new - r_old = -alpha q
            # (the form without the cancelling subtraction, as the fused path)
            beta = torch.clamp(-alpha * torch.dot(z_new, q) / rzz, min=0.0)
            rzz = torch.dot(r_new, z_new)
            pp = z_new + beta * pp
            rr = r_new
        r.copy_(rr)
        p.copy_(pp)
        rz.copy_(rzz)

    def _captured(self, state, k: int):
        """Capture ``k`` iterations on ``state`` = (x, r, p, rz) as a CUDA graph
        and return its replay function.  The state tensors are the graph's
        fixed inputs and outputs: their values change, their storage must not."""
        x, r, p, rz = state
        saved = [t.clone() for t in state]
        side = torch.cuda.Stream(device=x.device)
        side.wait_stream(torch.cuda.current_stream(x.device))
        with torch.cuda.stream(side):
            self._iterate(x, r, p, rz, 1)          # warm-up: library handles, allocator
        torch.cuda.current_stream(x.device).wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._iterate(x, r, p, rz, k)
        for t, v in zip(state, saved):             # capture records, the warm-up ran: restore
            t.copy_(v)
        self._graph = g
        return g.replay

    def solve(self, A, b, x, rtol=1e-8, atol=0.0, maxiter=10000, coords=None, check_every: int = 8,
              fallback: bool = True, graph: bool = True):
        """Flexible CG (Polak-Ribiere beta) with this preconditioner; falls
        back to Jacobi-PCG if the residual stagnates (``fallback=False``
        returns after ``maxiter`` iterations instead).  x is updated in place."""
        if coords is None:
            coords = self.coords
        if coords is None:
            raise ValueError("the learned preconditioner needs dof coordinates (coords=) for its coarse space")
        t0 = time.perf_counter()
        self.setup(A, coords)
        bn = float(torch.linalg.vector_norm(b.double()))
        tol = max(rtol * bn, atol)
        xw = x.clone() if graph and x.is_cuda else x
        r = b - self._K(xw)
        z = self(r)
        p = z.clone()
        rz = torch.dot(r, z)
        it = 0
        best = float("inf")
        stall = 0
        status = _lib.TM_ERR_MAXITER
        run = self._captured((xw, r, p, rz), check_every) if xw is not x else None
        while it < maxiter:
            rn = float(torch.linalg.vector_norm(r))
            if rn <= tol:
                status = _lib.TM_OK
                break
            if not math.isfinite(rn):
                status = _lib.TM_ERR_BREAKDOWN
                break
            best, stall = (rn, 0) if rn < 0.999 * best else (best, stall + check_every)
            if stall > 64:
                break
            k = min(check_every, maxiter - it)
            if run is not None and k == check_every:
                run()
            else:
                self._iterate(xw, r, p, rz, k)
            it += k
        if xw is not x:
            x.copy_(xw)
        if status == _lib.TM_ERR_MAXITER and float(torch.linalg.vector_norm(r)) <= tol:
            status = _lib.TM_OK
        true_res = true_relative_residual(A.indptr, A.indices, A.values, b, x, bn)
        fell_back = False
        if fallback and (status != _lib.TM_OK or true_res > rtol * 1.0000001):
            fb = pcg_jacobi_raw(A.indptr, A.indices, A.values.contiguous(), b, x, rtol, atol, maxiter)
            it += fb.iterations
            status, true_res, fell_back = fb.status, fb.residual, True
        return LearnedSolveInfo(status, it, true_res, true_res, 0, "learned", fell_back, time.perf_counter() - t0)


# -- training --------------------------------------------------------------------
def generate_pairs(systems, iterations=(1, 3, 8, 20), rtol=1e-10, coarse_target: int = 512):
    """Residual/error pairs seen by the preconditioner inside its own solver.

    systems: iterable of (A, b, coords).  For each, x* comes from Jacobi-PCG
    to ``rtol``; then flexible PCG with the two-level method at w = 1 runs and
    the residual r_k and error e_k = x* - x_k are taken after each count in
    ``iterations``.  Pairs are grouped per system: (A, coords, [(r, e), ...])."""
    out = []
    for A, b, coords in systems:
        xs = torch.zeros_like(b)
        pcg_jacobi_raw(A.indptr, A.indices, A.values, b, xs, rtol, 0.0, 100000)
        base = LearnedPreconditioner(None, device=b.device, coarse_target=coarse_target, use_network=False)
        pr = []
        for k in iterations:
            xk = torch.zeros_like(b)
            base.solve(A, b, xk, rtol=1e-30, maxiter=k, coords=coords, check_every=k, fallback=False, graph=False)
            r = b - spmv_raw(A.indptr, A.indices, A.values, xk)
            pr.append((r.float(), (xs - xk).float()))
        out.append((A, coords, pr))
    return out


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


def train(precond: LearnedPreconditioner, systems, epochs: int = 2, lr: float = 2e-3, log=None,
          n_random: int = 4, seed: int = 0) -> List[float]:
    """Fit the network that sets the smoother weights by a condition-number
    proxy of the preconditioned operator M K.

    For an error e with residual r = K e, rho(e) = r^T M r / e^T K e lies in
    [lambda_min, lambda_max] of M K.  The errors of the solver's own iterates
    sit near lambda_min and random errors spread over the spectrum, so the
    loss per system is mean(-log rho) over the iterate pairs plus
    mean(log rho) over ``n_random`` Gaussian errors: a proxy for
    log(lambda_max / lambda_min), the quantity PCG's iteration count follows.
    (A common scale of the weights does not change it: the coarse part of M K
    is the identity on its own K-orthogonal subspace.)

    With s = S r1, r1 = (I - K C) r, z = M r = C r + (I - C K) s and
    d log(r^T z) / dz = r / r^T z, the gradient with respect to s is
    (I - K C) r / r^T z, so dL/dw_i = g_s,i (D^-1 r1)_i and
    dL/dy_i = dL/dw_i (w_i - 1/2) (3/2 - w_i).  Per system the network runs
    forward once and backward once on the summed gradient."""
    model = precond.model
    precond.use_network = True
    opt = Adam(model.params, lr=lr)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    losses = []
    for ep in range(epochs):
        for (A, coords, pr) in systems:
            precond._setup_key = None
            precond.setup(A, coords)
            G, C = precond.G, precond.coarse
            w, (y, saved) = precond.weights(keep=True)
            dinv = G.dinv.float()
            K = lambda v: spmv_raw(A.indptr, A.indices, A.values, v.double().contiguous()).float()  # noqa: E731
            gy = torch.zeros_like(y)
            rand = [torch.randn(G.n, generator=gen).to(y.device) for _ in range(n_random)]
            terms = [(r, e, -1.0 / len(pr)) for r, e in pr] + [(K(e), e, 1.0 / n_random) for e in rand]
            total = 0.0
            for r, e, sgn in terms:
                yc = C.restrict_solve(r)
                r1 = r - C.kp(yc).float()
                u = dinv * r1                         # D^-1 r1
                s = w * u
                z = yc.float()[C.agg] + s - C.apply(K(s)).float()
                rz = float(torch.dot(r, z))
                eke = float(torch.dot(e, K(e)))
                if not (rz > 0 and eke > 0):
                    continue
                total += sgn * math.log(rz / eke)
                gs = (r - K(C.apply(r).float())) * (sgn / rz)
                gy += gs * u * (w - 0.5) * (1.5 - w)
            losses.append(total)
            grads = model.backward(G, saved, gy)
            opt.step(grads)
            model.invalidate()
        if log is not None:
            log(ep, sum(losses[-len(systems):]) / max(1, len(systems)))
    return losses
