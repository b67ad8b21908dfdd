"""Batched assembly + Jacobi-PCG of many independent meshes in one persistent,
graph-captured launch, with an autotuner for its launch shape.

The reference has no batched path: a user loops over meshes in Python,
calling ``Assembler.from_mesh(mesh)(...)``, ``Condenser`` and ``K.solve``
once per mesh.  ``BatchedPoisson`` takes the
list of meshes once, builds a union patch plan whose patches never straddle
instances, and then every call

    u, info = batch(kappa)          # kappa: per-element coefficients, concatenated

assembles K_k = int kappa grad u . grad v and b_k = int f v for every
instance k (float32) and solves K_ii u_i = f_i (zero Dirichlet on each
instance's boundary) with Jacobi-PCG -- all inside ONE kernel launch
(``tm_batched_assemble_pcg``), captured in a CUDA graph and replayed.

Size-aware clusters: the batch time is set by its largest instances, whose
PCG iterations are latency-bound on a small cluster, while the many small
instances want many small clusters.  The ``n_big`` largest instances therefore
run in a second persistent launch with ``cluster_big`` CTAs per cluster (8 or
16, distributed shared memory across the cluster), concurrently on a forked
stream with the launch that serves the rest; both are captured in the same
CUDA graph.  ``autotune`` times the launch for patch sizes x cluster sizes x
big-group shapes and keeps the fastest; results are cached per (device,
element, batch signature) in a JSON file (``TM_AUTOTUNE_CACHE`` or
~/.cache/tensormesh_gb300/autotune.json).
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
from dataclasses import dataclass
from typing import List, Optional, Sequence

import torch

from . import _lib, element as E_
from .plan import PatchPlan, node_pattern

from .autotune import load_cache as _load_cache, store_cache as _store_cache


@dataclass
class BatchInfo:
    status: torch.Tensor      # int32 [n_inst] (0 = converged, 3 = iteration cap, 4 = breakdown)
    iterations: torch.Tensor  # int32 [n_inst]
    residual: torch.Tensor    # float32 [n_inst] recurrence ||r|| / ||b||


class BatchedPoisson:
    """Float32 assembly + Jacobi-PCG of independent P1 meshes in one launch."""

    def __init__(self, meshes: Sequence, quadrature_order: int = 1, source: float = 1.0,
                 slot_budget: int = 2048, cluster: Optional[int] = None, device=None,
                 cluster_big: Optional[int] = None, n_big: int = 0):
        if not meshes:
            raise ValueError("empty batch")
        etypes = {m.default_element_type for m in meshes}
        if len(etypes) != 1 or next(iter(etypes)) not in ("triangle", "tetra"):
            raise NotImplementedError("batched path: all meshes must be P1 triangles or P1 tetrahedra")
        self.element_type = next(iter(etypes))
        self.el_id, self.dim, self.n_basis, _ = E_.element_info(self.element_type)
        dev = torch.device(device) if device is not None else meshes[0].points.device
        if dev.type != "cuda":
            raise RuntimeError("the batched path runs on CUDA only")
        self.device = dev
        self.quadrature_order = quadrature_order
        self.source = float(source)
        pts, els, bds, grp = [], [], [], []
        n_off = 0
        self.node_ptr = [0]
        self.elem_ptr = [0]
        for k, m in enumerate(meshes):
            el = m.elements()
            pts.append(m.points.to(dev, torch.float32))
            els.append(el.to(dev).long() + n_off)
            bds.append(m.boundary_mask.to(dev))
            grp.append(torch.full((m.n_points,), k, dtype=torch.int64, device=dev))
            n_off += m.n_points
            self.node_ptr.append(n_off)
            self.elem_ptr.append(self.elem_ptr[-1] + int(el.shape[0]))
        self.points = torch.cat(pts).contiguous()
        self.elements = torch.cat(els)
        self.dirichlet = torch.cat(bds).to(torch.uint8).contiguous()
        self.groups = torch.cat(grp)
        self.n_inst = len(meshes)
        self.n_rows = n_off
        self.n_elements = self.elem_ptr[-1]
        self.pattern = node_pattern(self.elements, self.n_rows)
        sizes = torch.tensor([self.node_ptr[k + 1] - self.node_ptr[k] for k in range(self.n_inst)])
        self.order = torch.argsort(sizes, descending=True, stable=True).to(torch.int32).to(dev)
        self.inst_rbeg = torch.tensor(self.node_ptr, dtype=torch.int64, device=dev)
        self.values = torch.empty(self.pattern.nnz, dtype=torch.float32, device=dev)
        self.b = torch.empty(self.n_rows, dtype=torch.float32, device=dev)
        self.x = torch.empty(self.n_rows, dtype=torch.float32, device=dev)
        self.work = torch.empty(6 * self.n_rows, dtype=torch.float32, device=dev)
        self.status = torch.empty(self.n_inst, dtype=torch.int32, device=dev)
        self.iters = torch.empty(self.n_inst, dtype=torch.int32, device=dev)
        self.resid = torch.empty(self.n_inst, dtype=torch.float32, device=dev)
        self.queue = torch.zeros(2, dtype=torch.int32, device=dev)   # one counter per launch group
        self.tables = E_.kernel_tables(self.element_type, quadrature_order, dev)
        self.kappa = torch.ones(self.n_elements, dtype=torch.float32, device=dev)
        self._plans = {}
        self._graph = None
        self._config = None
        self._side = None
        self.set_config(slot_budget, cluster, cluster_big, n_big)

    # -- configuration ---------------------------------------------------------
    def _plan(self, slot_budget: int):
        if slot_budget not in self._plans:
            plan = PatchPlan(self.elements, self.points, self.pattern, slot_budget=slot_budget,
                             max_rows_cap=1024, groups=self.groups)
            inst_of_patch = self.groups[plan.rows.long()[plan.rptr[:-1].long().clamp(max=self.n_rows - 1)]]
            pbeg = torch.zeros(self.n_inst + 1, dtype=torch.int64, device=self.device)
            pbeg[1:] = torch.cumsum(torch.bincount(inst_of_patch, minlength=self.n_inst), 0)
            self._plans[slot_budget] = (plan, plan.to_struct(), pbeg.to(torch.int32))
        return self._plans[slot_budget]

    def set_config(self, slot_budget: int, cluster: Optional[int], cluster_big: Optional[int] = None,
                   n_big: int = 0):
        """Patch size, cluster size of the main launch, and the big group: the
        ``n_big`` largest instances on clusters of ``cluster_big`` CTAs (no big
        group when n_big is 0 or cluster_big is None)."""
        lib = _lib.load()
        plan, pstruct, pbeg = self._plan(slot_budget)
        chunk = 128
        smem = max(lib.tm_patch_smem_bytes(self.el_id, _lib.TM_FORM_LAPLACE, 1, _lib.TM_F32, ctypes.byref(pstruct),
                                           _lib.TM_COEF_ELEMENT, chunk),
                   lib.tm_patch_smem_bytes(self.el_id, _lib.TM_FORM_LOAD, 1, _lib.TM_F32, ctypes.byref(pstruct),
                                           _lib.TM_COEF_SCALAR, chunk))
        cluster = cluster or 4
        n_big = int(n_big) if cluster_big else 0
        n_big = max(0, min(n_big, self.n_inst - 1))
        cap = lib.tm_batched_max_clusters(self.el_id, cluster, smem)
        if cap <= 0:
            raise _lib.TensorMeshCudaError("tm_batched_max_clusters", -cap if cap < 0 else 6)
        groups = []
        if n_big > 0:
            cap_big = lib.tm_batched_max_clusters(self.el_id, cluster_big, smem)
            if cap_big <= 0:
                raise _lib.TensorMeshCudaError("tm_batched_max_clusters", -cap_big if cap_big < 0 else 6)
            nb = min(n_big, cap_big)
            groups.append(dict(cluster=cluster_big, n_clusters=nb, first=0, count=n_big))
            # the main launch takes the clusters the big group leaves free
            used = -(-nb * cluster_big // cluster)
            cap = max(1, cap - used)
        groups.append(dict(cluster=cluster, n_clusters=cap, first=n_big, count=self.n_inst - n_big))
        self._config = dict(slot_budget=slot_budget, cluster=cluster, n_clusters=groups[-1]["n_clusters"],
                            cluster_big=cluster_big if n_big else None, n_big=n_big,
                            n_clusters_big=groups[0]["n_clusters"] if n_big else 0, smem=int(smem), chunk=chunk)
        self._groups = groups
        self._graph = None
        self._build_args(plan, pstruct, pbeg)

    def _build_args(self, plan, pstruct, pbeg):
        cfg = self._config
        mat = _lib.AssembleArgs()
        mat.element, mat.form, mat.dtype, mat.precision = self.el_id, _lib.TM_FORM_LAPLACE, _lib.TM_F32, 0
        mat.coef_kind, mat.n_comp = _lib.TM_COEF_ELEMENT, 1
        mat.n_quad = E_.n_quadrature(self.element_type, self.quadrature_order)
        mat.tables, mat.points, mat.coef = self.tables.data_ptr(), self.points.data_ptr(), self.kappa.data_ptr()
        mat.scal[0] = 1.0
        mat.out = self.values.data_ptr()
        load = _lib.AssembleArgs()
        load.element, load.form, load.dtype, load.precision = self.el_id, _lib.TM_FORM_LOAD, _lib.TM_F32, 0
        load.coef_kind, load.n_comp, load.n_quad = _lib.TM_COEF_SCALAR, 1, mat.n_quad
        load.tables, load.points, load.coef = self.tables.data_ptr(), self.points.data_ptr(), 0
        load.scal[0] = self.source
        load.out = self.b.data_ptr()
        self._keep = (pstruct, mat, load, plan, pbeg)
        self._args = []
        for gi, g in enumerate(self._groups):
            a = _lib.BatchedArgs()
            a.element, a.cluster, a.n_clusters, a.n_inst = self.el_id, g["cluster"], g["n_clusters"], g["count"]
            a.maxiter, a.chunk, a.rtol = 20000, cfg["chunk"], 1e-5
            a.n_rows, a.smem_bytes = self.n_rows, cfg["smem"]
            a.plan, a.mat, a.load = ctypes.pointer(pstruct), ctypes.pointer(mat), ctypes.pointer(load)
            a.order = self.order.data_ptr() + 4 * g["first"]
            a.inst_pbeg, a.inst_rbeg = pbeg.data_ptr(), self.inst_rbeg.data_ptr()
            a.indices, a.dirichlet = self.pattern.indices.data_ptr(), self.dirichlet.data_ptr()
            a.x, a.work = self.x.data_ptr(), self.work.data_ptr()
            a.status, a.iters, a.resid = self.status.data_ptr(), self.iters.data_ptr(), self.resid.data_ptr()
            a.queue = self.queue.data_ptr() + 4 * gi
            a.stream = 0
            self._args.append(a)

    @property
    def config(self) -> dict:
        return dict(self._config)

    @property
    def patch_plan(self) -> PatchPlan:
        return self._plan(self._config["slot_budget"])[0]

    # -- execution ---------------------------------------------------------------
    def launch(self, rtol: float = 1e-5, maxiter: int = 20000):
        """The launch group(s) on the current stream (no host synchronisation):
        with a big group, the main launch runs on a side stream forked from
        and joined back into the current one, so the two overlap."""
        cur = torch.cuda.current_stream(self.device)
        for a in self._args:
            a.rtol = float(rtol)
            a.maxiter = int(maxiter)
        if len(self._args) == 1:
            _lib.call("tm_batched_assemble_pcg", ctypes.byref(self._args[0]), cur.cuda_stream)
            return
        if self._side is None:
            self._side = torch.cuda.Stream(self.device)
        self._side.wait_stream(cur)
        _lib.call("tm_batched_assemble_pcg", ctypes.byref(self._args[0]), cur.cuda_stream)
        with torch.cuda.stream(self._side):
            _lib.call("tm_batched_assemble_pcg", ctypes.byref(self._args[1]), self._side.cuda_stream)
        cur.wait_stream(self._side)

    def capture(self, rtol: float = 1e-5, maxiter: int = 20000) -> torch.cuda.CUDAGraph:
        """Capture the launch group(s) in a CUDA graph (replayed by ``replay``)."""
        self._captured_at = (float(rtol), int(maxiter))
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.launch(rtol, maxiter)  # warm: sets kernel attributes outside capture
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(rtol, maxiter)
        self._graph = g
        return g

    def replay(self):
        if self._graph is None:
            self.capture()
        self._graph.replay()

    def __call__(self, kappa: torch.Tensor, rtol: float = 1e-5, maxiter: int = 20000, graph: bool = True):
        """Assemble and solve every instance; returns (u [n_rows] float32
        concatenated node-major, BatchInfo)."""
        if kappa.shape[0] != self.n_elements:
            raise AssertionError(f"kappa must have {self.n_elements} entries, got {kappa.shape[0]}")
        self.kappa.copy_(kappa.to(self.device, torch.float32))
        if graph:
            if self._graph is None or self._captured_at != (float(rtol), int(maxiter)):
                self.capture(rtol, maxiter)
            self._graph.replay()
        else:
            self.launch(rtol, maxiter)
        return self.x, BatchInfo(self.status, self.iters, self.resid)

    def split(self, v: torch.Tensor) -> List[torch.Tensor]:
        return [v[self.node_ptr[k]:self.node_ptr[k + 1]] for k in range(self.n_inst)]

    # -- autotuning --------------------------------------------------------------
    def signature(self) -> str:
        h = hashlib.sha1()
        h.update(f"{self.element_type}|{self.n_inst}|{self.n_rows}|{self.n_elements}".encode())
        return h.hexdigest()[:16]

    def autotune(self, kappa: torch.Tensor, clusters=(2, 4, 8), budgets=(1024, 2048, 4096), reps: int = 3,
                 rtol: float = 1e-5, use_cache: bool = True, big=((None, 0), (8, 4), (16, 2), (16, 8))) -> dict:
        """Time every (slot budget, cluster, big group) candidate on this batch
        and keep the fastest; ``big`` lists (cluster_big, n_big) shapes,
        (None, 0) being a single launch.  Returns the chosen config with its
        time in ms."""
        name = torch.cuda.get_device_name(self.device)
        key = f"batched2|{name}|{self.signature()}|{rtol}"
        if use_cache:
            hit = _load_cache().get(key)
            if hit:
                self.set_config(hit["slot_budget"], hit["cluster"], hit.get("cluster_big"), hit.get("n_big", 0))
                return hit
        self.kappa.copy_(kappa.to(self.device, torch.float32))
        results = []
        for bgt in budgets:
            for cl in clusters:
                for cb, nbig in big:
                    try:
                        self.set_config(bgt, cl, cb, nbig)
                        self.launch(rtol)
                        torch.cuda.synchronize(self.device)
                        e0 = torch.cuda.Event(enable_timing=True)
                        e1 = torch.cuda.Event(enable_timing=True)
                        e0.record()
                        for _ in range(reps):
                            self.launch(rtol)
                        e1.record()
                        torch.cuda.synchronize(self.device)
                        results.append((e0.elapsed_time(e1) / reps, bgt, cl, cb or 0, nbig if cb else 0))
                    except _lib.TensorMeshCudaError:
                        continue
        if not results:
            raise RuntimeError("autotune: no launch configuration ran")
        ms, bgt, cl, cb, nbig = min(results)
        self.set_config(bgt, cl, cb or None, nbig)
        best = dict(slot_budget=bgt, cluster=cl, cluster_big=cb or None, n_big=nbig, ms=ms,
                    n_clusters=self._config["n_clusters"], n_clusters_big=self._config["n_clusters_big"],
                    candidates=[dict(ms=r[0], slot_budget=r[1], cluster=r[2], cluster_big=r[3] or None, n_big=r[4])
                                for r in results])
        if use_cache:
            _store_cache(key, best)
        return best
