"""Headline benchmark: FP64 assembly of the 128^3 P1-tet Poisson problem.

Workload (one "step" = one assembly of the global stiffness matrix):
  unit cube, 128^3 cells, 6 Kuhn tetrahedra per cell (12,582,912 tets,
  2,146,689 nodes, 31,802,497 CSR entries), float64, 1-point quadrature,
  per-element kappa piecewise constant on 8^3 blocks of 16^3 cells with
  log kappa ~ N(0, 2^2) per block (seeded); integrand kappa * gradu . gradv.
  Synthetic inputs; the inputs (608 MB of algorithmic bytes per step) are
  larger than the 129 MB L2, so no flush is needed between steps.

metric = elements/s assembled.  ``value`` times the assembly with inputs
resident in HBM; ``e2e`` times the public API call with host (pinned)
buffers and the host<->device copies inside the timed region.  ``roofline``
divides the algorithmic bytes 4*B*E + 8*D*N + 8*E + 8*nnz by the kernel's
CUDA-event duration.  ``cpu_baseline`` times the CPU oracle port on a
bounded sample of the same workload on this host's cores.  A second block,
``pcg``, reports the wall time of Jacobi-PCG to a 1e-8 FP64 relative
residual on the condensed system (zero Dirichlet on all faces, f = 1).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Replicas only: with N > 1 (torchrun) every rank assembles its own copy and
``value`` sums the ranks' elements over the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_CELLS = 128
BLOCKS = 8
SEED = 2024


def log_kappa_blocks(n_cells, blocks, seed):
    rng = np.random.default_rng(seed)
    g = rng.normal(0.0, 2.0, size=(blocks, blocks, blocks))   # indexed [bk, bj, bi]
    c = np.arange(n_cells ** 3)
    i, j, k = c % n_cells, (c // n_cells) % n_cells, c // (n_cells * n_cells)
    s = n_cells // blocks
    per_cell = g[k // s, j // s, i // s]
    return np.repeat(per_cell, 6)                              # 6 tets per cell, cell-major


def algorithmic_bytes(E, B, D, N, nnz, itemsize=8):
    return 4 * B * E + itemsize * D * N + itemsize * E + itemsize * nnz


def read_profile_value(prefix: str):
    """A number from the committed ncu summary of the headline kernel."""
    path = os.path.join(ROOT, "profiles", "assemble_p1tet_fp64_128cube.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(prefix):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def read_profile_traffic():
    return read_profile_value("dram_bytes_per_launch_full_size:")


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = os.path.join("/tmp", f"tm_clocks_{os.getpid()}.csv")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def aggregate_over_ranks(total_ms: float, units: int, device):
    """(the timed region's duration, max over ranks, in ms; the units all
    ranks processed, summed).  With one process the inputs come back."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(total_ms), int(units)
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    u = torch.tensor([int(units)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), int(u.item())


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


CPU_KIND = "reference-torch"
CPU_SAMPLE_NOTE = ("the reference's own torch operation sequence of ElementAssembler.__call__ (Jacobian einsum, "
                   "torch.inverse, det, vmapped integrand, einsum, index_add_; oracle/torch_ref.py, timed within "
                   "+-25% of the reference itself by tests/test_cpu_baseline.py) with torch on all host threads")


def cpu_baseline_run(points, elements, kappa, sample_elems, threads, reps=2):
    """The reference's CPU operation sequence (oracle.torch_ref) on the first
    ``sample_elems`` elements with ``threads`` torch threads; the per-mesh
    set-up (pattern, slot map) is untimed, as the reference's from_mesh is.
    Returns (elements/s, seconds of the best rep)."""
    import torch
    from oracle.torch_ref import ReferenceOps
    torch.set_num_threads(threads)
    el = elements[:sample_elems]
    ops = ReferenceOps(points, el, "tetra", 1)
    pts_t = torch.from_numpy(np.ascontiguousarray(points))
    kp = torch.from_numpy(np.ascontiguousarray(kappa[:sample_elems]))
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        ops.values(pts_t, kp)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return sample_elems / best, best


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import torch
    from tensormesh_gb300 import Mesh
    mesh = Mesh.gen_unit_cube(N_CELLS)
    pts = mesh.points.numpy()
    el = mesh.cells["tetra"].numpy()
    kappa = np.exp(log_kappa_blocks(N_CELLS, BLOCKS, SEED))
    threads = os.cpu_count() or 1
    sample = min(el.shape[0], 1 << 20)
    for _ in range(args.warmup):
        cpu_baseline_run(pts, el, kappa, sample, threads, reps=1)
    times = []
    for _ in range(args.steps):
        eps, dt = cpu_baseline_run(pts, el, kappa, sample, threads, reps=1)
        times.append(dt)
    t = float(np.mean(times))
    v = sample / t
    print(json.dumps({
        "impl": "reference", "metric": "elements/s assembled", "value": v, "unit": "elements/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"P1-tet Poisson assembly, {N_CELLS}^3 Kuhn cube, FP64, kappa on 8^3 blocks; "
                               f"CPU sample = first {sample} elements", "global_batch": sample},
        "cpu_baseline": {"value": v, "unit": "elements/s", "cores": threads, "kind": CPU_KIND,
                         "sample": f"first {sample} of {el.shape[0]} elements; {CPU_SAMPLE_NOTE}"},
        "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_ours(args):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    peak, peak_src = hbm_peak()
    import tensormesh_gb300 as tg
    # the per-call finiteness check of the inputs waits on the device (a host
    # synchronisation per call); the reference has no such check, and it would
    # serialise the pipelined end-to-end steps, so the benchmark turns it off
    tg.set_input_checks(False)

    t_init = time.perf_counter()
    torch.zeros(1, device=dev).sum().item()          # CUDA context + allocator warm
    init_s = time.perf_counter() - t_init

    class KappaLaplace(tg.ElementAssembler):
        def forward(self, gradu, gradv, kappa):
            return kappa * (gradu @ gradv)

    # first use of the library kernels the set-up calls (torch's sorts and
    # scans, the project's own kernels): on a fresh machine their code is
    # paged in from disk here, which a 4^3 mesh shows apart from the set-up
    t_first = time.perf_counter()
    tiny = tg.Mesh.gen_unit_cube(4, device=dev)
    KappaLaplace.from_mesh(tiny, quadrature_order=1)(tiny.points, element_data={
        "kappa": torch.ones(tiny.cells["tetra"].shape[0], dtype=torch.float64, device=dev)})
    torch.cuda.synchronize()
    first_use_s = time.perf_counter() - t_first
    t_setup = time.perf_counter()
    mesh = tg.Mesh.gen_unit_cube(N_CELLS, device=dev)
    kappa_h = torch.from_numpy(np.exp(log_kappa_blocks(N_CELLS, BLOCKS, SEED)))
    kappa = kappa_h.to(dev)

    asm = KappaLaplace.from_mesh(mesh, quadrature_order=1)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t_setup
    # patch size chosen by the project's autotuner on these inputs (not timed)
    if args.slot_budget:
        asm.slot_budget, tuned = args.slot_budget, {"table": []}
    else:
        tuned = asm.autotune(mesh.points, element_data={"kappa": kappa}, use_cache=False,
                             budgets=(512, 1024, 2048, 3072, 4096, 6144))
    topo = asm.topology
    E, N, B, D = topo.n_elements, topo.n_points, topo.n_basis, topo.dim
    nnz = topo.pattern.nnz
    stream = torch.cuda.current_stream(dev)

    def step():
        return asm(mesh.points, element_data={"kappa": kappa}).values

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    # the clock sampler polls every 200 ms and the timed region lasts a few
    # tens of ms, so it starts under a further ~0.6 s of untimed steps: its
    # samples then show the clocks of the loaded GPU around the timed region
    clocks = ClockSampler(local)
    t_load = time.perf_counter()
    while time.perf_counter() - t_load < 0.6:
        for _ in range(20):
            step()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    torch.cuda.nvtx.range_push("bench_timed")   # lets a profiler select exactly the timed launches
    for i in range(args.steps):
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.nvtx.range_pop()
    t1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    if clk is not None:
        clk["window"] = "0.6 s of untimed steps, then the timed region"
    total_ms = t0.elapsed_time(t1)
    kernel_ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    total_ms, units = aggregate_over_ranks(total_ms, E * args.steps, dev)
    ms_per_step = total_ms / args.steps
    value = units / (total_ms * 1e-3)

    # ---- float32 variant of the same assembly (secondary line item)
    def time_calls(fn, reps=5):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b_ = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b_.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b_) / reps

    fp32 = None
    if want_extra(args, "fp32"):
        pts32 = mesh.points.float().contiguous()
        kap32 = kappa.float()
        asm32 = KappaLaplace.from_assembler(asm)
        tuned32 = asm32.autotune(pts32, element_data={"kappa": kap32}, use_cache=False,
                                 budgets=(512, 1024, 2048, 3072, 4096, 6144))
        ms32 = time_calls(lambda: asm32(pts32, element_data={"kappa": kap32}))
        alg32 = algorithmic_bytes(E, B, D, N, nnz, itemsize=4)
        fp32 = {"elements_per_s": E / (ms32 * 1e-3), "kernel_ms": ms32, "algorithmic_bytes": alg32,
                "achieved_gbs": alg32 / (ms32 * 1e-3) / 1e9, "slot_budget": tuned32["slot_budget"]}
        peaks_path_ = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(peaks_path_):
            fp32["hbm_frac"] = fp32["achieved_gbs"] / float(json.load(open(peaks_path_))["hbm_gbs"])

    # ---- boundary traction load (FacetAssembler) on the same 128^3 mesh, FP64
    facet = None
    if want_extra(args, "facet"):
        class Traction(tg.FacetAssembler):
            def forward(self, v):
                return v[:, None] * torch.tensor([0.0, 0.3, -1.0], dtype=v.dtype, device=v.device)
        t0 = time.perf_counter()
        fasm = Traction.from_mesh(mesh, quadrature_order=2)
        torch.cuda.synchronize()
        f_setup = time.perf_counter() - t0
        ms_f = time_calls(lambda: fasm(mesh.points))
        S = fasm.topology.n_sel
        facet = {"workload": "128^3 Kuhn cube, traction (0, 0.3, -1) on every facet with all nodes on the boundary, "
                             "facet rule of order 2, FP64",
                 "facets": S, "ms_per_load": ms_f, "facets_per_s": S / (ms_f * 1e-3),
                 "setup_seconds": round(f_setup, 3)}
        del fasm

    # ---- 64^3 P1-tet linear elasticity, per-element E, FP64 (secondary)
    elast = None
    hyper = None
    if want_extra(args, "elasticity"):
        m2 = tg.Mesh.gen_unit_cube(64, device=dev)
        rng = np.random.default_rng(SEED + 2)
        Emod = torch.from_numpy(np.exp(0.5 * rng.normal(size=m2.n_elements))).to(dev)

        class EElast(tg.ElementAssembler):
            def forward(self, gradu, gradv, E):
                lam, mu = tg.forms.reference_lame(1.0, 0.3)
                return E * tg.forms.elasticity_block(gradu, gradv, lam, mu)
        easm = EElast.from_mesh(m2, quadrature_order=1)
        ms2 = time_calls(lambda: easm(m2.points, element_data={"E": Emod}), reps=3)
        t2 = easm.topology
        dnnz = 9 * t2.pattern.nnz
        alg2 = 4 * 4 * t2.n_elements + 8 * 3 * t2.n_points + 8 * t2.n_elements + 8 * dnnz
        elast = {"workload": "64^3 Kuhn cube P1-tet elasticity, per-element E = exp(0.5 g), nu = 0.3, FP64",
                 "elements_per_s": t2.n_elements / (ms2 * 1e-3), "kernel_ms": ms2, "algorithmic_bytes": alg2,
                 "achieved_gbs": alg2 / (ms2 * 1e-3) / 1e9}
        # the C2 solve: x = 0 face clamped, body force (0, 0, -1), Jacobi-PCG to
        # a 1e-8 FP64 relative residual (checked with the plain FP64 SpMV)
        if not args.no_pcg:
            K2 = easm(m2.points, element_data={"E": Emod})
            f2 = tg.const_node_assembler(torch.tensor([0.0, 0.0, -1.0], dtype=torch.float64)).from_mesh(m2, quadrature_order=1)(m2.points)
            clamp = (m2.points[:, 0] == 0.0).repeat_interleave(3)
            K2_ii, f2_i = tg.Condenser(clamp)(K2, f2)
            K2_ii.solve(f2_i, rtol=1e-8, maxiter=args.pcg_maxiter * 4)   # warm (workspace, launch)
            torch.cuda.synchronize()
            ta2 = time.perf_counter()
            K2_ii.solve(f2_i, rtol=1e-8, maxiter=args.pcg_maxiter * 4)
            torch.cuda.synchronize()
            tb2 = time.perf_counter()
            i2 = K2_ii.last_solve_info
            it2 = 12 * K2_ii.nnz + 4 * (K2_ii.shape[0] + 1) + 80 * K2_ii.shape[0]
            elast["pcg_c2"] = {"jacobi_seconds_to_1e-8": tb2 - ta2, "iterations": i2.iterations,
                               "true_residual": i2.residual, "status": i2.status, "n": K2_ii.shape[0],
                               "nnz": K2_ii.nnz, "per_iteration_algorithmic_bytes": it2,
                               "achieved_gbs": it2 * i2.iterations / (tb2 - ta2) / 1e9}
            del K2, K2_ii
        # Neo-Hookean energy + its displacement gradient (ElementAssembler.energy
        # and backward) on the same mesh
        nh = tg.NeoHookeanModel.from_mesh(m2, quadrature_order=1, E=1.0, nu=0.3)
        g_u = torch.from_numpy(np.random.default_rng(SEED + 5).normal(size=tuple(m2.points.shape)))
        u_nh = (g_u * (0.1 / 64)).to(dev).requires_grad_(True)

        def nh_step():
            u_nh.grad = None
            nh.energy(u_nh).backward()
        ms_nh = time_calls(nh_step)
        hyper = {"workload": "64^3 Kuhn cube, Neo-Hookean energy and its displacement gradient, FP64, "
                             "u ~ N(0, (0.1 h)^2) per node",
                 "elements_per_s": t2.n_elements / (ms_nh * 1e-3), "ms_per_energy_and_gradient": ms_nh}
        del easm, m2, nh

    # ---- gradient of the compliance J = b^T u, K(kappa, x) u = b, with
    #      respect to the per-element kappa and the nodal coordinates, 256^2
    #      split square, FP64 (forward assembly + Jacobi-PCG + adjoint solve +
    #      backward assembly)
    adjoint = None
    if want_extra(args, "adjoint"):
        m4 = tg.Mesh.gen_unit_square(256, device=dev)
        k4 = torch.from_numpy(np.exp(np.random.default_rng(SEED + 4).normal(size=m4.n_elements))).to(dev)
        a4 = KappaLaplace.from_mesh(m4, quadrature_order=1)
        l4 = tg.const_node_assembler(1.0).from_mesh(m4, quadrature_order=1)
        c4 = tg.Condenser(m4.boundary_mask)

        from tensormesh_gb300.learned import LearnedPreconditioner
        two4 = LearnedPreconditioner(None, coarse_target=256, use_network=False,
                                     coords=m4.points[~m4.boundary_mask].contiguous())

        def c4_step(pre):
            x = m4.points.clone().requires_grad_(True)
            kk = k4.clone().requires_grad_(True)
            K4 = a4(x, element_data={"kappa": kk})
            b4 = l4(x)
            K_ii4, f_i4 = c4(K4, b4)
            kw = {} if pre is None else {"preconditioner": pre}
            u4 = c4.recover(K_ii4.solve(f_i4, rtol=1e-10, **kw))
            (b4 * u4).sum().backward()
            return K_ii4.last_solve_info.iterations
        res4 = {}
        for name, pre in (("jacobi_pcg", None), ("two_level_pcg", two4)):
            c4_step(pre)
            torch.cuda.synchronize()
            ta4 = time.perf_counter()
            its4 = c4_step(pre)
            torch.cuda.synchronize()
            res4[name] = {"seconds_per_gradient": time.perf_counter() - ta4, "iterations_forward_solve": its4}
        adjoint = {"workload": "256^2 split unit square, P1, kappa = exp(N(0,1)) per element, FP64: dJ/dkappa and "
                               "dJ/dx of J = b^T u (forward assembly, PCG to 1e-10, adjoint solve, "
                               "backward assembly)",
                   "elements": m4.n_elements, **res4}
        del a4, l4, c4, m4, two4

    # ---- 256 uneven 2D Poisson meshes, assembled + Jacobi-PCG in one
    #      persistent, graph-captured launch (FP32), autotuned launch shape
    batched = None
    if want_extra(args, "batched"):
        from tensormesh_gb300.batched import BatchedPoisson
        rng = np.random.default_rng(SEED + 3)
        sizes = rng.integers(32, 257, size=256)
        meshes = [tg.Mesh.gen_unit_square(int(k), device=dev) for k in sizes]
        kap = torch.from_numpy(np.exp(rng.normal(size=sum(m.n_elements for m in meshes)))).to(dev)
        t0b = time.perf_counter()
        bp = BatchedPoisson(meshes)
        tune = bp.autotune(kap, clusters=(2, 4, 8), budgets=(1024, 2048), reps=2, rtol=1e-5, use_cache=False)
        u_b, info_b = bp(kap, rtol=1e-5)           # capture + first replay
        torch.cuda.synchronize()
        setup_b = time.perf_counter() - t0b
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(3):
            bp.replay()
        ev1.record(stream)
        torch.cuda.synchronize()
        ms_b = ev0.elapsed_time(ev1) / 3
        st = info_b.status.cpu()
        # algorithmic bytes of the launch: the assembly reads connectivity,
        # kappa and coordinates and writes values and b; each PCG iteration of
        # instance k streams its CSR (4 B value + 4 B column per entry) and
        # ten float vector passes over its rows
        its = info_b.iterations.cpu().numpy().astype(np.int64)
        ipb = bp.pattern.indptr.cpu().numpy()
        npb = np.asarray(bp.node_ptr, dtype=np.int64)
        nnz_k = ipb[npb[1:]] - ipb[npb[:-1]]
        rows_k = npb[1:] - npb[:-1]
        alg_b = (16 * bp.n_elements + 12 * bp.n_rows + 4 * int(ipb[-1])
                 + int(np.sum(its * (8 * nnz_k + 40 * rows_k))))
        batched = {"workload": "256 unit-square P1 meshes, N ~ U{32..256} (seeded), kappa = exp(N(0,1)) per element, "
                               "f = 1, zero Dirichlet, FP32 assembly + Jacobi-PCG to 1e-5, one graph-replayed launch",
                   "instances": len(meshes), "elements": int(bp.n_elements), "rows": int(bp.n_rows),
                   "ms_per_launch": ms_b, "elements_per_s": bp.n_elements / (ms_b * 1e-3),
                   "converged": int((st == 0).sum()), "max_iterations": int(info_b.iterations.max()),
                   "autotuned": {k: tune[k] for k in ("cluster", "slot_budget", "n_clusters", "cluster_big", "n_big",
                                                      "n_clusters_big", "ms")},
                   "roofline": {"bound": "hbm", "achieved": alg_b / (ms_b * 1e-3) / 1e9, "peak": peak,
                                "unit": "GB/s", "frac": alg_b / (ms_b * 1e-3) / 1e9 / peak,
                                "algorithmic_bytes": alg_b, "peak_source": peak_src,
                                "note": "per-instance working sets are L2-sized, so the launch can exceed the "
                                        "HBM roofline; the figure says how far the launch is from streaming"},
                   "setup_seconds": setup_b, "gpu_launches_per_step": 2 if tune.get("n_big") else 1}
        del bp, meshes

    # ---- end to end through the public API with host buffers: every step
    #      copies its inputs from pinned host memory, assembles, and reads the
    #      CSR values back; consecutive steps take streams in turn so one
    #      step's copies overlap the neighbouring steps' work
    pts_h = mesh.points.cpu().pin_memory()
    kap_h = kappa_h.pin_memory()
    n_streams = 3
    streams = [torch.cuda.Stream(dev) for _ in range(n_streams)]
    outs_h = [torch.empty(nnz, dtype=torch.float64).pin_memory() for _ in streams]
    pts_d = [torch.empty_like(mesh.points) for _ in streams]      # per-stream device inputs
    kap_d = [torch.empty_like(kappa) for _ in streams]

    def e2e_step(i):
        j = i % n_streams
        with torch.cuda.stream(streams[j]):
            pts_d[j].copy_(pts_h, non_blocking=True)
            kap_d[j].copy_(kap_h, non_blocking=True)
            v = asm(pts_d[j], element_data={"kappa": kap_d[j]}).values
            outs_h[j].copy_(v, non_blocking=True)

    for i in range(n_streams):
        e2e_step(i)
    torch.cuda.synchronize()
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for st in streams:
        st.wait_stream(stream)
    for i in range(args.steps):
        e2e_step(i)
    for st in streams:
        stream.wait_stream(st)
    s1.record(stream)
    torch.cuda.synchronize()
    e2e_total, e2e_units = aggregate_over_ranks(s0.elapsed_time(s1), E * args.steps, dev)
    e2e_ms = e2e_total / args.steps
    h2d = pts_h.numel() * 8 + kap_h.numel() * 8
    d2h = nnz * 8

    alg = algorithmic_bytes(E, B, D, N, nnz)
    achieved = alg / (kernel_ms * 1e-3) / 1e9
    traffic = read_profile_traffic()

    # ---- Jacobi-PCG to a 1e-8 FP64 relative residual on the condensed system
    pcg = None
    if not args.no_pcg:
        K = asm(mesh.points, element_data={"kappa": kappa})
        b = tg.const_node_assembler(1.0).from_mesh(mesh, quadrature_order=1)(mesh.points)
        K_ii, f_i = tg.Condenser(mesh.boundary_mask)(K, b)
        K_ii.solve(f_i, rtol=1e-8, maxiter=args.pcg_maxiter)  # warm (workspace, launch)
        torch.cuda.synchronize()
        ta = time.perf_counter()
        K_ii.solve(f_i, rtol=1e-8, maxiter=args.pcg_maxiter)
        torch.cuda.synchronize()
        tb = time.perf_counter()
        info = K_ii.last_solve_info
        it_bytes = 12 * K_ii.nnz + 4 * (K_ii.shape[0] + 1) + 80 * K_ii.shape[0]
        from tensormesh_gb300 import solve as solve_mod
        _, n_pad, narrow = solve_mod.sell_plan(K_ii.indptr, K_ii.indices)
        ach = it_bytes * info.iterations / (tb - ta) / 1e9
        pcg = {"jacobi_seconds_to_1e-8": tb - ta, "iterations": info.iterations, "true_residual": info.residual,
               "status": info.status, "n": K_ii.shape[0], "nnz": K_ii.nnz,
               "kernel": "tm_pcg_jacobi_sell, standard form, SELL-32 copy (%d padded entries, %s-bit columns)"
                         % (n_pad, "16" if narrow else "32"),
               "per_iteration_algorithmic_bytes": it_bytes, "ms_per_iteration": 1e3 * (tb - ta) / max(1, info.iterations),
               "achieved_gbs": ach,
               "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                            "peak_source": peak_src,
                            "note": "whole solve (plan cached, SELL fill, iterations, FP64 true-residual check) "
                                    "over iterations x the algorithmic bytes of one iteration"},
               "learned_seconds_to_1e-8": None}
        if rank == 0 and world == 1 and not args.no_cpu:
            # the reference's Jacobi-PCG operation sequence on the host cores,
            # timed on a bounded number of iterations of the same system
            from oracle.torch_ref import ReferenceJacobiPCG
            threads = os.cpu_count() or 1
            torch.set_num_threads(threads)
            ref = ReferenceJacobiPCG(K_ii.indptr.cpu().numpy(), K_ii.indices.cpu().numpy(),
                                     K_ii.values.cpu().numpy())
            bh = f_i.cpu()
            ref.iterate(bh, 2)
            n_it = 20
            t0c = time.perf_counter()
            ref.iterate(bh, n_it)
            sec_it = (time.perf_counter() - t0c) / n_it
            pcg["cpu_baseline"] = {"seconds_per_iteration": sec_it, "cores": threads, "kind": "reference-torch",
                                   "projected_seconds_to_1e-8": sec_it * info.iterations,
                                   "sample": f"{n_it} iterations of the reference's CG loop with its Jacobi "
                                             "preconditioner (torch CSR on the host, oracle/torch_ref.py), "
                                             "projected to the GPU solve's iteration count"}
            del ref
        wpath = os.path.join(ROOT, "tensormesh_gb300", "weights", "mpnn_poisson_kuhn32.npz")
        if os.path.exists(wpath) and not args.no_learned:
            from tensormesh_gb300.learned import LearnedPreconditioner
            from tensormesh_gb300.train_learned import load_weights
            coords = mesh.points[~mesh.boundary_mask].contiguous()
            model = load_weights(wpath, dev)
            two = {}
            for name, use in (("learned", True), ("unit_weights", False)):
                pre = LearnedPreconditioner(model, coarse_target=512, use_network=use)
                pre.solve(K_ii, f_i, torch.zeros_like(f_i), rtol=1e-8, coords=coords, maxiter=3000)  # warm-up
                pre._setup_key = None
                torch.cuda.synchronize()
                t0s = time.perf_counter()
                pre.setup(K_ii, coords)
                torch.cuda.synchronize()
                t_setup = time.perf_counter() - t0s
                x = torch.zeros_like(f_i)
                linfo = pre.solve(K_ii, f_i, x, rtol=1e-8, coords=coords, maxiter=3000)
                torch.cuda.synchronize()
                t_solve = time.perf_counter() - t0s - t_setup
                two[name] = {"seconds_to_1e-8": t_setup + t_solve, "setup_seconds": t_setup,
                             "solve_seconds": t_solve, "iterations": linfo.iterations,
                             "true_residual": linfo.residual, "status": linfo.status, "fallback": linfo.fallback,
                             "vs_jacobi_time_ratio": (t_setup + t_solve) / (tb - ta)}
            L = two["learned"]
            pcg.update({"learned_seconds_to_1e-8": L["seconds_to_1e-8"], "learned_setup_seconds": L["setup_seconds"],
                        "learned_iterations": L["iterations"], "learned_true_residual": L["true_residual"],
                        "learned_status": L["status"], "learned_fallback": L["fallback"],
                        "learned_vs_jacobi_time_ratio": L["vs_jacobi_time_ratio"],
                        "two_level_unit_weights": two["unit_weights"]})

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        pts_np = mesh.points.cpu().numpy()
        el_np = topo.elements.cpu().numpy().astype(np.int64)
        threads = os.cpu_count() or 1
        sample = min(E, 1 << 20)
        eps, _ = cpu_baseline_run(pts_np, el_np, kappa_h.numpy(), sample, threads, reps=2)
        cpu = {"value": eps, "unit": "elements/s", "cores": threads, "kind": CPU_KIND,
               "sample": f"first {sample} of {E} elements; {CPU_SAMPLE_NOTE}"}

    if rank == 0:
        line = {
            "metric": "elements/s assembled", "value": value, "unit": "elements/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"P1-tet Poisson assembly, {N_CELLS}^3 Kuhn cube ({E} tets, {N} nodes, "
                                   f"{nnz} CSR values), FP64, 1-point quadrature, kappa piecewise constant "
                                   f"on 8^3 blocks, log kappa ~ N(0, 2^2)",
                       "global_batch": E * world, "l2": "inputs larger than L2 (608 MB per step), no flush",
                       "input_checks": "off (tensormesh_gb300.set_input_checks(False)): the finiteness check "
                                       "synchronises the host per call; the reference has none",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "patches": topo.plan_for(1, asm.slot_budget)[0].n_patches,
                       "element_redundancy": round(topo.plan_for(1, asm.slot_budget)[0].redundancy, 4),
                       "slot_budget": asm.slot_budget,
                       "autotune_ms": {str(t["candidate"]): round(t.get("ms", -1), 4) for t in tuned["table"]},
                       "setup_seconds": round(setup_s, 3),
                       "setup_split_seconds": {"cuda_and_torch_init": round(init_s, 3),
                                               "first_use_of_library_kernels_4cube": round(first_use_s, 3),
                                               **{k: round(v, 3) for k, v in topo.timings.items()}}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                         "algorithmic_bytes_per_launch": alg, "kernel_ms": kernel_ms,
                         "ncu_issue_active_pct": read_profile_value("smsp__issue_active.avg.pct_of_peak_sustained_active:"),
                         "limiter": "instruction issue (double-float arithmetic on the FP32 pipe), not HBM"},
            "e2e": {"value": e2e_units / (e2e_total * 1e-3), "unit": "elements/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                    "pipelining": f"consecutive steps on {n_streams} streams in turn"},
            "cpu_baseline": cpu,
            "fp32_variant": fp32,
            "elasticity_64cube": elast,
            "facet_traction_128cube": facet,
            "neo_hookean_energy": hyper,
            "adjoint_256_square": adjoint,
            "batched_256_meshes": batched,
            "gpu_launches": args.steps,
            "clocks": clk,
            "pcg": pcg,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


EXTRAS = ("fp32", "facet", "elasticity", "adjoint", "batched")


def want_extra(args, name: str) -> bool:
    """Whether the side measurement ``name`` runs: all of them by default,
    none with --no-extra, a comma-separated subset with --extra."""
    if args.no_extra:
        return False
    return args.extra is None or name in args.extra.split(",")


def hbm_peak():
    """(GB/s, "measured" | "fallback"): the copy bandwidth in MEASURED_PEAKS.json,
    else the fallback figure of an earlier GB300 measurement."""
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        return float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def main():
    global N_CELLS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-pcg", action="store_true")
    ap.add_argument("--cube", type=int, default=N_CELLS, help="cells per side (profiling runs use smaller cubes)")
    ap.add_argument("--pcg-maxiter", type=int, default=200000)
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip every side measurement")
    ap.add_argument("--extra", default=None,
                    help="comma-separated side measurements to run, of " + ",".join(EXTRAS) + " (default: all)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--slot-budget", type=int, default=0, help="fixed patch slot budget instead of autotuning")
    args = ap.parse_args()
    N_CELLS = args.cube
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
