"""Benchmark of the GB300 sparse Krylov engine.

Headline (one "step" = one full solve): plain FP64 pipelined CG
(linalg::solve(A, b, cg_tag(1e-10, 10000)), the reference's no-preconditioner
path) on the 3D 7-point Laplacian 128^3 = 2,097,152 rows / 14,581,760 nnz,
b ~ U[-1,1] (seed 1), to relative residual 1e-10; value = seconds per solve
with the matrix and b resident in HBM.  e2e = the same solve through the
public API starting from pinned host CSR arrays and b (H2D copies, matrix
creation, solve, D2H of x inside the timed region).

Secondary fields: SpMV GB/s per format on the 128^3 Laplacian and the 4M-row
lognormal matrix, BiCGStab and GMRES(30) on the lognormal matrix, the 192^3
variable-coefficient diffusion solved by FP32-inner/FP64-refined CG against
the plain FP64 Jacobi-PCG path, and the reference's CPU-runnable 256^2 case.

--impl reference times the reference's own CPU algorithm (the C restatement
in oracle/, OpenMP on all host cores) on the headline workload.
Multi-GPU: the path does not shard, so N ranks run N independent replicas.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "viennacl-dev_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import vclgb_gen as gen  # noqa: E402

METRIC = "CG solve s @1e-10 FP64 resid: mixed/batched vs plain FP64 on GPU; SpMV GB/s"
# DRAM bytes (read + write) of one launch of the CG SpMV phase kernel on the
# 128^3 Laplacian in the solve's steady state, with the solve's vectors held in
# the persisting L2 window: the ncu capture summarised in
# profiles/csr_fixed_laplace3d_128.md (183,556,096 read + 1,039,872 written, the
# mean of two consecutive launches; the matrix alone is 183.4 MB)
TRAFFIC_SPMV_CG = 184595968
WORKLOAD = "3D 7-point Laplacian 128^3 (2,097,152 rows, 14,581,760 nnz), FP64 CSR, pipelined CG to 1e-10"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def spmv_bytes(n, nnz, sv=8, beta=False):
    """Algorithmic bytes of one SpMV (format independent): values+indices once,
    row_ptr once, x read once, y written once (+ read when beta != 0)."""
    return nnz * (sv + 4) + (n + 1) * 4 + n * sv + n * sv + (n * sv if beta else 0)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
def dist_setup(backend):
    import torch.distributed as dist
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value, ws):
    """Max of a float over ranks (identity on one rank)."""
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
def graph_apply_time(V, torch, P, vec, reps):
    """Device time of one preconditioner apply replayed from a CUDA graph:
    a second backend on a side stream, one apply captured on it, replayed
    `reps` times between CUDA events on that stream.  None if the capture
    fails."""
    try:
        s = torch.cuda.Stream()
        be = V.Backend(stream=s.cuda_stream)
        ptr = V._ptr(vec)
        torch.cuda.synchronize()
        for _ in range(3):
            be.check(be.lib.vclgbPrecondApply(be.h, P.h, ptr))
        be.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            be.check(be.lib.vclgbPrecondApply(be.h, P.h, ptr))
        with torch.cuda.stream(s):
            for _ in range(3):
                g.replay()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(reps):
                g.replay()
            e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps
    except Exception:
        return None


def time_events(fn, reps):
    """Average device time of fn() over reps, CUDA events, synchronised both sides."""
    import torch
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / 1e3 / reps


def spmv_gbs(V, M, n, nnz, reps, x, y):
    t = time_events(lambda: V.prod(M, x, y=y), reps)
    b = spmv_bytes(n, nnz)
    return t, b / t / 1e9


def run_ours(args):
    import torch
    import vclgb as V
    ws, rank, local = dist_setup("nccl")
    torch.cuda.set_device(local)
    peak, peak_kind = peaks()
    out = {"metric": METRIC, "unit": "s", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generators, vclgb_gen.py)"}

    # ---- headline workload -------------------------------------------------
    rp, ci, v = gen.laplace3d(128)
    n, nnz = len(rp) - 1, int(rp[-1])
    b = gen.rhs_uniform(n, 1)
    A = V.compressed_matrix(rp, ci, v)
    bd = torch.tensor(b, device="cuda")
    xd = torch.empty(n, dtype=torch.float64, device="cuda")
    tol, maxit = 1e-10, 10000

    def solve_once():
        tag = V.cg_tag(tol, maxit)
        V.solve(A, bd, tag, None, x=xd)
        return tag

    for _ in range(max(args.warmup, 3)):
        tag = solve_once()
    barrier(ws)
    torch.cuda.synchronize()
    l0 = A.be.launches()
    clk = ClockSampler(local)
    clk.start()
    tags = []
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(args.steps):
        tags.append(solve_once())
    e.record()
    torch.cuda.synchronize()
    clocks = clk.stop()
    barrier(ws)
    t_solve = s.elapsed_time(e) / 1e3 / args.steps
    t_solve = max_over_ranks(t_solve, ws)
    launches = A.be.launches() - l0
    iters = tags[-1].iters()
    rel = true_rel_residual(rp, ci, v, xd.cpu().numpy(), b)
    out["value"] = t_solve
    out["ms_per_step"] = t_solve * 1e3
    out["config"] = {"workload": WORKLOAD, "solver": "pipelined CG (cg.hpp:128-187), no preconditioner",
                     "tol": tol, "rhs": "U[-1,1] seed 1", "iterations": iters,
                     "true_rel_residual": rel, "solver_error_estimate": tags[-1].error(),
                     "l2": "working set (250 MB) larger than the 126 MB L2; no flush",
                     "parallelism": "replicas" if ws > 1 else "single GPU"}
    out["gpu_launches"] = int(launches)
    out["clocks"] = clocks

    # ---- roofline: the dominant kernel of the solve ---------------------------
    # One more solve of the same workload with the backend's kernel timing on:
    # CUDA event pairs around every SpMV phase (the CSR product with the fused
    # CG dots, csr_fixed_kernel<1,7,double,EpiCg>) and every fused vector pass
    # (vec_pass_kernel<CgUpdate>), recorded as nodes of the solver's captured
    # graphs on its stream.  Launches after convergence inside the last graph
    # chunk return at their first instruction; they are the durations below
    # half the median and are left out.
    A.be.set_kernel_timing(True)
    try:
        tag_t = solve_once()
        t_spmv_all, t_vec_all = A.be.kernel_times(0), A.be.kernel_times(1)
    finally:
        A.be.set_kernel_timing(False)

    def active(t):
        t = np.asarray(t, dtype=np.float64)
        return t[t > 0.5 * np.median(t)] if t.size else t
    t_spmv, t_vec = active(t_spmv_all), active(t_vec_all)
    b_spmv = spmv_bytes(n, nnz)      # p read once, Ap written; p[r] of the dots is the same array
    b_vec = 7 * 8 * n                # x, p, r, Ap read; x, p, r written
    us_spmv, us_vec = float(t_spmv.mean()) * 1e3, float(t_vec.mean()) * 1e3
    gbs = b_spmv / (us_spmv * 1e-6) / 1e9
    out["roofline"] = {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                       "frac": gbs / peak, "peak_kind": peak_kind,
                       "kernel": "csr_fixed_kernel<1,7,double,EpiCg<double>> (CSR SpMV + CG dots, "
                                 "thread per row; 67% of the solve's device time)",
                       "algorithmic_bytes_per_launch": b_spmv,
                       "avg_launch_us": us_spmv, "launches_timed": int(t_spmv.size),
                       "traffic": TRAFFIC_SPMV_CG,
                       "traffic_source": "profiles/csr_fixed_laplace3d_128.md (ncu, steady-state "
                                         "launches, vectors in the L2 window)",
                       "second_kernel": {
                           "kernel": "vec_pass_kernel<double,CgUpdate<double>>",
                           "algorithmic_bytes_per_launch": b_vec, "avg_launch_us": us_vec,
                           "achieved": b_vec / (us_vec * 1e-6) / 1e9,
                           "frac": b_vec / (us_vec * 1e-6) / 1e9 / peak},
                       "per_iteration": {
                           "us": t_solve * 1e6 / max(iters, 1),
                           "algorithmic_bytes": b_spmv + b_vec,
                           "hbm_floor_us": (b_spmv + b_vec) / (peak * 1e9) * 1e6,
                           "fp64_fma_per_iteration": nnz + 6 * n}}
    # the plain product (linalg::prod, no epilogue work) on the same matrix
    xs = torch.tensor(gen.rhs_uniform(n, 11), device="cuda")
    ys = torch.empty(n, dtype=torch.float64, device="cuda")
    for _ in range(5):
        V.prod(A, xs, y=ys)
    t_plain, gbs_plain = spmv_gbs(V, A, n, nnz, 50, xs, ys)
    out["roofline"]["plain_prod"] = {"kernel": "csr_fixed_kernel<1,7,double,EpiAxpbyM<double,0,true>>",
                                     "avg_launch_us": t_plain * 1e6, "achieved": gbs_plain,
                                     "frac": gbs_plain / peak}

    # ---- e2e from host buffers ----------------------------------------------
    h_rp = torch.from_numpy(rp.view(np.int32)).pin_memory()
    h_ci = torch.from_numpy(ci.view(np.int32)).pin_memory()
    h_v = torch.from_numpy(v).pin_memory()
    h_b = torch.from_numpy(b).pin_memory()
    h_x = torch.empty(n, dtype=torch.float64).pin_memory()
    d_rp = torch.empty_like(h_rp, device="cuda")
    d_ci = torch.empty_like(h_ci, device="cuda")
    d_v = torch.empty_like(h_v, device="cuda")
    d_b = torch.empty_like(h_b, device="cuda")

    def e2e_step():
        d_rp.copy_(h_rp, non_blocking=True)
        d_ci.copy_(h_ci, non_blocking=True)
        d_v.copy_(h_v, non_blocking=True)
        d_b.copy_(h_b, non_blocking=True)
        M = V.compressed_matrix(d_rp, d_ci, d_v, n, n)
        tag = V.cg_tag(tol, maxit)
        x = V.solve(M, d_b, tag)
        h_x.copy_(x, non_blocking=True)
        return tag

    for _ in range(2):
        e2e_step()
    t_e2e = time_events(e2e_step, args.steps)
    t_e2e = max_over_ranks(t_e2e, ws)
    h2d = h_rp.numel() * 4 + h_ci.numel() * 4 + h_v.numel() * 8 + h_b.numel() * 8
    out["e2e"] = {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": int(h2d),
                  "d2h_bytes_per_step": int(n * 8),
                  "what": "pinned host CSR+b -> H2D, compressed_matrix (validate+analyse), "
                          "solve, x -> host"}
    del A

    # ---- secondary measurements ----------------------------------------------
    sec = {}
    if not args.quick:
        sec = secondaries(V, torch, peak, args)
    out["secondary"] = sec

    # ---- CPU baseline (rank 0, N=1): the reference algorithm on host cores ---
    if rank == 0 and ws == 1 and not args.quick:
        out["cpu_baseline"] = cpu_baseline_cg(rp, ci, v, b, tol, maxit)
        try:
            out["cpu_baseline"]["preconditioners"] = cpu_baseline_preconditioners()
        except Exception as e:  # a side figure: it never takes the bench line with it
            out["cpu_baseline"]["preconditioners"] = {"error": str(e)}
    else:
        out["cpu_baseline"] = None
    if rank == 0:
        print(json.dumps(out))


def secondaries(V, torch, peak, args):
    sec = {}
    # SpMV format sweep on the 128^3 Laplacian
    rp, ci, v = gen.laplace3d(128)
    n, nnz = len(rp) - 1, int(rp[-1])
    A = V.compressed_matrix(rp, ci, v)
    x = torch.tensor(gen.rhs_uniform(n, 1), device="cuda")
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    r = {}
    for name, M in (("csr", A), ("ell", V.ell_matrix(A)), ("sell_c32_s1", V.sliced_ell_matrix(A, 32, 1)),
                    ("hyb", V.hyb_matrix(A))):
        for _ in range(3):
            V.prod(M, x, y=y)
        t, g = spmv_gbs(V, M, n, nnz, 30, x, y)
        r[name] = {"us": t * 1e6, "GBs": g, "frac_of_peak": g / peak,
                   "GFLOPs": 2 * nnz / t / 1e9}
    r["autotune"] = A.autotune()
    t, g = spmv_gbs(V, A, n, nnz, 30, x, y)
    r["autotuned"] = {"us": t * 1e6, "GBs": g, "frac_of_peak": g / peak}
    A.autotune_clear()
    sec["spmv_laplace3d_128"] = r
    del A
    # 4M-row lognormal matrix
    t0 = time.time()
    rp, ci, v = gen.lognormal_random(4194304, seed=1)
    n, nnz = len(rp) - 1, int(rp[-1])
    gen_s = time.time() - t0
    A = V.compressed_matrix(rp, ci, v)
    x = torch.tensor(gen.rhs_uniform(n, 1), device="cuda")
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    r = {"rows": n, "nnz": nnz, "generate_s": gen_s}
    mats = [("csr", A), ("sell_c32_s256", V.sliced_ell_matrix(A, 32, 256)),
            ("sell_c32_s1", V.sliced_ell_matrix(A, 32, 1)), ("hyb", V.hyb_matrix(A))]
    for name, M in mats:
        for _ in range(3):
            V.prod(M, x, y=y)
        t, g = spmv_gbs(V, M, n, nnz, 20, x, y)
        r[name] = {"us": t * 1e6, "GBs": g, "frac_of_peak": g / peak, "stored": int(M.info().stored)}
    r["ell"] = "skipped: max row length 2000 pads ELL to ~100 GB"
    del mats
    # the per-matrix autotuner's choice, and the product on the chosen form
    r["autotune"] = A.autotune()
    t, g = spmv_gbs(V, A, n, nnz, 20, x, y)
    r["autotuned"] = {"us": t * 1e6, "GBs": g, "frac_of_peak": g / peak}
    A.autotune_clear()
    sec["spmv_lognormal_4M"] = r
    # BiCGStab / GMRES(30) on the lognormal matrix (no preconditioner, as configured)
    b = gen.rhs_uniform(n, 1)
    bd = torch.tensor(b, device="cuda")
    s = {}
    PJ = V.jacobi_precond(A)
    for name, tag, P in (("bicgstab", V.bicgstab_tag(1e-10, 3000), None),
                         ("gmres30", V.gmres_tag(1e-10, 3000, 30), None),
                         ("bicgstab_jacobi", V.bicgstab_tag(1e-10, 3000), PJ),
                         ("gmres30_jacobi", V.gmres_tag(1e-10, 3000, 30), PJ),
                         ("bicgstab_jacobi_1e-12", V.bicgstab_tag(1e-12, 3000), PJ),
                         ("gmres30_jacobi_1e-12", V.gmres_tag(1e-12, 3000, 30), PJ)):
        torch.cuda.synchronize()
        t0 = time.time()
        xx = V.solve(A, bd, tag, P)
        torch.cuda.synchronize()
        s[name] = {"s": time.time() - t0, "iters": tag.iters(), "status": V.STATUS_NAMES[tag.status()],
                   "error_estimate": tag.error(),
                   "true_rel_residual": true_rel_residual(rp, ci, v, xx.cpu().numpy(), b)}
    # the oracle's runs of the same matrix and right-hand side
    # (tests/golden/make_lognormal_solvers.py): the unpreconditioned stall, and the
    # reference's Jacobi GMRES(30) ending falsely converged
    ref_file = os.path.join(ROOT, "tests", "golden", "lognormal_4194304_solvers.json")
    if os.path.exists(ref_file):
        with open(ref_file) as fh:
            s["oracle"] = {k: {kk: vv for kk, vv in r.items() if kk != "seconds"}
                           for k, r in json.load(fh)["runs"].items()}
    sec["solvers_lognormal_4M"] = s
    del A
    # 192^3 variable-coefficient diffusion: refined (FP32 inner) vs plain FP64 Jacobi-PCG
    rp, ci, v, f = gen.diffusion3d(192)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    fd = torch.tensor(f, device="cuda")
    P = V.jacobi_precond(A)
    res = {}

    def c3_arm(name, make_tag, precond):
        ts = []
        for rep in range(2):
            tag = make_tag()
            torch.cuda.synchronize()
            t0 = time.time()
            xx = V.solve(A, fd, tag, precond)
            torch.cuda.synchronize()
            ts.append(time.time() - t0)
        res[name] = {"s": min(ts), "iters": tag.iters(), "status": V.STATUS_NAMES[tag.status()],
                     "tol": tag.tolerance(),
                     "true_rel_residual": true_rel_residual(rp, ci, v, xx.cpu().numpy(), f)}
        if hasattr(tag, "outer"):
            res[name]["outer"] = tag.outer
        return res[name]

    plain = c3_arm("plain_fp64_jacobi_pcg", lambda: V.cg_tag(1e-10, 20000), P)
    c3_arm("refined_fp32_inner", lambda: V.refined_cg_tag(1e-10, 40000, 1e-4), None)
    res["speedup"] = res["plain_fp64_jacobi_pcg"]["s"] / res["refined_fp32_inner"]["s"]
    # Jacobi-PCG stops on <r, D^-1 r> / <b, D^-1 b> (cg.hpp:306-310), whose ratio
    # to the true ||b - Ax|| / ||b|| is steady late in the solve: the plain arm
    # is run again with its tolerance scaled so that its true residual is below
    # 1e-10 as well, and the speed-up is also reported at equal true residual
    if plain["true_rel_residual"] > 1e-10:
        tol2 = 1e-10 * 0.9 * 1e-10 / plain["true_rel_residual"]
        c3_arm("plain_fp64_jacobi_pcg_true_1e-10", lambda: V.cg_tag(tol2, 40000), P)
        res["speedup_at_true_1e-10"] = (res["plain_fp64_jacobi_pcg_true_1e-10"]["s"] /
                                        res["refined_fp32_inner"]["s"])
    sec["diffusion3d_192_mixed_vs_plain"] = res
    del A, P
    sec["ilu0_convdiff2d_512"] = bench_ilu0(V, torch)
    sec["chow_patel"] = bench_chow_patel(V, torch, peak)
    sec["batched_4096"] = bench_batched(V, torch)
    sec["adjoint_diffusion2d_512"] = bench_adjoint(V, torch)
    # the reference's CPU-runnable case: 256^2 Laplacian, Jacobi-PCG to 1e-8
    rp, ci, v = gen.laplace2d(256, 256, scaled=True)
    b = gen.rhs_uniform(len(rp) - 1, 0)
    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A)
    bd = torch.tensor(b, device="cuda")
    for _ in range(3):
        V.solve(A, bd, V.cg_tag(1e-8, 2000), P)
    tag = V.cg_tag(1e-8, 2000)
    t = time_events(lambda: V.solve(A, bd, tag, P), 10)
    sec["laplace2d_256_jacobi_pcg"] = {"s": t, "iters": tag.iters(),
                                       "us_per_iter": 1e6 * t / max(tag.iters(), 1)}
    # small-system latency: 70^2 Laplacian (4,900 rows), Jacobi-PCG to 1e-10;
    # the whole solve is launch- and latency-bound, so this is the cost of one
    # iteration's kernel chain on the device-side loop
    rp, ci, v = gen.laplace2d(70, 70)
    b = gen.rhs_uniform(len(rp) - 1, 0)
    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A)
    bd = torch.tensor(b, device="cuda")
    for _ in range(3):
        V.solve(A, bd, V.cg_tag(1e-10, 2000), P)
    tag = V.cg_tag(1e-10, 2000)
    t = time_events(lambda: V.solve(A, bd, tag, P), 20)
    sec["laplace2d_70_jacobi_pcg_latency"] = {"s": t, "iters": tag.iters(),
                                              "us_per_iter": 1e6 * t / max(tag.iters(), 1)}
    # the same for a nonsymmetric 70^2 convection-diffusion matrix with BiCGStab
    rp, ci, v = gen.convdiff2d(70, 70, peclet=5.0, shift=0.05)
    A = V.compressed_matrix(rp, ci, v)
    for _ in range(3):
        V.solve(A, bd, V.bicgstab_tag(1e-10, 2000))
    tag = V.bicgstab_tag(1e-10, 2000)
    t = time_events(lambda: V.solve(A, bd, tag), 20)
    sec["convdiff2d_70_bicgstab_latency"] = {"s": t, "iters": tag.iters(),
                                             "us_per_iter": 1e6 * t / max(tag.iters(), 1)}
    # and GMRES(20) on it (one cluster launch with the basis in shared memory)
    for _ in range(3):
        V.solve(A, bd, V.gmres_tag(1e-10, 2000, 20))
    tag = V.gmres_tag(1e-10, 2000, 20)
    t = time_events(lambda: V.solve(A, bd, tag), 20)
    sec["convdiff2d_70_gmres20_latency"] = {"s": t, "iters": tag.iters(),
                                            "us_per_iter": 1e6 * t / max(tag.iters(), 1)}
    return sec


def bench_ilu0(V, torch):
    """ILU0 on a 512^2 upwind convection-diffusion matrix: the device
    factorisation, the level-scheduled apply (runs of levels of up to 512 rows
    in one single-block launch), the same for block ILU0 with the reference's
    default 8 blocks, and BiCGStab with each against BiCGStab with Jacobi, to
    1e-10; ILU0 on the 128^3 Laplacian (levels of up to 12,288 rows, one
    cluster launch a triangle) with ILU0-CG to 1e-10."""
    rp, ci, v = gen.convdiff2d(512, 512, peclet=10.0, shift=0.01)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 5)
    A = V.compressed_matrix(rp, ci, v)
    bd = torch.tensor(b, device="cuda")
    V.ilu0_precond(A)  # first-use costs
    torch.cuda.synchronize()
    t0 = time.time()
    P = V.ilu0_precond(A)
    torch.cuda.synchronize()
    t_setup = time.time() - t0
    inf = P.info()
    z = bd.clone()
    t_apply = time_events(lambda: P.apply(z), 10)
    out = {"rows": n, "nnz": int(rp[-1]), "setup_s": t_setup, "levels_L": int(inf.num_levels_L),
           "levels_U": int(inf.num_levels_U), "apply_us": t_apply * 1e6}
    torch.cuda.synchronize()
    t0 = time.time()
    PB = V.block_ilu_precond(A, num_blocks=8)
    torch.cuda.synchronize()
    out["block_ilu8"] = {"setup_s": time.time() - t0, "levels_L": int(PB.info().num_levels_L),
                         "apply_us": time_events(lambda: PB.apply(z), 10) * 1e6}
    for name, pc in (("bicgstab_ilu0", P), ("bicgstab_block_ilu8", PB),
                     ("bicgstab_jacobi", V.jacobi_precond(A))):
        tag = V.bicgstab_tag(1e-10, 5000)
        V.solve(A, bd, V.bicgstab_tag(1e-10, 5000), pc)
        torch.cuda.synchronize()
        t0 = time.time()
        x = V.solve(A, bd, tag, pc)
        torch.cuda.synchronize()
        out[name] = {"s": time.time() - t0, "iters": tag.iters(), "status": V.STATUS_NAMES[tag.status()],
                     "true_rel_residual": true_rel_residual(rp, ci, v, x.cpu().numpy(), b)}
    del A, P, PB
    # 3D: the 128^3 Laplacian's 381 levels a triangle hold up to 12,288 rows;
    # runs of them go to a thread-block cluster (up to 16 CTAs of 1,024 threads)
    rp, ci, v = gen.laplace3d(128)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 5)
    A = V.compressed_matrix(rp, ci, v)
    bd = torch.tensor(b, device="cuda")
    torch.cuda.synchronize()
    t0 = time.time()
    P = V.ilu0_precond(A)
    torch.cuda.synchronize()
    r3 = {"rows": n, "nnz": int(rp[-1]), "setup_s": time.time() - t0,
          "levels_L": int(P.info().num_levels_L)}
    z = bd.clone()
    r3["apply_us"] = time_events(lambda: P.apply(z), 10) * 1e6
    tag = V.cg_tag(1e-10, 5000)
    V.solve(A, bd, V.cg_tag(1e-10, 5000), P)
    torch.cuda.synchronize()
    t0 = time.time()
    x = V.solve(A, bd, tag, P)
    torch.cuda.synchronize()
    r3["cg_ilu0"] = {"s": time.time() - t0, "iters": tag.iters(), "status": V.STATUS_NAMES[tag.status()],
                     "true_rel_residual": true_rel_residual(rp, ci, v, x.cpu().numpy(), b)}
    out["laplace3d_128"] = r3
    return out


def bench_chow_patel(V, torch, peak):
    """Chow-Patel preconditioners, default tag (3 sweeps, 2 Jacobi steps):
    ILU on the 512^2 convection-diffusion matrix (setup, apply with its
    algorithmic bytes, BiCGStab to 1e-10) and IC0 on the 128^3 Laplacian
    (CG to 1e-10 against the pipelined CG without a preconditioner)."""
    out = {}
    rp, ci, v = gen.convdiff2d(512, 512, peclet=10.0, shift=0.01)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 5)
    A = V.compressed_matrix(rp, ci, v)
    bd = torch.tensor(b, device="cuda")
    V.chow_patel_ilu_precond(A)
    torch.cuda.synchronize()
    t0 = time.time()
    P = V.chow_patel_ilu_precond(A)
    torch.cuda.synchronize()
    t_setup = time.time() - t0
    inf = P.info()
    z = bd.clone()
    t_apply = time_events(lambda: P.apply(z), 20)
    # div: v, D_L read, b_L written; per Jacobi step: N (12 B/entry + row_ptr),
    # x and b read, x written; the last L step also reads D_U
    steps = 2
    nb = inf.nnz_L * 12 + inf.nnz_U * 12 + 2 * (n + 1) * 4
    apply_bytes = 24 * n + steps * nb + 2 * steps * 24 * n + 8 * n
    r = {"rows": n, "setup_s": t_setup, "nnz_L": int(inf.nnz_L), "nnz_U": int(inf.nnz_U),
         "apply_us": t_apply * 1e6, "apply_bytes": int(apply_bytes),
         "apply_GBs": apply_bytes / t_apply / 1e9,
         "apply_frac_of_peak": apply_bytes / t_apply / 1e9 / peak,
         "apply_timing": "vclgbPrecondApply called from the host 20 times: the five "
                         "launches' host submission sets the pace"}
    t_graph = graph_apply_time(V, torch, P, bd.clone(), 50)
    if t_graph is not None:
        r["apply_graph_us"] = t_graph * 1e6
        r["apply_graph_frac_of_peak"] = apply_bytes / t_graph / 1e9 / peak
        r["apply_graph_timing"] = ("one apply captured in a CUDA graph on a side stream and "
                                   "replayed 50 times, as the solvers run it inside their "
                                   "captured iterations")
    tag = V.bicgstab_tag(1e-10, 5000)
    V.solve(A, bd, V.bicgstab_tag(1e-10, 5000), P)
    torch.cuda.synchronize()
    t0 = time.time()
    x = V.solve(A, bd, tag, P)
    torch.cuda.synchronize()
    r["bicgstab"] = {"s": time.time() - t0, "iters": tag.iters(),
                     "status": V.STATUS_NAMES[tag.status()],
                     "true_rel_residual": true_rel_residual(rp, ci, v, x.cpu().numpy(), b)}
    out["ilu_convdiff2d_512"] = r
    del A, P
    rp, ci, v = gen.laplace3d(128)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 1)
    A = V.compressed_matrix(rp, ci, v)
    bd = torch.tensor(b, device="cuda")
    torch.cuda.synchronize()
    t0 = time.time()
    P = V.chow_patel_icc_precond(A)
    torch.cuda.synchronize()
    r = {"rows": n, "setup_s": time.time() - t0}
    inf = P.info()
    z = bd.clone()
    t_apply = time_events(lambda: P.apply(z), 20)
    nb = inf.nnz_L * 12 + inf.nnz_U * 12 + 2 * (n + 1) * 4
    apply_bytes = 24 * n + steps * nb + 2 * steps * 24 * n + 8 * n
    r.update(apply_us=t_apply * 1e6, apply_bytes=int(apply_bytes),
             apply_GBs=apply_bytes / t_apply / 1e9,
             apply_frac_of_peak=apply_bytes / t_apply / 1e9 / peak)
    for name, pc in (("cg_ic0", P), ("cg_pipelined", None)):
        tag = V.cg_tag(1e-10, 5000)
        V.solve(A, bd, V.cg_tag(1e-10, 5000), pc)
        torch.cuda.synchronize()
        t0 = time.time()
        x = V.solve(A, bd, tag, pc)
        torch.cuda.synchronize()
        r[name] = {"s": time.time() - t0, "iters": tag.iters(),
                   "status": V.STATUS_NAMES[tag.status()],
                   "true_rel_residual": true_rel_residual(rp, ci, v, x.cpu().numpy(), b)}
    out["ic0_laplace3d_128"] = r
    return out


def bench_batched(V, torch):
    """4,096 systems (n log-uniform in [500, 20000]): one persistent launch
    against a loop of plain single-system solves (matrices prepared before
    the timed loop)."""
    t0 = time.time()
    rp, ci, v, sp, methods, b = gen.batch_systems(4096)
    gen_s = time.time() - t0
    A = V.compressed_matrix(rp, ci, v)
    bd = torch.tensor(b, device="cuda")
    bt = V.Batch(A, sp, methods)
    t0 = time.time()
    block, lanes = bt.tune(bd)
    tune_s = time.time() - t0
    bt.solve(bd, 1e-10, 20000)
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
        t0 = time.time()
        x, iters, status, err = bt.solve(bd, 1e-10, 20000)
        torch.cuda.synchronize()
        ts.append(time.time() - t0)
    t_batch = min(ts)
    # loop of plain solves over the same systems
    rp64 = rp.astype(np.int64)
    mats, rhs = [], []
    for k in range(len(methods)):
        r0, r1 = int(sp[k]), int(sp[k + 1])
        s, e = int(rp64[r0]), int(rp64[r1])
        Ak = V.compressed_matrix(torch.tensor((rp64[r0:r1 + 1] - s).astype(np.int32), device="cuda"),
                                 torch.tensor((ci[s:e].astype(np.int64) - r0).astype(np.int32), device="cuda"),
                                 torch.tensor(v[s:e], device="cuda"), r1 - r0, r1 - r0)
        mats.append(Ak)
        rhs.append(bd[r0:r1])
    torch.cuda.synchronize()
    t0 = time.time()
    loop_iters = []
    for k, Ak in enumerate(mats):
        tag = V.cg_tag(1e-10, 20000) if methods[k] == 0 else V.bicgstab_tag(1e-10, 20000)
        V.solve(Ak, rhs[k], tag)
        loop_iters.append(tag.iters())
    torch.cuda.synchronize()
    t_loop = time.time() - t0
    del mats
    # algorithmic bytes of the batch: per iteration of a system, its SpMV
    # (12 B/nnz + 20 B/row: values, indices, row pointers, x and y) and the
    # vector traffic of the pipelined recurrences (CG: 7 vectors; BiCGStab: two
    # SpMVs and 13 vectors), each vector counted once per pass; a system's
    # working set (at most 20,000 rows) stays in L2 during its solve, so this is
    # mostly L2 traffic and the HBM fraction is a lower bound of the work rate
    n_k = np.diff(sp.astype(np.int64))
    nnz_k = rp.astype(np.int64)[sp[1:].astype(np.int64)] - rp.astype(np.int64)[sp[:-1].astype(np.int64)]
    spmv_b = 12 * nnz_k + 20 * n_k
    per_it = np.where(methods == 0, spmv_b + 56 * n_k, 2 * spmv_b + 104 * n_k)
    alg_bytes = float(np.sum(per_it * iters.astype(np.int64)))
    li = np.array(loop_iters, dtype=np.int64)
    dev = np.abs(iters.astype(np.int64) - li) / np.maximum(li, 1)
    return {"systems": len(methods), "rows": int(sp[-1]), "nnz": int(rp[-1]), "generate_s": gen_s,
            "batched_s": t_batch, "loop_of_plain_solves_s": t_loop, "speedup": t_loop / t_batch,
            "tuned_block": block, "tuned_lanes": lanes, "tune_s": tune_s,
            "all_converged": bool((status == V.SUCCESS).all()),
            "iters_max": int(iters.max()), "iters_mean": float(iters.mean()),
            "iters_equal_to_loop": int(np.sum(li == iters)),
            "iters_worst_rel_dev_vs_loop": {"cg": float(dev[methods == 0].max()),
                                            "bicgstab": float(dev[methods == 1].max())},
            "algorithmic_bytes": alg_bytes, "algorithmic_GBs": alg_bytes / t_batch / 1e9,
            "bytes_note": "SpMV + recurrence vectors per iteration per system; mostly L2 traffic"}


def bench_adjoint(V, torch):
    """512^2 edge-coefficient diffusion: forward Jacobi-PCG to 1e-12, adjoint
    CG on A^T = A, gradient on the pattern; 8 central-difference checks."""
    N = 512
    rp, ci, v, (kx, ky) = gen.diffusion2d_edges(N, contrast=1e3, seed=4)
    n = len(rp) - 1
    rng = np.random.default_rng(4)
    b = rng.uniform(-1, 1, n)
    xt = rng.uniform(0, 1, n)
    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A)
    bd = torch.tensor(b, device="cuda")
    xtd = torch.tensor(xt, device="cuda")
    # warm-up of both directions (first-use costs are not part of a solve)
    xw = V.solve(A, bd, V.cg_tag(1e-12, 50000), P)
    V.solve_adjoint(A, xw, xw - xtd, V.cg_tag(1e-12, 50000), solver="cg", precond=P,
                    symmetric=True)
    torch.cuda.synchronize()
    t0 = time.time()
    tag = V.cg_tag(1e-12, 50000)
    x = V.solve(A, bd, tag, P)
    torch.cuda.synchronize()
    t_fwd = time.time() - t0
    t0 = time.time()
    atag = V.cg_tag(1e-12, 50000)
    lam, gA = V.solve_adjoint(A, x, x - xtd, atag, solver="cg", precond=P, symmetric=True)
    torch.cuda.synchronize()
    t_bwd = time.time() - t0
    lam, gA = lam.cpu().numpy(), gA.cpu().numpy()

    def loss(vals, bb):
        M = V.compressed_matrix(rp, ci, vals)
        xx = V.solve(M, bb, V.cg_tag(1e-13, 50000), V.jacobi_precond(M)).cpu().numpy()
        return 0.5 * np.sum((xx - xt) ** 2)

    worst = 0.0
    for d in range(8):
        rd = np.random.default_rng(1000 + d)
        if d % 2 == 0:
            db = rd.standard_normal(n)
            fd = (loss(v, b + 0.5 * db) - loss(v, b - 0.5 * db)) / 1.0
            an = lam @ db
        else:
            dkx, dky = rd.standard_normal(kx.shape) * kx, rd.standard_normal(ky.shape) * ky
            eps = 1e-4
            _, _, vp = gen._fv_diffusion(np.ones((N, N)), [kx + eps * dkx, ky + eps * dky])
            _, _, vm = gen._fv_diffusion(np.ones((N, N)), [kx - eps * dkx, ky - eps * dky])
            fd = (loss(vp, b) - loss(vm, b)) / (2 * eps)
            an = gA @ ((vp - vm) / (2 * eps))
        worst = max(worst, abs(fd - an) / abs(an))
    return {"rows": n, "forward_s": t_fwd, "forward_iters": tag.iters(), "adjoint_s": t_bwd,
            "adjoint_iters": atag.iters(), "fd_directions": 8, "fd_worst_rel_err": worst,
            "fd_64_directions": "tests/test_gpu_adjoint.py::test_finite_differences_spd_64_directions[512]"}


def true_rel_residual(rp, ci, v, x, b):
    """||b - A x|| / ||b|| in FP64 on the host (scipy), checked outside the timed region."""
    import scipy.sparse as sp
    n = len(rp) - 1
    A = sp.csr_matrix((np.asarray(v, np.float64), np.asarray(ci, np.int64), np.asarray(rp, np.int64)),
                      shape=(n, len(x)))
    r = np.asarray(b, np.float64) - A @ np.asarray(x, np.float64)
    return float(np.linalg.norm(r) / np.linalg.norm(b))


def cpu_baseline_cg(rp, ci, v, b, tol, maxit):
    import oracle
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    t0 = time.time()
    x, it, err = oracle.solve("cg", rp, ci, v, b, tol, maxit, "none")
    t = time.time() - t0
    return {"value": t, "unit": "s", "cores": cores, "kind": "port",
            "sample": "one full pipelined-CG solve of the headline workload (%d iterations)" % it,
            "iters": it}


def cpu_baseline_preconditioners():
    """The reference's host algorithms (C restatement, OpenMP on all host cores)
    for the preconditioner figures of the secondary section, on the same
    matrices: ILU0 (factorisation + level sets, level-scheduled apply), block
    ILU0 with 8 blocks, Chow-Patel ILU (3 sweeps, 2 Jacobi steps) on the 512^2
    convection-diffusion matrix, Chow-Patel IC0 on the 128^3 Laplacian.  Each
    apply is the mean of 5."""
    import oracle
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)

    def timed(fn, reps=1):
        t0 = time.time()
        for _ in range(reps):
            r = fn()
        return (time.time() - t0) / reps, r

    out = {"cores": cores, "kind": "port", "unit": "s"}
    rp, ci, v = gen.convdiff2d(512, 512, peclet=10.0, shift=0.01)
    b = gen.rhs_uniform(len(rp) - 1, 5)

    def ilu0_setup():
        lu = oracle.ilu0_factor(rp, ci, v)
        ud = oracle.diag(rp, ci, lu)
        return lu, ud, oracle.level_setup(rp, ci, lu, ud, False), oracle.level_setup(rp, ci, lu, ud, True)

    t_set, (lu, ud, L, U) = timed(ilu0_setup)
    t_app, _ = timed(lambda: oracle.level_substitute(U, oracle.level_substitute(L, b) / ud), 5)
    out["ilu0_convdiff2d_512"] = {"setup_s": t_set, "apply_s": t_app}
    t_set, B = timed(lambda: oracle.block_ilu0(rp, ci, v, num_blocks=8))
    t_app, _ = timed(lambda: oracle.block_ilu0_apply(B, b), 5)
    out["block_ilu8_convdiff2d_512"] = {"setup_s": t_set, "apply_s": t_app}
    t_set, F = timed(lambda: oracle.chow_patel_ilu(rp, ci, v, 3))
    t_app, _ = timed(lambda: oracle.chow_patel_apply(F, b, 2), 5)
    out["chow_patel_ilu_convdiff2d_512"] = {"setup_s": t_set, "apply_s": t_app}
    rp, ci, v = gen.laplace3d(128)
    b = gen.rhs_uniform(len(rp) - 1, 1)
    t_set, F = timed(lambda: oracle.chow_patel_icc(rp, ci, v, 3))
    t_app, _ = timed(lambda: oracle.chow_patel_apply(F, b, 2), 5)
    out["chow_patel_ic0_laplace3d_128"] = {"setup_s": t_set, "apply_s": t_app}
    return out


def run_reference(args):
    """The reference's own CPU algorithm (C restatement, OpenMP, all host cores)."""
    ws, rank, local = dist_setup("gloo")
    if rank != 0:
        return
    import oracle
    rp, ci, v = gen.laplace3d(128)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 1)
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    tol, maxit = 1e-10, 10000
    for _ in range(args.warmup):
        oracle.solve("cg", rp, ci, v, b, tol, maxit, "none")
    ts = []
    for _ in range(args.steps):
        t0 = time.time()
        x, it, err = oracle.solve("cg", rp, ci, v, b, tol, maxit, "none")
        ts.append(time.time() - t0)
    t = sum(ts) / len(ts)
    out = {"impl": "reference", "metric": METRIC, "value": t, "unit": "s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded generators, vclgb_gen.py)",
           "config": {"workload": WORKLOAD, "iterations": it,
                      "true_rel_residual": true_rel_residual(rp, ci, v, x, b)},
           "cpu_baseline": {"value": t, "unit": "s", "cores": cores, "kind": "port",
                            "sample": "full pipelined-CG solves of the headline workload"},
           "e2e": {"value": t, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def profile_kernels(args):
    """Small fixed workloads for ncu captures.  laplace: a few SpMVs per format
    on the 128^3 Laplacian (about 300 MB on the device), one short CG solve and
    a short refined solve on 96^3 diffusion; lognormal: a few SpMVs per format on a 1M-row lognormal random
    matrix (about 21M nnz, 250 MB of CSR arrays).

    The backend's kernel timing is on for these workloads: the solvers then
    run their iterations as host-polled graph chunks, whose kernels ncu
    profiles; it does not profile the kernels of a graph's device-side WHILE
    body, the solvers' loop otherwise."""
    import torch
    import vclgb as V
    V.backend().set_kernel_timing(True)
    if args.profile_case == "preconditioners":
        # three applies each of ILU0, block ILU0 (8 blocks) and Chow-Patel ILU on
        # the 512^2 convection-diffusion matrix, of Chow-Patel IC0 and ILU0 on 128^3
        rp, ci, v = gen.convdiff2d(512, 512, peclet=10.0, shift=0.01)
        A = V.compressed_matrix(rp, ci, v)
        z = torch.tensor(gen.rhs_uniform(len(rp) - 1, 5), device="cuda")
        for P in (V.ilu0_precond(A), V.block_ilu_precond(A, num_blocks=8),
                  V.chow_patel_ilu_precond(A)):
            for _ in range(3):
                P.apply(z)
        rp, ci, v = gen.laplace3d(128)
        A = V.compressed_matrix(rp, ci, v)
        z = torch.tensor(gen.rhs_uniform(len(rp) - 1, 1), device="cuda")
        P = V.chow_patel_icc_precond(A)
        for _ in range(3):
            P.apply(z)
        del P
        P = V.ilu0_precond(A)  # 3D levels: cluster runs
        for _ in range(3):
            P.apply(z)
        torch.cuda.synchronize()
        print("profile workload done")
        return
    if args.profile_case == "coverage":
        # one or a few launches of every kernel family outside the headline:
        # conversions and Jacobi-PCG (4 iterations) on the 128^3 Laplacian,
        # pipelined BiCGStab (4 iterations) and GMRES(30) (one cycle) on 2D
        # convection-diffusion 2048^2, a batch of 256 systems, and the adjoint's
        # transpose and gradient on 512^2 diffusion
        rp, ci, v = gen.laplace3d(128)
        A = V.compressed_matrix(rp, ci, v)
        fmts = [V.ell_matrix(A), V.sliced_ell_matrix(A, 32, 256), V.hyb_matrix(A),
                V.coordinate_matrix(A)]
        b = torch.tensor(gen.rhs_uniform(len(rp) - 1, 1), device="cuda")
        V.solve(A, b, V.cg_tag(1e-30, 4), V.jacobi_precond(A))
        del fmts, A
        rp, ci, v = gen.convdiff2d(2048, 2048, peclet=10.0, shift=0.01)
        A = V.compressed_matrix(rp, ci, v)
        b = torch.tensor(gen.rhs_uniform(len(rp) - 1, 3), device="cuda")
        V.solve(A, b, V.bicgstab_tag(1e-30, 4))
        V.solve(A, b, V.gmres_tag(1e-30, 30, 30))
        V.solve(A, b, V.gmres_tag(1e-30, 30, 30), V.jacobi_precond(A))
        del A
        rp, ci, v, sp, methods, bb = gen.batch_systems(256)
        A = V.compressed_matrix(rp, ci, v)
        bt = V.Batch(A, sp, methods)
        bt.solve(torch.tensor(bb, device="cuda"), 1e-10, 20000)
        del bt, A
        rp, ci, v, _ = gen.diffusion2d_edges(512, contrast=1e3, seed=4)
        A = V.compressed_matrix(rp, ci, v)
        b = torch.tensor(gen.rhs_uniform(len(rp) - 1, 4), device="cuda")
        x = V.solve(A, b, V.cg_tag(1e-6, 300), V.jacobi_precond(A))
        V.solve_adjoint(A, x, x - b, V.cg_tag(1e-6, 300), solver="cg")
        # small systems (70^2 = 4,900 rows) in one cluster launch each: CG,
        # Jacobi-PCG, BiCGStab, GMRES(20) (kernel timing off: it keeps the
        # per-phase path)
        V.backend().set_kernel_timing(False)
        rp, ci, v = gen.laplace2d(70, 70)
        A = V.compressed_matrix(rp, ci, v)
        b = torch.tensor(gen.rhs_uniform(len(rp) - 1, 5), device="cuda")
        V.solve(A, b, V.cg_tag(1e-10, 2000))
        V.solve(A, b, V.cg_tag(1e-10, 2000), V.jacobi_precond(A))
        rp, ci, v = gen.convdiff2d(70, 70, peclet=5.0, shift=0.05)
        A = V.compressed_matrix(rp, ci, v)
        V.solve(A, b, V.bicgstab_tag(1e-10, 2000))
        V.solve(A, b, V.gmres_tag(1e-10, 2000, 20))
        torch.cuda.synchronize()
        print("profile workload done")
        return
    if args.profile_case == "lognormal":
        rp, ci, v = gen.lognormal_random(1 << 20, mu=2.5, sigma=1.0, hi=2000, seed=1)
        n = len(rp) - 1
        A = V.compressed_matrix(rp, ci, v)
        x = torch.tensor(gen.rhs_uniform(n, 1), device="cuda")
        y = torch.empty(n, dtype=torch.float64, device="cuda")
        for M in (A, V.sliced_ell_matrix(A, 32, 256), V.hyb_matrix(A)):
            for _ in range(3):
                V.prod(M, x, y=y)
        torch.cuda.synchronize()
        print("profile workload done")
        return
    rp, ci, v = gen.laplace3d(128)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    x = torch.tensor(gen.rhs_uniform(n, 1), device="cuda")
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    for M in (A, V.ell_matrix(A), V.sliced_ell_matrix(A, 32, 1)):
        for _ in range(3):
            V.prod(M, x, y=y)
    V.solve(A, x, V.cg_tag(1e-10, 20))
    # a short refined solve (FP32 inner iterations on the DIA copy) on 96^3 diffusion
    rp2, ci2, v2, f2 = gen.diffusion3d(96)
    A2 = V.compressed_matrix(rp2, ci2, v2)
    V.solve(A2, f2, V.refined_cg_tag(1e-6, 60, 1e-4))
    torch.cuda.synchronize()
    print("profile workload done")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--profile-kernels", action="store_true",
                    help="run the small fixed workload used for ncu captures")
    ap.add_argument("--profile-case", default="laplace",
                    choices=["laplace", "lognormal", "preconditioners", "coverage"])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="headline only (for profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.profile_kernels:
        profile_kernels(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
