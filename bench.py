"""Benchmark: k=50 centred+scaled PCA time-to-tol (1e-5) on the 2,000-gene x
1.3M-cell, ~10%-dense synthetic count matrix (FP32 values), in the
FP32+FP64-steps form, with the plain FP64 GPU form and the CPU oracle timed
beside it.

One step = one full PCA to tolerance (column statistics, deferred centring and
scaling, the IRLBA restart loop, output assembly). The matrix is ~260M nonzeros,
larger than L2 (129 MB), so no flush is needed between steps.

Usage:
  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun (N > 1) every rank solves its own copy (replicas; the path has no
data-parallel exchange), the timing is the max over ranks.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "k=50 PCA time-to-tol (FP32+FP64-steps vs plain FP64, 1 GB300); SpMV HBM GB/s"
NUMBER = 50
TOL = 1e-5
# CPU reference solves: full solves to tolerance are repeated while they fit in
# this many seconds (at least one, at most --steps).
CPU_SOLVE_BUDGET_S = 180.0


T_START = time.time()


def log(msg):
    """Progress to stderr (the JSON line alone goes to stdout)."""
    print("[bench %7.1fs] %s" % (time.time() - T_START, msg), file=sys.stderr, flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cells", type=int, default=1300000)
    ap.add_argument("--genes", type=int, default=2000)
    ap.add_argument("--density", type=float, default=0.10)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 GPU comparator")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baselines")
    ap.add_argument("--no-extra", action="store_true",
                    help="default workload only: skip the 20k x 50k FP64, batched and adjoint sub-records")
    ap.add_argument("--cpu-restarts", type=int, default=2, help="restarts in the bounded CPU samples of the "
                    "secondary workloads")
    ap.add_argument("--workload", default="scrna_2k", choices=["scrna_2k", "batch", "adjoint", "csc20k"],
                    help="scrna_2k: the headline PCA (default); batch: 256 uneven PCAs in one persistent "
                         "launch; adjoint: truncated-SVD forward + backward; csc20k: plain FP64 PCA of the "
                         "20,000-gene x 50,000-cell matrix")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--coding", action="store_true",
                    help="dictionary-coded values for the FP32 matrix (off by default)")
    ap.add_argument("--spmv-shape", type=int, default=None,
                    help="SpMV launch shape of this run's FP32 matrices (see cppirlba_gb300.set_spmv_shape)")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x, device):
    """Largest value of x over the ranks of the default process group (x when
    there is none or it has one rank); the timed value is the slowest rank's."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        under = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(under), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# DRAM traffic of the SpMV pair per stored nonzero, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum) of the same kernels on the
# 800,000-cell case of the headline workload (160,011,127 nonzeros; multiply
# 973.8 MB, adjoint 967.8 MB per launch). The traffic is the stored bytes (FP32
# value + u16 panel offset) plus vectors, so it scales with the nonzeros.
SPMV_TRAFFIC_PER_NNZ = {"mul": 973.8e6 / 160011127, "adj": 967.8e6 / 160011127}


def spmv_alg_bytes(rows, cols, nnz, vec_bytes, val_bytes=4, idx_bytes=4):
    """Algorithmic bytes of one SpMV on the int32-index basis:
    nnz (val + idx) + (rows + 1) 8-byte pointers + input and output vectors."""
    return nnz * (val_bytes + idx_bytes) + (rows + 1) * 8 + (rows + cols) * vec_bytes


def solve_alg_bytes(m, n, nnz, steps, restarts, work, s_vec):
    """Algorithmic bytes of one whole solve, summed over the kernel classes:
    per Lanczos step one multiply and one adjoint SpMV (int32-index basis) and
    two CGS calls (W side, length m, and V side, length n: 2 c L s_vec + 3 L
    s_vec each, c the basis columns at that step); per restart the two
    rotations ((w + k) L s_vec for V and W). The columns per step and k are not
    recorded per restart: the first Lanczos run starts from k = 0 and the later
    ones from the mean k = work - (steps - work) / (restarts - 1)."""
    spmv = steps * (spmv_alg_bytes(m, n, nnz, s_vec) + spmv_alg_bytes(n, m, nnz, s_vec))
    later = max(restarts - 1, 0)
    kbar = work - (steps - work) / later if later else 0.0
    def run_cols(k):  # sum over j = k .. work - 1 of (j + 1)
        return (work - k) * (work + k + 1) / 2.0
    cols = run_cols(0) + later * run_cols(kbar)
    cgs = 2 * cols * (m + n) * s_vec + 3 * steps * (m + n) * s_vec
    rot = later * (work + kbar) * (m + n) * s_vec
    return {"spmv": spmv, "cgs": cgs, "rotation": rot, "total": spmv + cgs + rot}


def vendor_spmv_ms(inp, reps=5, device="cuda"):
    """cuSPARSE CSR SpMV through torch (a vendor reference bar for the gather
    kernel): best of `reps` products y = A x and y = A^T x on the same FP32
    matrix, with A^T built on the device by a transpose."""
    import warnings
    import torch
    primary = len(inp.ptr) - 1
    secondary = inp.nrow if inp.column_major else inp.ncol
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")   # torch's beta-status notice for sparse CSR
        P = torch.sparse_csr_tensor(torch.tensor(inp.ptr, dtype=torch.int64, device=device),
                                    torch.tensor(inp.idx, dtype=torch.int64, device=device),
                                    torch.tensor(inp.val, dtype=torch.float32, device=device),
                                    size=(primary, secondary))
        T = P.to_sparse_coo().t().coalesce().to_sparse_csr()
    A, At = (T, P) if inp.column_major else (P, T)
    out = {}
    for name, M in (("multiply", A), ("adjoint", At)):
        x = torch.randn(M.shape[1], 1, device=device)
        best = None
        for _ in range(reps + 1):
            if device == "cuda":
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                y = torch.sparse.mm(M, x)
                e1.record()
                torch.cuda.synchronize()
                t = e0.elapsed_time(e1)
            else:
                t0 = time.perf_counter()
                y = torch.sparse.mm(M, x)
                t = (time.perf_counter() - t0) * 1e3
            best = t if best is None else min(best, t)
        assert y.shape[0] == M.shape[0]
        out[name] = best
    del A, At, P, T
    if device == "cuda":
        torch.cuda.empty_cache()
    return out


def make_input(args):
    from cppirlba_gb300 import datagen
    return datagen.scrna_pca_input(args.genes, args.cells, args.density, args.seed, np.float32, cell_major=False)


def cpu_solve(inp, init, threads, max_restarts=-1):
    """The oracle's pca() (CppIrlba's pca.hpp:55-139 restated, FP64 arithmetic,
    ParallelSparseMatrix products on `threads` OpenMP threads) on the same
    matrix: FP32 values stay FP32 in memory (a float value array, as the
    reference's ParallelSparseMatrix accepts) and are promoted to FP64 in every
    product. Runs to tolerance unless max_restarts >= 0. Returns (seconds,
    result dict)."""
    import oracle
    spec = oracle.Spec.sparse(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major, threads)
    t0 = time.perf_counter()
    r = oracle.pca(spec, True, True, NUMBER, oracle.options(initial=init, convergence_tolerance=TOL),
                   dense_threads=threads, max_restarts=max_restarts)
    return time.perf_counter() - t0, r


def run_reference(args):
    """CPU reference arm: the oracle's full pca() to tolerance on the host cores.
    One step = one whole solve (column statistics, the restart loop to tol 1e-5,
    output assembly), measured, not extrapolated. A full solve takes tens of
    seconds, so the requested --steps/--warmup are capped: one short warm-up
    sample (statistics + one restart, to page the matrix in), then full solves
    while they fit in CPU_SOLVE_BUDGET_S (at least one). The input comes from
    the generator compiled into the oracle library: no product library is
    loaded."""
    world, rank, local = dist_setup()
    if rank != 0:
        return
    import oracle
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    inp = oracle.scrna_pca_input(args.genes, args.cells, args.density, args.seed, np.float32, cell_major=False)
    t_gen = time.perf_counter() - t0
    init = np.random.default_rng(12345).standard_normal(inp.ncol)
    log("reference: generated %d x %d, nnz %d in %.1f s" % (inp.nrow, inp.ncol, inp.nnz, t_gen))
    warm = 0
    if args.warmup > 0:
        dt, _ = cpu_solve(inp, init, threads, max_restarts=1)
        warm = 1
        log("reference warm-up sample (statistics + 1 restart) %.1f s" % dt)
    times, res = [], None
    t_all = time.perf_counter()
    while len(times) < max(1, args.steps):
        dt, res = cpu_solve(inp, init, threads)
        times.append(dt)
        log("reference solve %d: %.1f s, %d restarts, %d Lanczos steps, converged %s" %
            (len(times), dt, res["iterations"], res["lanczos_steps"], res["converged"]))
        if (time.perf_counter() - t_all) + dt > CPU_SOLVE_BUDGET_S:
            break
    value = statistics.median(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": world,
        "steps": len(times), "warmup": warm, "steps_requested": args.steps, "warmup_requested": args.warmup,
        "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (same seeded matrix and start vector as the GPU arm)",
        "config": {"workload": "scrna_csr_2k: %d genes x %d cells (CSC cells x genes), density %.2f, nnz %d, "
                               "FP32 values; centred+scaled PCA k=%d, extra_work 7, tol %.0e" %
                               (args.genes, args.cells, args.density, inp.nnz, NUMBER, TOL),
                   "form": "fp64 (the reference's arithmetic)", "parallelism": "%d host threads" % threads},
        "converged": res["converged"], "restarts": res["iterations"], "lanczos_steps": res["lanczos_steps"],
        "solve_s": times,
        "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port",
                         "sample": "full pca() to tol, measured (%d solve(s), median): oracle = CppIrlba's "
                                   "compute/lanczos/pca restated in C++, ParallelSparseMatrix products and dense "
                                   "GEMV/GEMM on %d OpenMP threads" % (len(times), threads)},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _stream_ptr(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def run_batch(args):
    """Batched form: 256 sparse FP32 matrices of 2,000 genes x n_j cells (n_j
    lognormal, median 5,000, clamped to [200, 50,000]), density 8 %; centred
    PCA k=20, extra_work 7 for every matrix, one persistent launch replayed from
    a captured CUDA graph. One step = one batch solve."""
    import torch
    import cppirlba_gb300 as eng
    from cppirlba_gb300 import datagen
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    k = 20
    t0 = time.perf_counter()
    sizes = datagen.batched_sizes(count=args.batch_count)
    inputs = datagen.scrna_batch(sizes, genes=2000, density=0.08, seed=4)
    t_gen = time.perf_counter() - t0
    nnz = np.array([x.nnz for x in inputs], dtype=np.int64)
    log("generated %d matrices, cells %d..%d (median %d), nnz %d in %.1f s" %
        (len(inputs), sizes.min(), sizes.max(), int(np.median(sizes)), nnz.sum(), t_gen))
    mats = [(x.nrow, x.ncol, x.val, x.idx, x.ptr) for x in inputs]
    t0 = time.perf_counter()
    batch = eng.Batch(mats, True)
    t_ing = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    opts = eng.Options()
    for w in range(args.warmup):
        st = batch.pca(True, False, k, opts, stream=_stream_ptr(torch))
        log("warmup %d: %.1f ms device, tune %.1f ms, captured %d, single %d" %
            (w, st["device_ms"], st["tune_ms"], st["graph_captured"], st["single"]))
    clocks = Clocks(local)
    torch.cuda.synchronize()
    clocks.start()
    launches0 = eng.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        st = batch.pca(True, False, k, opts, stream=_stream_ptr(torch))
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = eng.launch_count() - launches0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    infos = [batch.result(j).stats for j in range(len(inputs))]
    steps = np.array([i["lanczos_steps"] for i in infos], dtype=np.int64)
    per_ms = np.array([i["ms"] for i in infos])
    conv = sum(i["converged"] for i in infos)
    gm, ga = batch.groups()
    # Algorithmic bytes: per Lanczos step one multiply and one adjoint SpMV
    # (int32-index basis) of that matrix.
    alg = float(sum(steps[j] * (spmv_alg_bytes(sizes[j], 2000, nnz[j], 4) + spmv_alg_bytes(2000, sizes[j], nnz[j], 4))
                    for j in range(len(inputs))))
    peak, peak_kind = load_peaks()
    achieved = alg / (st["device_ms"] * 1e-3) / 1e9
    out = {
        "metric": "batched centred PCA k=20 (256 uneven sparse matrices, one persistent launch) time",
        "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (FP64 coefficients, norms, recurrence, restart SVD)",
        "data": "synthetic (seeded scRNA-like log1p negative-binomial counts; no dataset)",
        "config": {"workload": "batch_256: %d matrices of 2000 genes x n_j cells, n_j lognormal(median 5000, "
                               "sigma 1) clamped to [200, 50000], density 0.08, FP32; centred PCA k=%d, "
                               "extra_work 7, tol 1e-5" % (len(inputs), k),
                   "total_nnz": int(nnz.sum()), "total_cells": int(sizes.sum()),
                   "l2_flush": "inputs larger than L2 (%.1f GB stored)" % (nnz.sum() * 12 / 1e9),
                   "parallelism": "single GPU; cluster teams of 1, 2 or 4 CTAs for the largest matrices, "
                                  "one CTA per matrix for the rest"},
        "converged": int(conv), "single_matrix_resolves": st["single"], "ctas": st["ctas"],
        "team_ctas": st.get("team"), "joint_matrices": st.get("joint"),
        "lanczos_steps_total": int(steps.sum()),
        "per_matrix_ms": {"min": float(per_ms.min()), "median": float(np.median(per_ms)),
                          "p90": float(np.percentile(per_ms, 90)), "max": float(per_ms.max()),
                          "sum": float(per_ms.sum())},
        "schedules": {"group_mul": {str(g): int((gm == g).sum()) for g in (4, 8, 16, 32)},
                      "group_adj": {str(g): int((ga == g).sum()) for g in (4, 8, 16, 32)},
                      "prefetch_mul": {str(p): int(sum(i["prefetch_mul"] == p for i in infos)) for p in (0, 1, 3)},
                      "prefetch_adj": {str(p): int(sum(i["prefetch_adj"] == p for i in infos)) for p in (0, 1, 3)}},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "batch_pca_kernel (persistent; SpMV pairs dominate)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None,
                     "alg_bytes_per_launch": alg},
        "clocks": clk,
        "setup_s": {"generate": t_gen, "ingest": t_ing},
    }
    if not args.no_e2e:
        h0, d0 = eng.transfer_bytes()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b2 = eng.Batch(mats, True)
        b2.pca(True, False, k, opts)
        for j in range(len(inputs)):
            b2.result(j)
        b2.close()
        e2e = time.perf_counter() - t0
        h1, d1 = eng.transfer_bytes()
        out["e2e"] = {"value": e2e, "unit": "s", "h2d_bytes_per_step": h1 - h0, "d2h_bytes_per_step": d1 - d0,
                      "note": "create (host ingestion of both directions, H2D), autotune, graph capture, solve, "
                              "D2H of every matrix's scores, rotation, variances"}
    if not args.no_cpu and rank == 0:
        import oracle
        threads = os.cpu_count() or 1
        order = np.argsort(sizes)
        pick = order[np.linspace(0, len(order) - 1, 5).astype(int)]
        t_cpu, w_cpu = 0.0, 0.0
        for j in pick:
            x = inputs[j]
            spec = oracle.Spec.sparse(x.nrow, x.ncol, x.val.astype(np.float64), x.idx, x.ptr, x.column_major, threads)
            t0 = time.perf_counter()
            oracle.pca(spec, True, False, k, oracle.options(), dense_threads=threads)
            t_cpu += time.perf_counter() - t0
            w_cpu += nnz[j]
        est = t_cpu * float(nnz.sum()) / w_cpu
        out["cpu_baseline"] = {"value": est, "unit": "s", "cores": threads, "kind": "port",
                               "sample": "FP64 oracle pca() (CppIrlba algorithm restated, OpenMP) of 5 matrices at "
                                         "size quantiles (%.1f s), scaled by total nnz / sample nnz" % t_cpu}
    return out


def run_adjoint(args):
    """Differentiation form: loss = sum w_i sigma_i + ||G^T U||_F^2 on the dense
    FP32 4096 x 1024 matrix with planted spectrum sigma_i = 50 / i plus
    N(0, 0.01) noise, k = 32; one step = forward (top-k SVD, FP32 form) +
    backward (truncated-SVD adjoint through the libtorch autograd Function)."""
    import torch
    import cppirlba_gb300 as eng
    from cppirlba_gb300 import autograd as ag
    from cppirlba_gb300 import datagen
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    eng.load_library()
    ag.load_extension()
    k = 32
    A = datagen.adjoint_dense(4096, 1024, seed=5)
    rng = np.random.default_rng(6)
    G = torch.tensor(rng.standard_normal((4096, k)), device="cuda", dtype=torch.float32)
    w = torch.tensor(rng.uniform(0.5, 1.5, k), device="cuda", dtype=torch.float32)
    At = torch.tensor(A, device="cuda", requires_grad=True)
    stream = torch.cuda.current_stream()

    def step():
        At.grad = None
        U, S, V = ag.truncated_svd(At, k, tol=1e-6)
        e_mid = torch.cuda.Event(enable_timing=True)
        e_mid.record(stream)
        L = (w * S).sum() + ((G.T @ U) ** 2).sum()
        L.backward()
        return e_mid

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    launches0 = eng.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    fwd = []
    ev0.record(stream)
    for _ in range(args.steps):
        e_start = torch.cuda.Event(enable_timing=True)
        e_start.record(stream)
        e_mid = step()
        torch.cuda.synchronize()
        fwd.append(e_start.elapsed_time(e_mid))
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = eng.launch_count() - launches0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    fwd_ms = statistics.median(fwd)
    # FP64 reference gradient from torch's autograd through a full SVD.
    Ar = torch.tensor(A, device="cuda", dtype=torch.float64, requires_grad=True)
    Ur, Sr, _ = torch.linalg.svd(Ar, full_matrices=False)
    ((w.double() * Sr[:k]).sum() + ((G.double().T @ Ur[:, :k]) ** 2).sum()).backward()
    rel = float(torch.linalg.norm(At.grad.double() - Ar.grad) / torch.linalg.norm(Ar.grad))
    out = {
        "metric": "differentiable truncated SVD (k=32) forward + backward time",
        "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 forward (FP64 steps), f64 adjoint",
        "data": "synthetic (planted spectrum sigma_i = 50/i plus N(0, 0.01) noise, seeded)",
        "config": {"workload": "adjoint_dense: 4096 x 1024 FP32, k=32, loss sum w_i sigma_i + ||G^T U||_F^2, "
                               "forward tol 1e-6, complement CG tol 1e-8",
                   "parallelism": "single GPU"},
        "forward_ms": fwd_ms, "backward_ms": ms - fwd_ms,
        "grad_rel_err_vs_fp64_full_svd": rel,
        "gpu_launches": launches, "clocks": clk,
    }
    if not args.no_cpu and rank == 0:
        from oracle import svd_adjoint as sa
        t0 = time.perf_counter()
        U0, S0, V0 = sa.top_k_svd(A.astype(np.float64), k)
        Gn, wn = G.double().cpu().numpy(), w.double().cpu().numpy()
        sa.truncated_svd_grad(A.astype(np.float64), k, 2 * Gn @ (Gn.T @ U0), wn, None, exact=False)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": dt, "unit": "s", "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": "numpy oracle: full LAPACK SVD + F-matrix and rank-k projection terms "
                                         "(the exact complement solve is O(m^3) there and is not timed)"}
    return out


def run_csc20k(args):
    """Plain FP64 form: centred+scaled PCA k=50 (tol 1e-5) of the 20,000-gene x
    50,000-cell, ~5 %-dense CSC count matrix with FP64 values (cells x genes
    CSR as the PCA input), against the FP64 oracle on the host cores. One step =
    one PCA to tolerance on device-resident data."""
    import torch
    import cppirlba_gb300 as eng
    from cppirlba_gb300 import datagen
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    lib = eng.load_library()
    t0 = time.perf_counter()
    inp = datagen.scrna_csc_20k()
    t_gen = time.perf_counter() - t0
    m, n, nnz = inp.nrow, inp.ncol, inp.nnz
    log("generated %d x %d, nnz %d in %.1f s" % (m, n, nnz, t_gen))
    init = datagen.start_vector(n)
    opts = eng.Options(initial=init, convergence_tolerance=TOL)
    t0 = time.perf_counter()
    mat = eng.ParallelSparseMatrix(m, n, inp.val, inp.idx, inp.ptr, inp.column_major, form=eng.FORM_FP64)
    t_ing = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    dU = torch.empty(m * NUMBER, dtype=torch.float64, device="cuda")
    dV = torch.empty(n * NUMBER, dtype=torch.float64, device="cuda")
    dD = torch.empty(NUMBER, dtype=torch.float64, device="cuda")

    def solve(profile=False):
        keep = []
        o = opts._to_c(keep)
        num, conv, iters, st = ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32(), eng.Stats()
        eng.set_profiling(profile)
        rc = lib.irlba_gb300_pca_device(mat.handle, 1, 1, NUMBER, ctypes.byref(o), ctypes.c_void_p(dU.data_ptr()),
                                        ctypes.c_void_p(dV.data_ptr()), ctypes.c_void_p(dD.data_ptr()),
                                        ctypes.byref(num), ctypes.byref(conv), ctypes.byref(iters), ctypes.byref(st),
                                        ctypes.c_void_p(stream.cuda_stream))
        eng.set_profiling(False)
        eng._check(rc)
        return iters.value, bool(conv.value), eng._stats_dict(st)

    for _ in range(args.warmup):
        solve()
    clocks = Clocks(local)
    torch.cuda.synchronize()
    clocks.start()
    launches0 = eng.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    prof = {k: [0.0, 0] for k in ["spmv_mul", "spmv_adj", "cgs", "restart", "rotate", "other"]}
    ev0.record(stream)
    for _ in range(args.steps):
        iters, conv, st = solve(profile=True)
        pr = eng.last_profile()
        for k in prof:
            prof[k][0] += pr[k]["ms"]
            prof[k][1] += pr[k]["launches"]
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = eng.launch_count() - launches0
    clk = clocks.stop()
    ms = reduce_max(ev0.elapsed_time(ev1), "cuda") / args.steps
    b_mul = spmv_alg_bytes(m, n, nnz, 8, val_bytes=8)
    b_adj = spmv_alg_bytes(n, m, nnz, 8, val_bytes=8)
    t_mul = prof["spmv_mul"][0] / max(prof["spmv_mul"][1], 1)
    t_adj = prof["spmv_adj"][0] / max(prof["spmv_adj"][1], 1)
    both = (b_mul + b_adj) / ((t_mul + t_adj) * 1e-3) / 1e9 if t_mul + t_adj > 0 else None
    peak, peak_kind = load_peaks()
    out = {
        "metric": "k=50 PCA time-to-tol, plain FP64 form (20,000 genes x 50,000 cells)",
        "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded scRNA-like log1p negative-binomial counts; no dataset)",
        "config": {"workload": "scrna_csc_20k: 20000 genes x 50000 cells CSC (cells x genes CSR input), density "
                               "0.05, nnz %d, FP64 values; centred+scaled PCA k=%d, extra_work 7, tol %.0e" %
                               (nnz, NUMBER, TOL),
                   "form": "fp64", "l2_flush": "inputs larger than L2 (%.2f GB per SpMV)" % (b_mul / 1e9),
                   "parallelism": "single GPU"},
        "converged": conv, "restarts": iters, "lanczos_steps": st["lanczos_steps"],
        "gpu_launches": launches,
        "kernel_ms_per_step": {k: v[0] / args.steps for k, v in prof.items()},
        "roofline": {"bound": "hbm", "kernel": "spmv (multiply + adjoint, fused centre/scale)", "achieved": both,
                     "peak": peak, "unit": "GB/s", "frac": both / peak if both else None, "peak_source": peak_kind,
                     "traffic": None, "avg_launch_ms": {"mul": t_mul, "adj": t_adj}},
        "clocks": clk, "setup_s": {"generate": t_gen, "ingest": t_ing},
    }
    if not args.no_e2e:
        def e2e_step():
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            mt = eng.ParallelSparseMatrix(m, n, inp.val, inp.idx, inp.ptr, inp.column_major, form=eng.FORM_FP64)
            eng.pca(mt, True, True, NUMBER, opts)
            mt.close()
            torch.cuda.synchronize()
            return time.perf_counter() - t1
        e2e_step()
        h0, d0 = eng.transfer_bytes()
        times = [e2e_step() for _ in range(max(1, args.steps))]
        h1, d1 = eng.transfer_bytes()
        out["e2e"] = {"value": reduce_max(statistics.median(times), "cuda"), "unit": "s",
                      "h2d_bytes_per_step": (h1 - h0) // len(times), "d2h_bytes_per_step": (d1 - d0) // len(times)}
    if not args.no_cpu and rank == 0:
        # One full FP64 oracle solve to tolerance (measured), also the parity
        # check of the GPU result at this size.
        import oracle
        threads = os.cpu_count() or 1
        spec = oracle.Spec.sparse(m, n, inp.val, inp.idx, inp.ptr, inp.column_major, threads)
        t1 = time.perf_counter()
        r = oracle.pca(spec, True, True, NUMBER, oracle.options(initial=init, convergence_tolerance=TOL),
                       dense_threads=threads)
        dt = time.perf_counter() - t1
        D_gpu = np.sqrt(dD.cpu().numpy() * (m - 1))
        D_orc = np.sqrt(np.asarray(r["variances"]) * (m - 1))
        out["cpu_baseline"] = {"value": dt, "unit": "s", "cores": threads, "kind": "port",
                               "sample": "one full FP64 oracle pca() to tol, measured: %d restarts, %d Lanczos "
                                         "steps, converged %s" % (r["iterations"], r["lanczos_steps"], r["converged"])}
        out["D_max_rel_err_vs_fp64_oracle"] = float(np.max(np.abs(D_gpu - D_orc) / D_orc))
        out["restarts_equal_oracle"] = iters == r["iterations"]
    return out


def sub_args(args):
    """Step counts of the secondary workloads inside the default run: a few
    timed steps each, so the whole default run stays within minutes."""
    sub = argparse.Namespace(**vars(args))
    sub.steps = max(1, min(args.steps, 3))
    sub.warmup = max(1, min(args.warmup, 1))
    return sub


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    standalone = {"batch": run_batch, "adjoint": run_adjoint, "csc20k": run_csc20k}
    if args.workload in standalone:
        out = standalone[args.workload](args)
        if dist_setup()[1] == 0:
            print(json.dumps(out), flush=True)
        return
    world, rank, local = dist_setup()
    import torch
    import cppirlba_gb300 as eng
    from cppirlba_gb300 import datagen
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(x):
        return reduce_max(x, "cuda")

    eng.load_library()
    if args.spmv_shape is not None:
        eng.set_spmv_shape(args.spmv_shape)
    if args.coding:
        eng.set_value_coding(True)
    t_gen = time.perf_counter()
    inp = make_input(args)
    t_gen = time.perf_counter() - t_gen
    log("generated %d x %d, nnz %d in %.1f s" % (inp.nrow, inp.ncol, inp.nnz, t_gen))
    init = datagen.start_vector(inp.ncol)
    m, n, nnz = inp.nrow, inp.ncol, inp.nnz
    opts = eng.Options(initial=init, convergence_tolerance=TOL)

    # Device-resident matrix for the timed value.
    t_ing = time.perf_counter()
    mat32 = eng.ParallelSparseMatrix(m, n, inp.val, inp.idx, inp.ptr, inp.column_major,
                                     form=eng.FORM_FP32_FP64STEPS)
    t_ing = time.perf_counter() - t_ing
    log("ingested FP32 form in %.1f s" % t_ing)
    lay = mat32.layout()
    stream = torch.cuda.current_stream()
    dU = torch.empty(m * NUMBER, dtype=torch.float64, device="cuda")
    dV = torch.empty(n * NUMBER, dtype=torch.float64, device="cuda")
    dD = torch.empty(NUMBER, dtype=torch.float64, device="cuda")
    lib = eng.load_library()

    def solve(matrix, profile=False):
        """One PCA step on device-resident data: statistics + compute + scores."""
        keep = []
        o = opts._to_c(keep)
        num = ctypes.c_int64()
        conv = ctypes.c_int32()
        iters = ctypes.c_int32()
        st = eng.Stats()
        eng.set_profiling(profile)
        rc = lib.irlba_gb300_pca_device(matrix.handle, 1, 1, NUMBER, ctypes.byref(o), ctypes.c_void_p(dU.data_ptr()),
                                        ctypes.c_void_p(dV.data_ptr()), ctypes.c_void_p(dD.data_ptr()),
                                        ctypes.byref(num), ctypes.byref(conv), ctypes.byref(iters),
                                        ctypes.byref(st), ctypes.c_void_p(stream.cuda_stream))
        eng.set_profiling(False)
        eng._check(rc)
        return {"converged": bool(conv.value), "iterations": iters.value, "stats": eng._stats_dict(st)}

    for w in range(args.warmup):
        r = solve(mat32)
        log("warmup %d: %d restarts, converged %s, %.1f ms" % (w, r["iterations"], r["converged"],
                                                              r["stats"]["device_ms"]))
    clocks = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    launches0 = eng.launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    results = []
    prof_ms = {k: 0.0 for k in ["spmv_mul", "spmv_adj", "cgs", "restart", "rotate", "other"]}
    prof_launch = dict(prof_ms)
    for _ in range(args.steps):
        results.append(solve(mat32, profile=True))
        log("step: %d restarts, %.1f ms" % (results[-1]["iterations"], results[-1]["stats"]["device_ms"]))
        pr = eng.last_profile()
        for k in prof_ms:
            prof_ms[k] += pr[k]["ms"]
            prof_launch[k] += pr[k]["launches"]
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = eng.launch_count() - launches0
    clk = clocks.stop()
    ms_total = max_over_ranks(ev0.elapsed_time(ev1))
    ms_per_step = ms_total / args.steps
    D32 = dD.cpu().numpy().copy()
    last = results[-1]

    # Roofline of the dominant kernel class (the SpMV pair), from the CUDA-event
    # durations measured inside the timed steps.
    mul_launch = max(prof_launch["spmv_mul"], 1)
    adj_launch = max(prof_launch["spmv_adj"], 1)
    b_mul = spmv_alg_bytes(m, n, nnz, 4)
    b_adj = spmv_alg_bytes(n, m, nnz, 4)
    t_mul = prof_ms["spmv_mul"] / mul_launch
    t_adj = prof_ms["spmv_adj"] / adj_launch
    peak, peak_kind = load_peaks()
    gbs_mul = b_mul / (t_mul * 1e-3) / 1e9 if t_mul > 0 else None
    gbs_adj = b_adj / (t_adj * 1e-3) / 1e9 if t_adj > 0 else None
    both = (b_mul + b_adj) / ((t_mul + t_adj) * 1e-3) / 1e9 if t_mul + t_adj > 0 else None
    actual_bytes = nnz * (lay["value_bytes"] + lay["index_bytes_mul"]) + nnz * (lay["value_bytes"] + lay["index_bytes_adj"])

    out = {
        "metric": METRIC,
        "value": ms_per_step / 1e3,
        "unit": "s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (FP64 coefficients, norms, recurrence, restart SVD)",
        "data": "synthetic (seeded scRNA-like log1p negative-binomial counts; no dataset)",
        "config": {"workload": "scrna_csr_2k: %d genes x %d cells (CSC cells x genes), density %.2f, nnz %d, "
                               "FP32 values; centred+scaled PCA k=%d, extra_work 7, tol %.0e" %
                               (args.genes, args.cells, args.density, nnz, NUMBER, TOL),
                   "form": "fp32_fp64steps", "l2_flush": "inputs larger than L2 (%.1f GB per SpMV)" % (b_mul / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "converged": last["converged"],
        "restarts": last["iterations"],
        "lanczos_steps": last["stats"]["lanczos_steps"],
        "matvecs": last["stats"]["matvecs"],
        "svd_sweeps_per_restart": last["stats"]["svd_sweeps"] / max(last["iterations"], 1),
        "gpu_launches": launches,
        "kernel_ms_per_step": {k: v / args.steps for k, v in prof_ms.items()},
        "roofline": {"bound": "hbm", "kernel": "spmv (multiply + adjoint, fused centre/scale)",
                     "achieved": both, "peak": peak, "unit": "GB/s",
                     "frac": (both / peak) if both else None, "peak_source": peak_kind,
                     "traffic": 0.5 * (SPMV_TRAFFIC_PER_NNZ["mul"] + SPMV_TRAFFIC_PER_NNZ["adj"]) * nnz,
                     "traffic_source": "ncu DRAM bytes per nonzero on the 800,000-cell case, scaled by nonzeros",
                     "traffic_per_launch": {k: v * nnz for k, v in SPMV_TRAFFIC_PER_NNZ.items()},
                     # DRAM bandwidth actually drawn (traffic / launch time): the
                     # int32-index algorithmic basis above counts 8 B per nonzero,
                     # the stored layout moves about 6.
                     "traffic_gbs": ((SPMV_TRAFFIC_PER_NNZ["mul"] + SPMV_TRAFFIC_PER_NNZ["adj"]) * nnz /
                                     ((t_mul + t_adj) * 1e-3) / 1e9) if t_mul + t_adj > 0 else None,
                     "traffic_frac": ((SPMV_TRAFFIC_PER_NNZ["mul"] + SPMV_TRAFFIC_PER_NNZ["adj"]) * nnz /
                                      ((t_mul + t_adj) * 1e-3) / 1e9 / peak) if t_mul + t_adj > 0 and peak else None,
                     "achieved_mul": gbs_mul, "achieved_adj": gbs_adj,
                     "alg_bytes_per_launch": {"mul": b_mul, "adj": b_adj},
                     "stored_bytes_per_nnz": {"mul": lay["value_bytes"] + lay["index_bytes_mul"],
                                              "adj": lay["value_bytes"] + lay["index_bytes_adj"]},
                     "avg_launch_ms": {"mul": t_mul, "adj": t_adj}},
        "clocks": clk,
        "setup_s": {"generate": t_gen, "ingest_fp32": t_ing},
    }

    # Whole solve against the roofline (an estimate: see solve_alg_bytes) and a
    # vendor bar for the sparse product.
    try:
        est = solve_alg_bytes(m, n, nnz, last["stats"]["lanczos_steps"], last["iterations"], NUMBER + 7, 4)
        out["solve_roofline"] = {"alg_bytes": est, "achieved_gbs": est["total"] / (ms_per_step * 1e-3) / 1e9,
                                 "frac": est["total"] / (ms_per_step * 1e-3) / 1e9 / peak if peak else None,
                                 "note": "algorithmic bytes of all SpMV, CGS and rotation launches of one solve "
                                         "(int32-index basis) / time to tol / measured copy peak"}
    except Exception as exc:
        out["solve_roofline"] = {"error": "%s: %s" % (type(exc).__name__, exc)}
    if rank == 0:
        try:
            v = vendor_spmv_ms(inp)
            out["vendor_spmv_ms"] = {"library": "cuSPARSE CSR SpMV through torch.sparse.mm (FP32, int64 indices)",
                                     "multiply": v["multiply"], "adjoint": v["adjoint"],
                                     "this_engine": {"multiply": t_mul, "adjoint": t_adj}}
        except Exception as exc:
            out["vendor_spmv_ms"] = {"error": "%s: %s" % (type(exc).__name__, exc)}

    # End to end through the public API with host buffers: ingestion (H2D of the
    # compressed matrix), PCA, D2H of scores, rotation and variances.
    if not args.no_e2e:
        def e2e_step():
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            mtmp = eng.ParallelSparseMatrix(m, n, inp.val, inp.idx, inp.ptr, inp.column_major,
                                            form=eng.FORM_FP32_FP64STEPS)
            eng.pca(mtmp, True, True, NUMBER, opts)
            mtmp.close()
            torch.cuda.synchronize()
            return time.perf_counter() - t0

        log("e2e warmup %.2f s" % e2e_step())
        e2e_times = []
        h0, d0 = eng.transfer_bytes()
        n_e2e = max(1, args.steps)
        for _ in range(n_e2e):
            e2e_times.append(e2e_step())
            log("e2e step %.2f s" % e2e_times[-1])
        h1, d1 = eng.transfer_bytes()
        e2e = max_over_ranks(statistics.median(e2e_times))
        out["e2e"] = {"value": e2e, "unit": "s", "h2d_bytes_per_step": (h1 - h0) // n_e2e,
                      "d2h_bytes_per_step": (d1 - d0) // n_e2e,
                      "note": "ParallelSparseMatrix from host arrays (H2D of the compressed matrix, device "
                              "transpose and panel layout) + pca() + D2H of scores, rotation, variances"}

    # Plain FP64 GPU form on the same matrix (values promoted to FP64).
    if not args.no_fp64:
        vals64 = inp.val.astype(np.float64)
        mat64 = eng.ParallelSparseMatrix(m, n, vals64, inp.idx, inp.ptr, inp.column_major, form=eng.FORM_FP64)
        del vals64
        log("ingested FP64 form")
        r = solve(mat64)
        log("fp64 warmup: %d restarts, %.1f ms" % (r["iterations"], r["stats"]["device_ms"]))
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r64 = solve(mat64, profile=True)
        e1.record(stream)
        torch.cuda.synchronize()
        pr64 = eng.last_profile()
        ms64 = e0.elapsed_time(e1)
        D64 = dD.cpu().numpy().copy()
        out["fp64_gpu"] = {"time_to_tol_s": ms64 / 1e3, "restarts": r64["iterations"],
                           "lanczos_steps": r64["stats"]["lanczos_steps"], "converged": r64["converged"],
                           "kernel_ms": {k: v["ms"] for k, v in pr64.items()},
                           "speedup_fp32_form": ms64 / ms_per_step,
                           "fp32_D_max_rel_err_vs_fp64": float(np.max(np.abs(np.sqrt(D32) - np.sqrt(D64)) /
                                                                     np.sqrt(D64)))}
        mat64.close()

    # The FP64 oracle on the host cores: one full solve to tolerance (measured),
    # also the FP64 reference for the FP32 form's singular values.
    if not args.no_cpu and rank == 0:
        threads = os.cpu_count() or 1
        log("cpu oracle solve on %d threads" % threads)
        dt, r = cpu_solve(inp, init, threads)
        log("cpu oracle %.1f s, %d restarts, %d steps" % (dt, r["iterations"], r["lanczos_steps"]))
        # pca variances are D^2 / (m - 1) (pca.hpp:131-136), on both sides:
        # compare singular values.
        D_orc = np.sqrt(np.asarray(r["variances"]) * (m - 1))
        D32s = np.sqrt(D32 * (m - 1))
        out["cpu_baseline"] = {"value": dt, "unit": "s", "cores": threads, "kind": "port",
                               "sample": "one full FP64 oracle pca() to tol, measured (CppIrlba algorithm restated, "
                                         "OpenMP): %d restarts, %d Lanczos steps, converged %s" %
                                         (r["iterations"], r["lanczos_steps"], r["converged"])}
        out["fp32_D_max_rel_err_vs_fp64_oracle"] = float(np.max(np.abs(D32s - D_orc) / D_orc))
        if "fp64_gpu" in out:
            D64s = np.sqrt(D64 * (m - 1))
            out["fp64_gpu"]["D_max_rel_err_vs_fp64_oracle"] = float(np.max(np.abs(D64s - D_orc) / D_orc))
            out["fp64_gpu"]["restarts_equal_oracle"] = out["fp64_gpu"]["restarts"] == r["iterations"]

    # The other benchmark configurations as sub-records of the same line, each
    # with its own roofline, clocks and CPU baseline (a few steps each).
    if not args.no_extra and world == 1:
        sub = sub_args(args)
        for key, fn in (("fp64_pca_20k_x_50k", run_csc20k), ("batched_256", run_batch),
                        ("adjoint_4096x1024", run_adjoint)):
            log("sub-record %s" % key)
            try:
                out[key] = fn(sub)
            except Exception as exc:  # a failed sub-record is reported, not fatal
                out[key] = {"error": "%s: %s" % (type(exc).__name__, exc)}

    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
