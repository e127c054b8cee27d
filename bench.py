"""Benchmark: solves/s at 1e-10 relative residual on the 3D P2 Lagrange operator
refined 5 times (N = 274,625, nnz = 7,678,721), multicolor (Rainbow) SSOR-PCG.

One step = one batch of `--batch` independent solves (seeded U[-1,1] right-hand
sides, x0 = 0), each to a true FP64 relative residual <= 1e-10, by the batched
mixed-precision engine (FP32 inner Rainbow SSOR-PCG with compensated dots inside
FP64 defect correction; right-hand sides per team and team size chosen by the
engine's autotuner for the batch, untimed) with the right-hand sides and
solutions resident in HBM. `e2e` is the same batch through the public System API with the right-hand sides copied in from pinned host memory
and the solutions copied back inside the timed region. Beside it: one solve on the
whole GPU (latency p50/p99), the plain FP64 GPU CG and the FP64 drop-in Rainbow
solver (the reference's own stopping rule) on the same matrix, and the oracle (a
plain-C restatement of the reference solver) timed on the host cores.

`python bench.py --impl reference` times the reference algorithm on the host
cores instead (the oracle restatement with OpenMP, the reference's own
parallelisation) on the same workload and prints the same JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(dim=3, r=2, L=5)
WORKLOAD_NAME = "3D P2 Lagrange stiffness+mass, unit cube (6 tets) refined 5x: N=274625, nnz=7678721; " \
                "Rainbow SSOR-PCG omega=1.0, x0=0, b~U[-1,1] seeded, 1e-10 true relative residual"
METRIC = "solves/s at 1e-10 rel. residual (3D P2 L5, Rainbow SSOR-PCG), mixed FP32/FP64"
PRECISION = 1e-10
DRAM_OVER_ALGORITHMIC_L5_K4_T512 = 1.304   # profiles/batched_solve_3d_p2_l5.md


def max_over_ranks(x, device=None):
    """Largest value of x over the ranks of the default process group (x itself when
    there is none): the timed region of the slowest replica bounds the whole job."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds):
    """Whole-job throughput of `world` replicas that each processed `units_per_rank`."""
    return world * units_per_rank / seconds


def rank_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def rainbow_iteration_bytes(n, nnz, S, w):
    """Algorithmic bytes of one Rainbow/SSOR-PCG iteration with split storage."""
    return S * (2 * nnz - n) + 12 * (n + 1) + 17 * w * n


def rainbow_restart_bytes(n, nnz, S, w):
    # residual SpMV + forward sweep + backward sweep + vector streams of the restart
    return S * nnz + 4 * (n + 1) + S * (nnz - n) + 8 * (n + 1) + 12 * w * n


def cg_iteration_bytes(n, nnz, S, w):
    return S * nnz + 4 * (n + 1) + 11 * w * n


def run_reference(args):
    """Reference algorithm on the host cores (oracle restatement, OpenMP like the reference)."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    from oracle import oracle
    from simplefem_gb300 import workloads
    oracle.build()
    A, C, V = workloads.lattice_matrix(**WORKLOAD)
    n = len(A) - 1
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    diag = oracle.csr_diagonal(A, C, V)
    rb = oracle.rainbow(A, C)
    times = []
    Ks = []
    for step in range(args.warmup + args.steps):
        b = workloads.uniform_vector(1000 + step, n)
        t0 = time.perf_counter()
        K, x, _ = oracle.cg_rainbow(A, C, V, b, diag, rb, 1.0, precision=PRECISION)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt); Ks.append(K)
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "solver": "Rainbow SSOR-PCG FP64, reference stopping rule",
                   "iterations": int(np.median(Ks))},
        "p50_ms": 1000 * float(np.percentile(times, 50)), "p99_ms": 1000 * float(np.percentile(times, 99)),
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"{len(times)} full solves of the workload (reference algorithm restated in C, "
                                   f"OpenMP within colors as in sparsesolver.cpp:1091-1116)"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


SPMV_WORKLOAD = dict(dim=3, r=1, L=7)   # 3D P1 refined 7x: N = 2,146,689, nnz = 31,802,497 (> L2)


def run_spmv(dev, reps=20):
    """Resident SpMV (MatrixCSR::apply on the device, SELL-32) on the largest operator of the
    mixed-precision configuration, FP64 and FP32 values, L2 flushed before every product."""
    import torch
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import System
    A, C, V = workloads.lattice_matrix(**SPMV_WORKLOAD)
    n = len(A) - 1
    nnz = len(C)
    sysm = System(A, C, V)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    x = torch.from_numpy(workloads.uniform_vector(3, n)).to(dev)
    y = torch.empty_like(x)
    x32 = x.float()
    y32 = torch.empty_like(x32)
    stream = torch.cuda.current_stream()
    peak, kind = measured_peaks()
    out = {"workload": "3D P1 Lagrange stiffness+mass refined 7x: N=2146689, nnz=31802497",
           "algorithmic_bytes": "S*nnz + 4(N+1) + 2w*N (S=12/8, w=8/4)"}
    for tag, xx, yy, S_, w in (("fp64", x, y, 12, 8), ("fp32", x32, y32, 8, 4)):
        sysm.apply(xx, yy)
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sysm.apply(xx, yy)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        t = float(np.median(ms))
        b = S_ * nnz + 4 * (n + 1) + 2 * w * n
        gbs = b / (t / 1000.0) / 1e9
        out[tag] = {"us": 1000 * t, "bytes": b, "achieved_gbs": gbs, "frac": gbs / peak, "kernel": f"sell_spmv_kernel<{'double' if tag == 'fp64' else 'float'}>"}
    out["peak_gbs"] = peak
    out["peak_kind"] = kind
    sysm.close()
    return out


def run_batched_uneven(dev, count=512, reps=3):
    """512 independent uneven systems (2D P1/P2, refinements 3-7, coefficient mass) in one
    graph-captured batched launch, mixed precision and FP64, each column to 1e-10."""
    import torch
    import simplefem_gb300 as S
    from simplefem_gb300 import workloads
    from simplefem_gb300.system import Batch, System
    specs = workloads.batched_uneven_systems(count, 4242)
    systems = []
    for sp in specs:
        A, C, V = workloads.lattice_matrix(**sp)
        n = len(A) - 1
        mat = S.MatrixCSR(n, n, A, C, V)
        rb = S.Rainbow(mat)
        sysm = System(A, C, V)
        sysm.set_rainbow(mat.getDiagonal().raw(), 1.0, rb.num_colors, rb.F, rb.B, rb.R)
        systems.append(sysm)
    out = {"systems": count, "n_min": min(s.n for s in systems), "n_max": max(s.n for s in systems),
           "unknowns_total": sum(s.n for s in systems)}
    for mode, method in (("mixed", "rainbow"), ("fp64", "rainbow"), ("fp64", "cg")):
        # the first right-hand sides are in place before the batch is made: a mixed batch
        # solves them once each way at creation to pick its inner precision
        bs = [torch.from_numpy(workloads.uniform_vector(i, s.n)).to(dev) for i, s in enumerate(systems)]
        xs = [torch.zeros(s.n, dtype=torch.float64, device=dev) for s in systems]
        batch = Batch(systems, bs, xs, method=method, mode=mode, precision=PRECISION)
        times = []
        for rep in range(reps + 1):
            for i, sysm in enumerate(systems):
                bs[i].copy_(torch.from_numpy(workloads.uniform_vector(77 * rep + i, sysm.n)))
                xs[i].zero_()
            torch.cuda.synchronize()
            infos, ms = batch.run()
            assert all(i["status"] == 0 and i["true_relres"] <= PRECISION for i in infos), f"{mode}/{method} failed"
            if rep > 0:
                times.append(ms)
        batch.close()
        t = float(np.median(times))
        out[f"{mode}_{method}"] = {"ms_per_batch": t, "solves_per_s": count / (t / 1000.0),
                                   "iterations_median": int(np.median([i["iterations"] for i in infos])),
                                   "inner_fp64": int(infos[0]["inner_fp64"])}
    for s in systems:
        s.close()
    return out


def _rainbow_system(A, C, V):
    import simplefem_gb300 as S
    from simplefem_gb300.system import System
    n = len(A) - 1
    mat = S.MatrixCSR(n, n, A, C, V)
    rb = S.Rainbow(mat)
    sysm = System(A, C, V)
    sysm.set_rainbow(mat.getDiagonal().raw(), 1.0, rb.num_colors, rb.F, rb.B, rb.R)
    return sysm, rb.num_colors


def run_block_rhs(dev, nrhs=64, reps=3):
    """64 right-hand sides of the 2D P2 L7 coefficient-mass system (N = 66,049) solved as
    one blocked batch (K right-hand sides per team share every matrix load), the launch
    configuration chosen by the autotuner for this batch size; plain CG and Rainbow
    SSOR-PCG, FP64 and mixed precision, each column to 1e-10. Beside it, single FP64
    CG solves on the whole GPU."""
    import torch
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(2, 2, 7, 1)
    n = len(A) - 1
    sysm, ncol = _rainbow_system(A, C, V)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    B = torch.from_numpy(np.stack([workloads.uniform_vector(4000 + j, n) for j in range(nrhs)])).to(dev)
    X = torch.zeros_like(B)
    out = {"workload": f"2D P2 Lagrange stiffness + coefficient mass (log-uniform [0.1, 10]) refined 7x: N={n}, "
                       f"nnz={len(C)}, {ncol} colors; {nrhs} right-hand sides", "nrhs": nrhs}
    for method, mode in (("cg", "fp64"), ("cg", "mixed"), ("rainbow", "fp64"), ("rainbow", "mixed")):
        cfg = sysm.tune_batch(method, mode, nrhs_hint=nrhs)
        ms, infos = [], None
        for rep in range(reps + 1):
            X.zero_()
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            infos = sysm.solve_batch(B, X, method=method, mode=mode, precision=PRECISION)
            e1.record(stream)
            torch.cuda.synchronize()
            if rep > 0:
                ms.append(e0.elapsed_time(e1))
        assert all(i["status"] == 0 and i["true_relres"] <= PRECISION for i in infos), f"block {method}/{mode}"
        t = float(np.median(ms))
        out[f"{method}_{mode}"] = {"ms_per_batch": t, "solves_per_s": nrhs / (t / 1000.0), "config": cfg,
                                   "iterations_median": int(np.median([i["iterations"] for i in infos])),
                                   "outer_median": int(np.median([i["outer_iterations"] for i in infos])),
                                   "fp64_fallbacks": int(sum(i["fp64_fallback"] for i in infos))}
    single = []
    for j in range(4):
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sysm.solve(B[j], x, method="cg", mode="fp64", precision=PRECISION)
        e1.record(stream)
        torch.cuda.synchronize()
        if j > 0:
            single.append(e0.elapsed_time(e1))
    out["fp64_cg_single_on_whole_gpu"] = {"ms": float(np.median(single)),
                                          "solves_per_s": 1000.0 / float(np.median(single))}
    sysm.close()
    return out


def run_mixed_large(dev, reps=3):
    """The mixed-precision target operator (3D P1 L7, N = 2,146,689): one solve on the whole
    GPU to 1e-10 in mixed precision and in FP64, each solution's error against an FP64 CG
    solve at 1e-13 true relative residual."""
    import torch
    from simplefem_gb300 import workloads
    A, C, V = workloads.lattice_matrix(3, 1, 7)
    n = len(A) - 1
    sysm, ncol = _rainbow_system(A, C, V)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    b = torch.from_numpy(workloads.uniform_vector(77, n)).to(dev)
    xr = torch.zeros(n, dtype=torch.float64, device=dev)
    ref = sysm.solve(b, xr, method="cg", mode="fp64", precision=1e-13)
    out = {"workload": f"3D P1 Lagrange stiffness+mass refined 7x: N={n}, nnz={len(C)}, {ncol} colors",
           "error_reference": {"solver": "FP64 CG to 1e-13 true relative residual", "iterations": ref["iterations"],
                               "true_relres": ref["true_relres"]}}
    for method, mode in (("rainbow", "mixed"), ("rainbow", "fp64"), ("cg", "mixed"), ("cg", "fp64")):
        # mixed: the system's first solve runs FP32 inner iterations and its second FP64 ones
        # (both untimed, both checked); the timed ones keep the faster per decade of fall
        warm = 2 if mode == "mixed" else 1
        ms, info, x, first = [], None, None, []
        for rep in range(reps + warm):
            x = torch.zeros(n, dtype=torch.float64, device=dev)
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            info = sysm.solve(b, x, method=method, mode=mode, precision=PRECISION)
            e1.record(stream)
            torch.cuda.synchronize()
            assert info["status"] == 0 and info["true_relres"] <= PRECISION, (method, mode, rep, info)
            if rep >= warm:
                ms.append(e0.elapsed_time(e1))
            else:
                first.append({"device_ms": info["device_ms"], "iterations": info["iterations"],
                              "inner_fp64": info["inner_fp64"],
                              "rel_error_vs_fp64_1e-13": float((x - xr).norm() / xr.norm())})
        err = float((x - xr).norm() / xr.norm())
        t = float(np.median(ms))
        out[f"{method}_{mode}"] = {"ms": t, "solves_per_s": 1000.0 / t, "iterations": info["iterations"],
                                   "outer_iterations": info["outer_iterations"], "true_relres": info["true_relres"],
                                   "rel_error_vs_fp64_1e-13": err, "fp64_fallback": info["fp64_fallback"],
                                   "inner_fp64": info["inner_fp64"],
                                   "lanes_per_row": info["lanes_per_row"], "grid_blocks": info["grid_blocks"]}
        if mode == "mixed":
            out[f"{method}_{mode}"]["choice_measured_on"] = first
    sysm.close()
    return out


def run_csr_algebra(with_cpu, reps=3):
    """CSR algebra through the C ABI with host arrays (upload, kernels, download inside the
    timed call): the operator product X*X of lattice operators and, at solver size, the
    transpose and a sum. Every GPU result is compared bit for bit with the oracle's (the
    oracle's OpenMP restatement of the reference's algorithm is the CPU time beside it)."""
    import simplefem_gb300 as S
    from simplefem_gb300 import workloads
    oracle = None
    if with_cpu:
        from oracle import oracle
        oracle.set_threads(os.cpu_count() or 1)

    def timed(fn, count):
        fn()
        t = []
        for _ in range(count):
            t0 = time.perf_counter(); r = fn(); t.append(time.perf_counter() - t0)
        return 1000.0 * float(np.median(t)), r

    def same(M, ref):
        return bool(np.array_equal(M.A, ref[0]) and np.array_equal(M.C, ref[1]) and
                    np.array_equal(M.V.view(np.int64), ref[2].view(np.int64)))

    out = {"note": "host arrays in and out (C ABI call incl. H2D/D2H and host-side index checks); "
                   "cpu = oracle restatement with OpenMP on the host cores; results compared bit for bit"}
    for (d, r, L) in ((3, 1, 5), (3, 2, 4)):
        A, C, V = workloads.lattice_matrix(d, r, L, 0)
        n = len(A) - 1
        X = S.MatrixCSR(n, n, A, C, V)
        ms, M = timed(lambda: S.MatrixCSRMultiplication(X, X), reps)
        leg = {"workload": f"{d}D P{r} refined {L}x: X*X, N={n}, nnz={len(C)} -> {M.getnumberofentries()}",
               "gpu_ms": ms}
        if oracle is not None:
            cms, ref = timed(lambda: oracle.csr_multiply(A, C, V, A, C, V), 1)
            leg.update({"cpu_ms": cms, "cpu_cores": os.cpu_count() or 1, "bit_identical": same(M, ref)})
        out[f"multiply_{d}d_p{r}_l{L}"] = leg
    # SparseMatrixMultiplication of two COO operands (3D P1 refined 5x, entries shuffled)
    A, C, V = workloads.lattice_matrix(3, 1, 5, 0)
    n = len(A) - 1
    rng = np.random.default_rng(4)
    perm = rng.permutation(len(C))
    rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(A))[perm]
    Lc = S.SparseMatrix(n, n, rows, C[perm], V[perm])
    ms, P = timed(lambda: S.SparseMatrixMultiplication(Lc, Lc), reps)
    leg = {"workload": f"3D P1 refined 5x: COO X*X, N={n}, {len(C)} entries -> {P.getnumberofentries()}",
           "gpu_ms": ms}
    if oracle is not None:
        cms, ref = timed(lambda: oracle.coo_multiply(n, (Lc.r, Lc.c, Lc.v), (Lc.r, Lc.c, Lc.v)), 1)
        leg.update({"cpu_ms": cms, "cpu_cores": 1, "bit_identical": bool(
            np.array_equal(P.r, ref[0]) and np.array_equal(P.c, ref[1]) and
            np.array_equal(P.v.view(np.int64), ref[2].view(np.int64)))})
    out["coo_multiply_3d_p1_l5"] = leg
    A, C, V = workloads.lattice_matrix(3, 2, 6, 0)
    n = len(A) - 1
    X = S.MatrixCSR(n, n, A, C, V)
    for name, fn, cfn in (("transpose", lambda: X.getTranspose(), lambda: oracle.csr_transpose(A, C, V, n)),
                          ("add", lambda: S.MatrixCSRAddition(X, X, 1.0, 0.5),
                           lambda: oracle.csr_add(A, C, V, A, C, V, 1.0, 0.5))):
        ms, M = timed(fn, reps)
        leg = {"workload": f"3D P2 refined 6x: {name}, N={n}, nnz={len(C)}", "gpu_ms": ms}
        if oracle is not None:
            cms, ref = timed(cfn, 1)
            leg.update({"cpu_ms": cms, "cpu_cores": os.cpu_count() or 1, "bit_identical": same(M, ref)})
        out[f"{name}_3d_p2_l6"] = leg
    return out


def run_krylov_more(with_cpu, hodge=True):
    """The further drop-in drivers through their host-pointer entry points (upload inside the
    call): conjugate residuals and MINRES beside plain CG on the 3D P1 operator refined 6x,
    and the Hodge conjugate residual solver (inner SSOR-PCG) on a block system. The CPU
    column is the oracle restatement with the reference's OpenMP loops, on every host core."""
    import simplefem_gb300 as S
    from simplefem_gb300 import workloads
    oracle = None
    cores = os.cpu_count() or 1
    if with_cpu:
        from oracle import oracle
        oracle.set_threads(cores)
    A, C, V = workloads.lattice_matrix(3, 1, 6, 0)
    n = len(A) - 1
    b = workloads.uniform_vector(17, n)
    out = {"workload": f"3D P1 refined 6x, N={n}, nnz={len(C)}, precision 1e-10, host arrays in and out"}
    for name, fn, ofn in (("cg", S.ConjugateGradientSolverCSR, None),
                          ("cr", S.ConjugateResidualSolverCSR, None if oracle is None else oracle.cr),
                          ("minres", S.MINRESCSR, None if oracle is None else oracle.minres)):
        x = np.zeros(n); res = np.zeros(n)
        fn(n, x, b, A, C, V, res, 1e-10, -3)                     # warm-up
        x = np.zeros(n); res = np.zeros(n)
        t0 = time.perf_counter()
        K = fn(n, x, b, A, C, V, res, 1e-10, -3)
        wall = 1000.0 * (time.perf_counter() - t0)
        info = S.last_info()
        leg = {"iterations": K, "status": info["status"], "call_ms": wall, "device_ms": info["device_ms"]}
        # algorithmic bytes per iteration (matrix once, vector streams): CG 11, CR 13, MINRES 14 vectors
        vec = {"cg": 11, "cr": 13, "minres": 14}[name]
        it_bytes = 12 * len(C) + 4 * (n + 1) + vec * 8 * n
        if K > 0 and info["device_ms"] > 0:
            gbs = it_bytes * K / (info["device_ms"] / 1000.0) / 1e9
            leg["roofline"] = {"bytes_per_iteration": it_bytes, "us_per_iteration": 1000.0 * info["device_ms"] / K,
                               "achieved_gbs": gbs, "frac_of_hbm": gbs / measured_peaks()[0],
                               "note": "matrix and vectors (~%d MB) stay in the 129 MB L2 across iterations: "
                                       "latency (grid barriers) bound, not HBM bound" % (it_bytes // 2**20)}
        if ofn is not None:
            t0 = time.perf_counter()
            K_o, _, _ = ofn(A, C, V, b, precision=1e-10)
            leg.update({"cpu_ms": 1000.0 * (time.perf_counter() - t0), "cpu_iterations": K_o, "cpu_cores": cores})
        out[name] = leg
    if not hodge:
        return out
    # Hodge: A = 3D P1 refined 5x (L = 35,937), C = 2D P1 refined 7x (N = 16,641), B 6 entries per row
    rng = np.random.default_rng(12)
    Am = workloads.lattice_matrix(3, 1, 5, 0)
    Cm = workloads.lattice_matrix(2, 1, 7, 3)
    L, N = len(Am[0]) - 1, len(Cm[0]) - 1
    cols = np.concatenate([np.sort(rng.choice(L, 6, replace=False)) for _ in range(N)]).astype(np.int32)
    Bm = (np.arange(0, 6 * N + 1, 6, dtype=np.int32), cols, rng.uniform(-1, 1, 6 * N))
    Btm = S.MatrixCSR(N, L, *Bm).getTranspose()
    Btm = (Btm.A, Btm.C, Btm.V)
    bh = rng.uniform(-1, 1, N)
    for key, fn, variant, inner_name in (("hodge_cr_ssor", S.HodgeConjugateResidualSolverCSR, 1, "SSOR-PCG"),
                                         ("hodge_cr_diagonal", S.HodgeConjugateResidualSolverCSR_diagonal, 0,
                                          "diagonal PCG")):
        x = np.zeros(N); res = np.zeros(N)
        t0 = time.perf_counter()
        K = fn(N, L, x, bh, Am, Bm, Btm, Cm, res, 1e-8, -3, 1e-10)
        wall = 1000.0 * (time.perf_counter() - t0)
        info = S.last_info()
        leg = {"workload": f"CR on B A^-1 Bt + C: A 3D P1 L5 (L={L}), C 2D P1 L7 (N={N}), B 6/row; "
                           f"precision 1e-8, inner {inner_name} to 1e-10",
               "outer_iterations": K, "inner_iterations": info["outer_iterations"], "status": info["status"],
               "call_ms": wall}
        if oracle is not None:
            t0 = time.perf_counter()
            K_o, _, _ = oracle.hodge_cr(variant, Am, Bm, Btm, Cm, bh, precision=1e-8, inner_precision=1e-10)
            leg.update({"cpu_ms": 1000.0 * (time.perf_counter() - t0), "cpu_outer_iterations": K_o,
                        "cpu_cores": cores})
        out[key] = leg
    return out


def run_small(with_cpu):
    """The drop-ins on the reference's own CPU-sized case, 2D P1 refined 6x (N = 4,225):
    host arrays in and out, median of 5 calls, beside the oracle at one thread (the
    reference's plain CG is only correct at one thread, its SSOR sweeps are serial)."""
    import simplefem_gb300 as S
    from simplefem_gb300 import workloads
    oracle = None
    if with_cpu:
        from oracle import oracle
        oracle.set_threads(1)
    A, C, V = workloads.lattice_matrix(2, 1, 6, 0)
    n = len(A) - 1
    b = workloads.uniform_vector(2024, n)
    mat = S.MatrixCSR(n, n, A, C, V)
    diag = mat.getDiagonal().raw()
    rb = S.Rainbow(mat)
    rbo = (rb.num_colors, rb.F, rb.B, rb.R)
    calls = {
        "cg": (lambda x, r: S.ConjugateGradientSolverCSR(n, x, b, A, C, V, r, 1e-10, -3),
               None if oracle is None else (lambda: oracle.cg(A, C, V, b, precision=1e-10))),
        "ssor": (lambda x, r: S.ConjugateGradientSolverCSR_SSOR(n, x, b, A, C, V, r, 1e-10, -3, diag, 1.0),
                 None if oracle is None else (lambda: oracle.cg_ssor(A, C, V, b, diag, 1.0, precision=1e-10))),
        "rainbow": (lambda x, r: S.ConjugateGradientSolverCSR_Rainbow(n, x, b, A, C, V, r, 1e-10, -3, diag, 1.0,
                                                                      *rbo),
                    None if oracle is None else (lambda: oracle.cg_rainbow(A, C, V, b, diag, rbo, 1.0,
                                                                           precision=1e-10))),
    }
    out = {"workload": f"2D P1 refined 6x, N={n}, nnz={len(C)}, {rb.num_colors} colors, precision 1e-10"}
    for name, (gpu, cpu) in calls.items():
        wall, dev_ms, K = [], [], 0
        for _ in range(6):
            x = np.zeros(n); r = np.zeros(n)
            t0 = time.perf_counter()
            K = gpu(x, r)
            wall.append(1000.0 * (time.perf_counter() - t0))
            dev_ms.append(S.last_info()["device_ms"])
        leg = {"iterations": K, "call_ms": float(np.median(wall[1:])), "device_ms": float(np.median(dev_ms[1:]))}
        if cpu is not None:
            ts = []
            for _ in range(5):
                t0 = time.perf_counter(); K_o, _, _ = cpu(); ts.append(1000.0 * (time.perf_counter() - t0))
            leg.update({"cpu_ms": float(np.median(ts)), "cpu_iterations": K_o, "cpu_cores": 1})
        out[name] = leg
    return out


def run_serving(mode, method, count=200, rate=200.0, slots=24, budget=120 * 10**9, resident=False):
    """Poisson-arrival request stream through the continuous-batching server. resident: the
    stream's distinct operators are registered first (timed apart) and the requests carry
    only their right-hand sides."""
    from simplefem_gb300 import workloads
    from simplefem_gb300.serving import Server
    reqs = workloads.serving_requests(count, 2026, rate_per_s=rate)
    pool = {}
    for rq in reqs:
        key = (rq["dim"], rq["r"], rq["L"], rq["coef_seed"])
        if key not in pool:
            pool[key] = workloads.lattice_matrix(*key)
    rhs = [workloads.uniform_vector(rq["rhs_seed"], rq["n"]) for rq in reqs]
    srv = Server(hbm_budget_bytes=budget, slots=slots, method=method, mode=mode)
    ops, register_s = {}, 0.0
    if resident:
        t0 = time.perf_counter()
        for key, (A, C, V) in pool.items():
            ops[key] = srv.add_operator(A, C, V)
        register_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    for rq, b in zip(reqs, rhs):
        dt = rq["t"] - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        key = (rq["dim"], rq["r"], rq["L"], rq["coef_seed"])
        if resident:
            srv.submit_rhs(ops[key], b, rq["tol"])
        else:
            A, C, V = pool[key]
            srv.submit(A, C, V, b, rq["tol"])
    ok = srv.wait(1800)
    makespan = time.perf_counter() - t0
    res = srv.poll(4096)
    stats = srv.stats()
    srv.close()
    lat = np.array([r["latency_ms"] for r in res])
    bad = [r for r in res if r["status"] != 0 or r["true_relres"] > [q for q in reqs][r["id"] - 1]["tol"]]
    out = {"mode": mode, "method": method, "requests": count, "arrival_rate_per_s": rate, "slots": slots,
            "hbm_budget_gb": budget / 1e9, "completed": len(res), "failed": len(bad), "all_done": bool(ok),
            "solves_per_s": len(res) / makespan, "makespan_s": makespan,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "peak_bytes": stats["peak_bytes"],
            "unknowns_range": [min(r["n"] for r in reqs), max(r["n"] for r in reqs)]}
    if resident:
        out.update({"resident_operators": len(ops), "register_s": register_s})
    return out


def run_ours(args):
    import torch
    import torch.distributed as dist

    rank, world, local = rank_info()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import simplefem_gb300 as S
    from simplefem_gb300 import _native, workloads
    from simplefem_gb300.system import System

    lib = _native.gpu()
    if args.only_spmv:
        if rank == 0:
            print(json.dumps({"spmv": run_spmv(dev)}), flush=True)
        return
    if args.only_uneven:
        if rank == 0:
            print(json.dumps({"batched_uneven": run_batched_uneven(dev)}), flush=True)
        return
    if args.only_block_rhs:
        if rank == 0:
            print(json.dumps({"block_rhs_64": run_block_rhs(dev)}), flush=True)
        return
    if args.only_mixed_large:
        if rank == 0:
            print(json.dumps({"mixed_large": run_mixed_large(dev)}), flush=True)
        return
    if args.only_small:
        if rank == 0:
            print(json.dumps({"small": run_small(not args.no_cpu)}), flush=True)
        return
    if args.only_krylov_more:
        if rank == 0:
            print(json.dumps({"krylov_more": run_krylov_more(not args.no_cpu)}), flush=True)
        return
    if args.only_csr_algebra:
        if rank == 0:
            print(json.dumps({"csr_algebra": run_csr_algebra(not args.no_cpu)}), flush=True)
        return
    if args.only_serving:
        if rank == 0:
            print(json.dumps({"serving": [run_serving("mixed", "rainbow", args.requests),
                                          run_serving("fp64", "cg", args.requests),
                                          run_serving("mixed", "rainbow", 100, rate=5.0),
                                          run_serving("fp64", "cg", 100, rate=5.0),
                                          run_serving("mixed", "rainbow", args.requests, resident=True),
                                          run_serving("mixed", "rainbow", 100, rate=5.0, resident=True)]}),
                  flush=True)
        return
    A, C, V = workloads.lattice_matrix(**dict(WORKLOAD, L=args.level))
    n = len(A) - 1
    nnz = len(C)
    mat = S.MatrixCSR(n, n, A, C, V)
    diag = mat.getDiagonal().raw()
    t0 = time.perf_counter()
    rb = S.Rainbow(mat)
    rb_ms = 1000.0 * (time.perf_counter() - t0)
    sysm = System(A, C, V)
    sysm.set_rainbow(diag, 1.0, rb.num_colors, rb.F, rb.B, rb.R)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MB > L2 (129 MB)
    stream = torch.cuda.current_stream()
    if args.only_single:
        # one solve at a time on the whole GPU (the persistent drop-in kernels), `--steps` solves
        # per method after `--warmup` untimed ones; L2 flushed before each
        out = {"workload": f"3D P2 refined {args.level}x, N={n}, nnz={nnz}"}
        for method, mode in (("rainbow", "reference"), ("cg", "reference"), ("rainbow", "mixed"), ("cg", "fp64")):
            ms, infos = [], []
            for k in range(args.warmup + args.steps):
                b = torch.from_numpy(workloads.uniform_vector(9000 + k, n)).to(dev)
                x = torch.zeros(n, dtype=torch.float64, device=dev)
                flush.zero_()
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                info = sysm.solve(b, x, method=method, mode=mode, precision=PRECISION)
                e1.record(stream)
                torch.cuda.synchronize()
                if k >= args.warmup:
                    ms.append(e0.elapsed_time(e1)); infos.append(info)
            out[f"{method}_{mode}"] = {"ms": float(np.median(ms)), "iterations": int(np.median([i["iterations"] for i in infos])),
                                       "device_ms": float(np.median([i["device_ms"] for i in infos])),
                                       "grid_blocks": infos[0]["grid_blocks"], "lanes_per_row": infos[0]["lanes_per_row"]}
        if rank == 0:
            print(json.dumps({"single": out}), flush=True)
        sysm.close()
        return
    B_RHS = args.batch
    if args.rhs_per_team > 0:
        # a fixed launch configuration (profiling captures: the kernel launches are then exactly
        # the warm-up and timed steps)
        sysm.set_batch_config("rainbow", "mixed", rhs_per_team=args.rhs_per_team, team_threads=args.team_threads,
                              team_blocks=args.team_blocks)
        tuned = {"rhs_per_team": args.rhs_per_team, "team_threads": args.team_threads,
                 "team_blocks": args.team_blocks, "fixed": True}
    else:
        # launch configuration of the batched engine from the autotuner, for this batch size (untimed)
        tuned = sysm.tune_batch("rainbow", "mixed", nrhs_hint=B_RHS)
    K_TEAM = tuned["rhs_per_team"]

    def rhs_block(step, count):
        return np.stack([workloads.uniform_vector(1000 + 100003 * rank + 4099 * step + j, n) for j in range(count)])

    # ---------------- headline: batched mixed-precision Rainbow SSOR-PCG ----------------
    Bdev = torch.empty((B_RHS, n), dtype=torch.float64, device=dev)
    Xdev = torch.empty((B_RHS, n), dtype=torch.float64, device=dev)
    per, infos_all = [], []
    for step in range(args.warmup):                       # untimed warm-up steps
        Bdev.copy_(torch.from_numpy(rhs_block(step, B_RHS)))
        Xdev.zero_()
        sysm.solve_batch(Bdev, Xdev, method="rainbow", mode="mixed", precision=PRECISION)
    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lib.feec_kernel_launches()
    clocks.start()
    for step in range(args.steps):
        Bdev.copy_(torch.from_numpy(rhs_block(args.warmup + step, B_RHS)))
        Xdev.zero_()
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        infos = sysm.solve_batch(Bdev, Xdev, method="rainbow", mode="mixed", precision=PRECISION)
        e1.record(stream)
        torch.cuda.synchronize()
        per.append(e0.elapsed_time(e1))
        infos_all.append(infos)
    clock_info = clocks.stop()
    launches = lib.feec_kernel_launches() - launches0
    total_ms = max_over_ranks(float(sum(per)), dev)
    if world > 1:
        dist.barrier()
    value = whole_job_rate(args.steps * B_RHS, world, total_ms / 1000.0)
    flat = [i for infos in infos_all for i in infos]
    assert all(i["status"] == 0 and 0 <= i["true_relres"] <= PRECISION for i in flat), "batched solve missed 1e-10"
    inner_iters = [i["iterations"] for i in flat]
    outer_iters = [i["outer_iterations"] for i in flat]

    # roofline of the batched kernel: algorithmic bytes over its event-timed duration. The
    # Rainbow inner solve is Eisenstat's formulation: per team iteration the strict lower and
    # strict upper parts are read once (FP32 value + int32 column) with two sweeps' row
    # bounds, plus 6 per-row FP32 factors (wd and sd three times each); per right-hand side
    # and iteration 15 FP32 vector streams (backward: d, r in, d, m out, m gathered;
    # forward: d, m in, q out, q gathered; update: c, m, q, r in, c, r out). Per segment: the
    # FP64 residual (whole matrix, FP64) and the L-solve of the restart per team, and 96
    # bytes per row and right-hand side (residual 24, restart 32, L-solve 20, x update 20).
    teams = (B_RHS + K_TEAM - 1) // K_TEAM
    mat_b = 8 * (nnz - n) + 8 * (n + 1) + 6 * 4 * n
    vec_b = 15 * 4 * n
    outer_team_b = 12 * nnz + 4 * (n + 1) + 4 * (nnz - n) + 4 * (n + 1)
    outer_col_b = 96 * n
    per_step_bytes = 0
    shared_bytes = 0      # the same with the operator counted once per iteration of the whole batch
    for infos in infos_all:
        its = [i["iterations"] for i in infos]
        outs = [i["outer_iterations"] for i in infos]
        for t0 in range(teams):
            cols = range(t0 * K_TEAM, min(B_RHS, (t0 + 1) * K_TEAM))
            team_it = max(its[j] for j in cols)
            vec_outer = sum(its[j] for j in cols) * vec_b + sum(outs[j] + 1 for j in cols) * outer_col_b
            per_step_bytes += team_it * mat_b + (max(outs[j] for j in cols) + 1) * outer_team_b + vec_outer
            shared_bytes += vec_outer
        shared_bytes += max(its) * mat_b + (max(outs) + 1) * outer_team_b
    per_step_bytes /= len(infos_all)
    shared_bytes /= len(infos_all)
    peak, peak_kind = measured_peaks()
    achieved = per_step_bytes / (total_ms / args.steps / 1000.0) / 1e9
    achieved_shared = shared_bytes / (total_ms / args.steps / 1000.0) / 1e9
    if tuned["team_blocks"] > 1:
        kernel_name = f"cluster_batched_kernel<float,{K_TEAM},true> ({tuned['team_blocks']}-block clusters)"
    else:
        kernel_name = f"batched_solve_kernel<float,{K_TEAM},true,{tuned['team_threads']}>"
    # DRAM traffic of this kernel configuration from one full-size ncu capture (one pass:
    # dram__bytes_read.sum + dram__bytes_write.sum; profiles/batched_solve_3d_p2_l5.md), as a
    # ratio to the algorithmic bytes of the captured launch, applied to this launch
    traffic = None
    if (K_TEAM, tuned["team_threads"], tuned["team_blocks"]) == (4, 512, 1) and DRAM_OVER_ALGORITHMIC_L5_K4_T512:
        traffic = DRAM_OVER_ALGORITHMIC_L5_K4_T512 * per_step_bytes
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": kernel_name, "launches_per_step": 1,
                "traffic_source": f"ncu DRAM bytes / algorithmic bytes = {DRAM_OVER_ALGORITHMIC_L5_K4_T512} measured "
                                  "on this workload (profiles/batched_solve_3d_p2_l5.md), applied to this launch"
                                  if traffic else None,
                "bytes_per_launch": per_step_bytes, "ms_per_launch": total_ms / args.steps,
                "shared_operator": {"bytes_per_launch": shared_bytes, "achieved": achieved_shared,
                                    "frac": achieved_shared / peak,
                                    "note": "operator counted once per iteration of the whole batch"},
                "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"}

    # ---------------- e2e: pinned host B -> device, batched solve, device X -> pinned host ----------------
    # Double-buffered as a user of the System API would run a stream of batches: the next
    # batch's right-hand sides go up and the previous batch's solutions come down on a copy
    # stream while the current batch solves (solve_batch releases the GIL and runs on the
    # compute stream). Every step's copies are inside the timed region; the first upload and
    # the last download are not overlapped.
    E2E_STEPS = args.steps                                 # the same number of batches as `value`
    hB = [torch.empty((B_RHS, n), dtype=torch.float64).pin_memory() for _ in range(2)]
    hX = [torch.empty((B_RHS, n), dtype=torch.float64).pin_memory() for _ in range(2)]
    for k in range(2):
        hB[k].copy_(torch.from_numpy(rhs_block(500 + k, B_RHS)))

    # ---------------- accuracy of the last timed batch (untimed) ----------------
    # a sample of its columns against FP64 plain CG solves on the GPU to 1e-13 true relative
    # residual (their own error is about 1e-12 here)
    sample = list(range(0, B_RHS, max(1, B_RHS // 8)))[:8]
    errs = []
    for j in sample:
        xt = torch.zeros(n, dtype=torch.float64, device=dev)
        sysm.solve(Bdev[j], xt, method="cg", mode="fp64", precision=1e-13)
        errs.append(float((Xdev[j] - xt).norm() / xt.norm()))
    accuracy = {"columns": len(sample), "rel_error_max": max(errs), "rel_error_median": float(np.median(errs)),
                "error_estimate_max": max(i["error_estimate"] for i in infos_all[-1]),
                "reference": "FP64 plain CG on the GPU to 1e-13 true relative residual"}

    Bd = [Bdev, torch.empty_like(Bdev)]
    Xd = [Xdev, torch.empty_like(Xdev)]
    copy_stream = torch.cuda.Stream()

    def e2e_run(steps):
        ready = [torch.cuda.Event(), torch.cuda.Event()]
        done = [torch.cuda.Event(), torch.cuda.Event()]
        with torch.cuda.stream(copy_stream):
            Bd[0].copy_(hB[0], non_blocking=True)
            Xd[0].zero_()
            ready[0].record(copy_stream)
        for k in range(steps):
            cur, nxt = k % 2, (k + 1) % 2
            with torch.cuda.stream(copy_stream):
                if k >= 1:                                 # previous batch's solutions down
                    copy_stream.wait_event(done[nxt])
                    hX[nxt].copy_(Xd[nxt], non_blocking=True)
                if k + 1 < steps:                          # next batch's right-hand sides up
                    Bd[nxt].copy_(hB[nxt], non_blocking=True)
                    Xd[nxt].zero_()
                    ready[nxt].record(copy_stream)
            stream.wait_event(ready[cur])
            sysm.solve_batch(Bd[cur], Xd[cur], method="rainbow", mode="mixed", precision=PRECISION)
            done[cur].record(stream)
        with torch.cuda.stream(copy_stream):
            last = (steps - 1) % 2
            copy_stream.wait_event(done[last])
            hX[last].copy_(Xd[last], non_blocking=True)
        torch.cuda.synchronize()

    e2e_run(2)                                             # untimed: maps the pinned buffers
    flush.zero_()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_run(E2E_STEPS)
    e2e_total = time.perf_counter() - t0
    e2e_per = [e2e_total / E2E_STEPS] * E2E_STEPS
    e2e_value = whole_job_rate(B_RHS * len(e2e_per), world, max_over_ranks(sum(e2e_per), dev))
    e2e = {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": 8 * n * B_RHS,
           "d2h_bytes_per_step": 8 * n * B_RHS, "steps": E2E_STEPS, "ms_per_step": 1000.0 * e2e_total / E2E_STEPS,
           "copies": "double-buffered on a copy stream, overlapped with the neighbouring batches' solves"}

    if args.only_batched:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                              "config": {"workload": f"3D P2 refined {args.level}x, N={n}, nnz={nnz}",
                                         "batch": B_RHS, "rhs_per_team": K_TEAM, "autotuner": tuned},
                              "inner_iterations": int(np.median(inner_iters)),
                              "outer_iterations": int(np.median(outer_iters)), "accuracy": accuracy,
                              "roofline": roofline, "e2e": e2e,
                              "gpu_launches": int(launches), "clocks": clock_info}), flush=True)
        sysm.close()
        if world > 1:
            dist.destroy_process_group()
        return

    # ---------------- like for like: the same 1216 solves by the batched FP64 engine ----------------
    tuned64 = sysm.tune_batch("rainbow", "fp64", nrhs_hint=B_RHS)
    fp64_batch_ms = []
    for rep in range(3):
        Bdev.copy_(torch.from_numpy(rhs_block(args.warmup + rep, B_RHS)))
        Xdev.zero_()
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        infos64 = sysm.solve_batch(Bdev, Xdev, method="rainbow", mode="fp64", precision=PRECISION)
        e1.record(stream)
        torch.cuda.synchronize()
        assert all(i["status"] == 0 and 0 <= i["true_relres"] <= PRECISION for i in infos64), "FP64 batch missed"
        if rep > 0:
            fp64_batch_ms.append(e0.elapsed_time(e1))
    fp64_batched = {"solves_per_s": B_RHS / (float(np.median(fp64_batch_ms)) / 1000.0),
                    "ms_per_batch": float(np.median(fp64_batch_ms)), "config": tuned64,
                    "iterations_median": int(np.median([i["iterations"] for i in infos64]))}
    del Bd, Xd, hB, hX

    # ---------------- single-solve latency (whole GPU per solve) and the FP64 baselines ----------------
    def single(method, mode, count, seed):
        # warm-up: one call; in mixed mode two (the system's first solve runs FP32 inner
        # iterations, its second FP64 ones, and later solves keep the faster per decade)
        warm = 2 if mode == "mixed" else 1
        out, inf, first = [], [], []
        for k in range(count + warm):
            b = torch.from_numpy(workloads.uniform_vector(seed + k, n)).to(dev)
            x = torch.zeros(n, dtype=torch.float64, device=dev)
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            info = sysm.solve(b, x, method=method, mode=mode, precision=PRECISION)
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= warm:
                out.append(e0.elapsed_time(e1)); inf.append(info)
            else:
                first.append(info)
        if mode == "mixed":
            single.measured = {"fp32_inner_device_ms": first[0]["device_ms"], "fp32_inner_iterations": first[0]["iterations"],
                               "fp64_inner_device_ms": first[1]["device_ms"], "fp64_inner_iterations": first[1]["iterations"]}
        return out, inf

    mixed1, mixed1_i = single("rainbow", "mixed", 5, 7000)
    mixed1_measured = single.measured
    cg64, cg64_i = single("cg", "fp64", 3, 8000)
    rb64, rb64_i = single("rainbow", "reference", 3, 9000)
    eis64, eis64_i = single("rainbow_eisenstat", "reference", 3, 9500)

    # drop-in host-pointer call (matrix uploaded inside the call, as the reference signature implies)
    b0 = workloads.uniform_vector(6000, n)
    dropin = []
    for step in range(3):
        xh = np.zeros(n); res = np.zeros(n)
        t0 = time.perf_counter()
        S.ConjugateGradientSolverCSR_Rainbow(n, xh, b0, A, C, V, res, PRECISION, -3, diag, 1.0,
                                             rb.num_colors, rb.F, rb.B, rb.R)
        if step > 0:
            dropin.append(time.perf_counter() - t0)
    dropin_K = S.last_info()["iterations"]

    spmv = run_spmv(dev)
    extras = {}
    if args.full:
        extras = {"batched_uneven": run_batched_uneven(dev), "block_rhs_64": run_block_rhs(dev),
                  "mixed_large": run_mixed_large(dev),
                  "csr_algebra": run_csr_algebra(rank == 0 and not args.no_cpu),
                  "krylov_more": run_krylov_more(rank == 0 and not args.no_cpu),
                  "small_dropins": run_small(rank == 0 and not args.no_cpu),
                  "serving": {"mixed_rainbow": run_serving("mixed", "rainbow", args.requests),
                              "fp64_cg": run_serving("fp64", "cg", args.requests)}}

    # CPU baseline: the oracle restatement of the reference Rainbow-PCG on the host cores, one solve
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle
        threads = os.cpu_count() or 1
        oracle.set_threads(threads)
        rbo = (rb.num_colors, rb.F, rb.B, rb.R)
        times = []
        for k in range(3):
            t0 = time.perf_counter()
            Ko, _, _ = oracle.cg_rainbow(A, C, V, workloads.uniform_vector(1000 + k, n), diag, rbo, 1.0,
                                         precision=PRECISION)
            times.append(time.perf_counter() - t0)
        dt = float(np.median(times))
        oracle.set_threads(1)
        t0 = time.perf_counter()
        oracle.cg_rainbow(A, C, V, workloads.uniform_vector(1000, n), diag, rbo, 1.0, precision=PRECISION)
        dt1 = time.perf_counter() - t0
        t0 = time.perf_counter()
        oracle.rainbow(A, C)
        rb_cpu = time.perf_counter() - t0
        oracle.set_threads(threads)
        cpu = {"value": 1.0 / dt, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"median of 3 full FP64 Rainbow SSOR-PCG solves of the workload ({Ko} iterations, "
                         f"reference stopping rule), oracle restatement with OpenMP within colors",
               "value_1_thread": 1.0 / dt1,
               "rainbow_construction_ms": {"cpu_oracle": 1000.0 * rb_cpu, "library_host": rb_ms}}

    def rate(ms_list):
        return len(ms_list) / (sum(ms_list) / 1000.0)

    if rank == 0:
        rb64_ms = float(np.median(rb64))
        cg64_ms = float(np.median(cg64))
        dropin_ms = 1000 * float(np.median(dropin))
        cpu_ms = 1000.0 / cpu["value"] if cpu else None
        # the same-config comparisons, compact and last on the line
        like = {
            "mixed_batched_solves_per_s": value,
            "fp64_batched_solves_per_s": fp64_batched["solves_per_s"],
            "mixed_over_fp64_batched": value / fp64_batched["solves_per_s"],
            "mixed_batched_over_fp64_plain_cg_single": value / (1000.0 / cg64_ms),
            "fp64_rainbow_gpu_single_ms": rb64_ms,
            "fp64_rainbow_dropin_host_call_ms": dropin_ms,
            "fp64_rainbow_cpu_ms": cpu_ms,
            "dropin_device_speedup_vs_cpu": (cpu_ms / rb64_ms) if cpu_ms else None,
            "dropin_host_call_speedup_vs_cpu": (cpu_ms / dropin_ms) if cpu_ms else None,
            "mixed_rel_error_max_vs_fp64": accuracy["rel_error_max"],
        }
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": WORKLOAD_NAME if args.level == 5 else
                       f"PROFILING CASE ONLY: 3D P2 refined {args.level}x, N={n}, nnz={nnz}",
                       "solver": "batched mixed precision: FP32 inner Rainbow SSOR-PCG (compensated dots) inside "
                                 "FP64 defect correction, K right-hand sides per team (autotuned)",
                       "batch": B_RHS, "rhs_per_team": K_TEAM, "autotuner": tuned,
                       "l2": "flushed (256 MB write) before every timed step; working set > L2",
                       "replicas": "independent batches per GPU (replicas only)"},
            "batch_latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99))},
            "p50_ms": float(np.percentile(mixed1, 50)), "p99_ms": float(np.percentile(mixed1, 99)),
            "latency_note": "p50/p99 of one solve on the whole GPU (mixed, persistent cooperative kernel); "
                            "batch_latency_ms is the time to finish a whole batch",
            "inner_iterations": int(np.median(inner_iters)), "outer_iterations": int(np.median(outer_iters)),
            "true_relres_max": max(i["true_relres"] for i in flat),
            "single_solve_mixed": {"solves_per_s": rate(mixed1), "ms": float(np.median(mixed1)),
                                   "iterations": int(np.median([i["iterations"] for i in mixed1_i])),
                                   "error_estimate": float(np.median([i["error_estimate"] for i in mixed1_i])),
                                   "inner_fp64": int(mixed1_i[-1]["inner_fp64"]),
                                   "choice_measured_on": mixed1_measured},
            "fp64_batched_rainbow": fp64_batched,
            "fp64_plain_cg": {"solves_per_s": rate(cg64), "ms": cg64_ms,
                              "iterations": int(np.median([i["iterations"] for i in cg64_i])),
                              "note": "plain FP64 CG on the whole GPU, stop at true relres 1e-10"},
            "fp64_rainbow_reference_rule": {"solves_per_s": rate(rb64), "ms": rb64_ms,
                                            "iterations": int(np.median([i["iterations"] for i in rb64_i]))},
            "fp64_eisenstat_rainbow_reference_rule": {"solves_per_s": rate(eis64), "ms": float(np.median(eis64)),
                                                      "iterations": int(np.median([i["iterations"] for i in eis64_i]))},
            "dropin_host_call": {"ms": dropin_ms, "iterations": dropin_K},
            "spmv": spmv,
            **extras,
            "accuracy": accuracy,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clock_info,
            "like_for_like": like,
        }
        print(json.dumps(line), flush=True)
    sysm.close()
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--batch", type=int, default=1216, help="right-hand sides per batched step")
    ap.add_argument("--only-spmv", action="store_true", help="only the resident SpMV measurement")
    ap.add_argument("--only-uneven", action="store_true", help="only the 512 uneven systems batch")
    ap.add_argument("--only-serving", action="store_true", help="only the serving stream")
    ap.add_argument("--only-block-rhs", action="store_true", help="only the 64 right-hand-side blocked batch")
    ap.add_argument("--only-mixed-large", action="store_true", help="only the 3D P1 L7 mixed-precision solves")
    ap.add_argument("--only-csr-algebra", action="store_true", help="only the CSR algebra leg (product, transpose, sum)")
    ap.add_argument("--only-krylov-more", action="store_true", help="only the CR / MINRES / Hodge leg")
    ap.add_argument("--only-small", action="store_true", help="only the drop-ins on 2D P1 L6 (N = 4,225)")
    ap.add_argument("--only-single", action="store_true",
                    help="only single solves on the whole GPU (drop-in persistent kernels) on the headline operator")
    ap.add_argument("--only-batched", action="store_true",
                    help="only the batched headline step (no single-solve, SpMV, CPU or extra legs)")
    ap.add_argument("--rhs-per-team", type=int, default=0,
                    help="fixed right-hand sides per team instead of the autotuner's choice (profiling)")
    ap.add_argument("--team-threads", type=int, default=512, help="with --rhs-per-team: threads per team block")
    ap.add_argument("--team-blocks", type=int, default=1, help="with --rhs-per-team: blocks per team (cluster)")
    ap.add_argument("--level", type=int, default=5,
                    help="refinement level of the 3D P2 headline operator (5 = the benchmark; smaller only for "
                         "profiling captures)")
    ap.add_argument("--requests", type=int, default=200, help="requests in the serving stream")
    ap.add_argument("--full", action="store_true",
                    help="also run the side legs (uneven batch, 64-RHS block, 3D P1 L7 mixed, CSR algebra, further "
                         "drivers, small drop-ins, serving); each has its own --only-* switch as well")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
