"""Benchmark: solves/s at 1e-10 relative residual on the 3D P2 Lagrange operator
refined 5 times (N = 274,625, nnz = 7,678,721), multicolor (Rainbow) SSOR-PCG.

One step = one complete solve of A x = b from x0 = 0 to a true FP64 relative
residual <= 1e-10, with a fresh seeded U[-1,1] right-hand side. The headline
`value` is the mixed-precision product path (FP32 inner Rainbow SSOR-PCG with
compensated dots inside an FP64 defect-correction loop) with b and x resident
in HBM; `e2e` is the same solve through the public System API with the
right-hand side copied in from pinned host memory and the solution copied back
inside the timed region. The plain FP64 GPU CG and the FP64 drop-in Rainbow
solver (the reference's own stopping rule) on the same matrix are reported beside
it, together with the oracle (a plain-C restatement of the reference solver)
timed on the host cores.

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
    A, C, V = workloads.lattice_matrix(**WORKLOAD)
    n = len(A) - 1
    nnz = len(C)
    mat = S.MatrixCSR(n, n, A, C, V)
    diag = mat.getDiagonal().raw()
    rb = S.Rainbow(mat)
    sysm = System(A, C, V)
    sysm.set_rainbow(diag, 1.0, rb.num_colors, rb.F, rb.B, rb.R)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)   # 256 MB > L2 (129 MB)

    def rhs(step):
        return workloads.uniform_vector(1000 + step + 7919 * rank, n)

    def timed_solves(method, mode, steps, warmup, seed_base=0):
        per = []
        infos = []
        stream = torch.cuda.current_stream()
        for step in range(warmup + steps):
            b = torch.from_numpy(rhs(seed_base + step)).to(dev)
            x = torch.zeros(n, dtype=torch.float64, device=dev)
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            info = sysm.solve(b, x, method=method, mode=mode, precision=PRECISION)
            e1.record(stream)
            torch.cuda.synchronize()
            if step >= warmup:
                per.append(e0.elapsed_time(e1))
                infos.append(info)
        return per, infos

    # warm-up of the headline path, then the timed region (clocks sampled during it)
    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lib.feec_kernel_launches()
    clocks.start()
    per, infos = timed_solves("rainbow", "mixed", args.steps, args.warmup)
    clock_info = clocks.stop()
    launches = lib.feec_kernel_launches() - launches0
    torch.cuda.synchronize()
    total_ms = float(sum(per))
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        dist.barrier()
    value = world * args.steps / (total_ms / 1000.0)
    assert all(i["status"] == 0 and i["true_relres"] <= PRECISION for i in infos), infos
    inner_iters = [i["iterations"] for i in infos]
    outer_iters = [i["outer_iterations"] for i in infos]

    # roofline of the dominant kernel: the FP32 inner persistent PCG launch
    it_b = rainbow_iteration_bytes(n, nnz, 8, 4)
    rs_b = rainbow_restart_bytes(n, nnz, 8, 4)
    inner_bytes = sum(o * rs_b + k * it_b for o, k in zip(outer_iters, inner_iters))
    inner_ms = sum(i["device_ms"] for i in infos)
    launches_inner = sum(outer_iters)
    peak, peak_kind = measured_peaks()
    achieved = inner_bytes / (inner_ms / 1000.0) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "kernel": "pcg_persistent<float>",
                "bytes_per_launch": inner_bytes / launches_inner, "ms_per_launch": inner_ms / launches_inner,
                "peak_kind": peak_kind}

    # end to end: pinned host b -> device, solve, device -> pinned host x, all inside the timed region
    e2e_per = []
    hb = torch.empty(n, dtype=torch.float64).pin_memory()
    hx = torch.empty(n, dtype=torch.float64).pin_memory()
    db = torch.empty(n, dtype=torch.float64, device=dev)
    for step in range(args.warmup + args.steps):
        hb.copy_(torch.from_numpy(rhs(500 + step)))
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        db.copy_(hb, non_blocking=True)
        x = torch.zeros(n, dtype=torch.float64, device=dev)
        sysm.solve(db, x, method="rainbow", mode="mixed", precision=PRECISION)
        hx.copy_(x, non_blocking=True)
        torch.cuda.synchronize()
        if step >= args.warmup:
            e2e_per.append(time.perf_counter() - t0)
    e2e_value = world * args.steps / sum(e2e_per)

    # plain FP64 GPU CG and the FP64 drop-in Rainbow (reference stopping rule) on the same matrix
    cg_steps = max(1, min(3, args.steps))
    cg_per, cg_infos = timed_solves("cg", "fp64", cg_steps, 1, seed_base=2000)
    rb64_per, rb64_infos = timed_solves("rainbow", "reference", max(1, min(5, args.steps)), 1, seed_base=3000)
    fp64_rb_per, fp64_rb_infos = timed_solves("rainbow", "fp64", max(1, min(5, args.steps)), 1, seed_base=4000)

    # drop-in host-pointer call (matrix uploaded inside the call, as the reference signature implies)
    b0 = rhs(6000)
    dropin = []
    for step in range(2):
        xh = np.zeros(n); res = np.zeros(n)
        t0 = time.perf_counter()
        S.ConjugateGradientSolverCSR_Rainbow(n, xh, b0, A, C, V, res, PRECISION, -3, diag, 1.0,
                                             rb.num_colors, rb.F, rb.B, rb.R)
        dropin.append(time.perf_counter() - t0)

    # CPU baseline: the oracle restatement of the reference Rainbow-PCG on the host cores, one solve
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle
        threads = os.cpu_count() or 1
        oracle.set_threads(threads)
        rbo = (rb.num_colors, rb.F, rb.B, rb.R)
        t0 = time.perf_counter()
        Ko, _, _ = oracle.cg_rainbow(A, C, V, rhs(0), diag, rbo, 1.0, precision=PRECISION)
        dt = time.perf_counter() - t0
        cpu = {"value": 1.0 / dt, "unit": "solves/s", "cores": threads, "kind": "port",
               "sample": f"1 full FP64 Rainbow SSOR-PCG solve of the workload ({Ko} iterations, reference "
                         f"stopping rule), oracle restatement with OpenMP"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": WORKLOAD_NAME, "solver": "mixed: FP32 inner Rainbow SSOR-PCG (compensated dots) + "
                       "FP64 defect correction", "l2": "flushed (256 MB write) before every solve",
                       "replicas": "independent solves per GPU (replicas only)"},
            "p50_ms": float(np.percentile(per, 50)), "p99_ms": float(np.percentile(per, 99)),
            "inner_iterations": int(np.median(inner_iters)), "outer_iterations": int(np.median(outer_iters)),
            "true_relres_max": max(i["true_relres"] for i in infos),
            "fp64_plain_cg": {"solves_per_s": cg_steps / (sum(cg_per) / 1000.0), "ms": float(np.median(cg_per)),
                              "iterations": int(np.median([i["iterations"] for i in cg_infos]))},
            "fp64_rainbow_reference_rule": {"solves_per_s": len(rb64_per) / (sum(rb64_per) / 1000.0),
                                            "ms": float(np.median(rb64_per)),
                                            "iterations": int(np.median([i["iterations"] for i in rb64_infos]))},
            "fp64_rainbow_true_residual": {"solves_per_s": len(fp64_rb_per) / (sum(fp64_rb_per) / 1000.0),
                                           "ms": float(np.median(fp64_rb_per)),
                                           "iterations": int(np.median([i["iterations"] for i in fp64_rb_infos]))},
            "dropin_host_call_ms": 1000 * float(np.median(dropin)),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n},
            "gpu_launches": int(launches),
            "clocks": clock_info,
        }
        print(json.dumps(line), flush=True)
    sysm.close()
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
