"""Replica aggregation of bench.py on CPU with two gloo ranks: the timed region of the
slowest replica bounds the job (max over ranks), whole-job throughput counts every
replica's units, and the reference arm runs on rank 0 only (other ranks exit without
output). Rendezvous on 127.0.0.1."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(10.0 * (rank + 1), "cpu")
    rate = bench.whole_job_rate(100, world, t)
    # the reference arm: only rank 0 does work and prints
    out = io.StringIO()
    if rank != 0:
        class A:  # the arguments run_reference reads before it returns on rank != 0
            steps = 1; warmup = 3; gpus = world
        with redirect_stdout(out):
            bench.run_reference(A())
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, rate, out.getvalue()))


def test_max_over_ranks_and_whole_job_rate_with_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, rate, out in res:
        assert t == 20.0                      # max over ranks, seen by every rank
        assert rate == pytest.approx(2 * 100 / 20.0)
    assert res[1][3] == ""                    # rank 1 of the reference arm prints nothing


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10, 1, 2.0) == 5.0


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` at N = 1: one JSON line with the arm's own metric, unit and
    config, whole solves of the headline workload timed on the host cores (the oracle's
    restatement of the reference's Rainbow SSOR-PCG), and zero-copy e2e."""
    import json
    import subprocess
    sys.path.insert(0, ROOT)
    import bench
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "solves/s"
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3          # W is raised to 3
    assert d["higher_is_better"] is True and d["config"]["workload"] == bench.WORKLOAD_NAME
    assert d["value"] > 0 and d["ms_per_step"] == pytest.approx(1000.0 / d["value"])
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["iterations"] > 0
