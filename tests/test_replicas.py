"""Multi-rank (replica) logic of bench.py on CPU: world size 2 over gloo.

TSQR does not shard across GPUs in this library (one problem per GPU), so a
run on N GPUs is N independent replicas. What the ranks share is host-side:
the barrier, the max-over-ranks of the step time, the whole-job rate and
rank 0 alone printing. These tests run that logic as two gloo processes on
127.0.0.1, and the reference arm under torchrun with two ranks.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_rank(rank, ws, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        dist.barrier()
        # rank r's step time; rank 1 is the slow one
        ms = bench.max_over_ranks(1.0 + 2.5 * rank, ws)
        flops = bench.flops(4096, 32)
        rate = bench.whole_job_rate(flops, ms, ws)
        q.put((rank, ms, rate))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_ws2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    assert all(p.exitcode == 0 for p in ps), [p.exitcode for p in ps]
    got = sorted(q.get(timeout=10) for _ in range(2))
    sys.path.insert(0, ROOT)
    import bench
    want_rate = 2 * bench.flops(4096, 32) / 3.5e-3
    for rank, ms, rate in got:
        assert ms == 3.5, (rank, ms)  # both ranks see the slowest rank's time
        assert rate == pytest.approx(want_rate, rel=1e-12)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.25, 1) == 2.25
    assert bench.whole_job_rate(100.0, 4.0, 1) == pytest.approx(25000.0)


def _bench_env(**kw):
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    env.update({k: str(v) for k, v in kw.items()})
    return env


def test_reference_arm_other_rank_exits_without_work():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--m", "8192"], cwd=ROOT,
                       env=_bench_env(WORLD_SIZE=2, RANK=1, LOCAL_RANK=1), capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_torchrun_ws2_prints_one_line(orc):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", "--master-port=%d" % _free_port(), "bench.py", "--impl", "reference",
           "--gpus", "2", "--rows", "16384", "--steps", "2", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, env=_bench_env(OMP_NUM_THREADS=2), capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 2
    assert d["value"] > 0 and d["unit"] == "TFLOP/s" and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0

