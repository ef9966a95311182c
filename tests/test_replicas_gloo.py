"""The N-GPU bench path is replicas (every rank runs the whole workload, no
collective in the data path): its only cross-rank pieces are the barrier,
the max-over-ranks time and the whole-job rate.  Checked here with two gloo
ranks on CPU, and the reference arm's rank rule (rank 0 alone runs it)."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, secs, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    dist.barrier()
    m = bench.max_over_ranks(torch, secs[rank], "cpu")
    q.put((rank, m, bench.job_rate(512 ** 3, 10, ws, m)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_with_two_gloo_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    secs = [0.25, 0.40]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, secs, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, rate in out:
        assert m == 0.40  # every rank reports the slowest rank's time
        assert rate == pytest.approx(512 ** 3 * 10 * 2 / 0.40 / 1e6)


def test_single_process_time_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(torch, 1.5, "cpu") == 1.5
    assert bench.job_rate(100, 2, 1, 0.5) == pytest.approx(100 * 2 / 0.5 / 1e6)


def _run_bench(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], env=env, capture_output=True,
                          text=True, timeout=600)


def test_reference_arm_runs_on_rank_zero_only():
    r = _run_bench({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--impl", "reference", "--gpus", "2")
    assert r.returncode == 0 and r.stdout.strip() == ""
    r = _run_bench({"RANK": "0", "WORLD_SIZE": "1"}, "--impl", "reference", "--steps", "4", "--ref-n", "32")
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
