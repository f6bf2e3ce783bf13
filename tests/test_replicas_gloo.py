"""Replica plumbing of ``bench.py`` for N > 1 ranks, on the CPU.

The path has no exchange step, so N GPUs run N independent replicas; what
the ranks share is the timing: the slowest rank's step time (all-reduce MAX)
and the whole-job rate (all ranks' units over that time).  Two ranks run
here as spawned processes on the ``gloo`` backend; the reference arm under
torchrun runs on rank 0 only and the other ranks exit without output.
"""

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = bench.slowest_rank_ms(10.0 + 2.0 * rank, world, torch.device("cpu"))
    rate = bench.replica_rate(2_000_000, world, ms)
    dist.barrier()
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"ms": ms, "rate": rate}))
    dist.destroy_process_group()


def test_slowest_rank_time_and_whole_job_rate(tmp_path):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    alive = [p for p in procs if p.is_alive()]
    for p in alive:
        p.kill()
    assert not alive, "a gloo rank did not finish"
    assert all(p.exitcode == 0 for p in procs)
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    for r in res:
        assert r["ms"] == 12.0  # the slower rank's time on every rank
        assert r["rate"] == pytest.approx(2 * 2_000_000 / 0.012 / 1e6)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.slowest_rank_ms(7.5, 1, None) == 7.5
    assert bench.replica_rate(1_000_000, 1, 10.0) == pytest.approx(100.0)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
