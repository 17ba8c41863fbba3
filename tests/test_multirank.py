"""Multi-process paths of bench.py on the CPU (gloo, world_size 2, 127.0.0.1).

The library runs one replica per GPU with no data-path collective; the only
cross-rank operations are the barrier and the max-over-ranks step time used for
the whole-job rate.  These tests exercise that logic with two gloo ranks, and the
reference arm under torchrun, where rank 0 alone runs and prints.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    r, ws, _, dist = bench.dist_init()
    try:
        local_ms = 2.0 + r            # rank 1 is the slower replica
        ms = bench.max_over_ranks(local_ms, dist)
        q.put((r, ws, ms, bench.whole_job_rate(50.0e9, ms, ws)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    for r, ws, ms, rate in got:
        assert ws == 2 and ms == 3.0                                 # both ranks see the slowest rank
        assert rate == pytest.approx(2 * 50.0e9 / 3.0e-3 / 1e9)      # whole-job GFLOP/s


def test_reference_arm_under_torchrun_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--chi", "256", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
