"""Multi-rank path on CPU (gloo, world size 2): the skeletonization path runs
as replicas, so the only cross-rank logic is the barrier and the slowest
rank's time; the CPU reference arm of bench.py runs on rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g
    rep = g.load_package().replicas
    r, w = rep.init("gloo")
    rep.barrier()
    m = rep.max_over_ranks(10.0 + r)          # rank 1 is the slow one
    out.put((r, w, m))
    rep.finish()


def test_max_over_ranks_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 11.0), (1, 2, 11.0)]


def test_bench_reference_arm_torchrun_world2():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--unknowns", "4096",
           "--holes", "4", "--nrhs", "2"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    # rank 0 alone does the CPU work: one worker, two ranks launched
    assert d["impl"] == "reference" and d["n_gpus"] == 1
    assert d["config"]["ranks_launched"] == 2 and d["config"]["ranks_working"] == 1
    assert d["metric"].endswith("relative residual")
    assert d["config"]["residual_reached_max"] <= d["config"]["target_residual"]
    assert d["cpu_baseline"]["kind"] == "port" and d["value"] > 0
