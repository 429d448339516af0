"""bench.py's multi-GPU form (independent replicas, one rank per GPU) on CPU:
world_size 2 over gloo.  The data path has no collective; the ranks only meet
at the barriers around the timed region and in the max-over-ranks of the time."""

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

REPO = Path(__file__).resolve().parent.parent


def _ranks(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(REPO))
    import bench
    w, r = bench.dist_setup()
    assert (w, r) == (world, rank)
    import torch.distributed as dist
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    # each rank "took" a different time; the job time is the slowest rank's
    t = bench.allreduce_max(w, 1.0 + rank)
    mlups = bench.whole_job_mlups(w, 1000, 10, t)
    out.put((rank, t, mlups))
    bench.barrier(w)
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_value():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_ranks, args=(r, 2, 29517, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _ in res] == [2.0, 2.0]
    assert all(abs(m - 2 * 1000 * 10 / 2.0 / 1e6) < 1e-12 for _, _, m in res)


def test_reference_arm_under_torchrun_runs_on_rank_zero_only(tmp_path):
    """--impl reference with two ranks: rank 0 prints the one JSON line, rank 1 exits 0."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29531", str(REPO / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "3", "--size", "20", "--radius", "3"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["unit"] == "MLUPS" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
