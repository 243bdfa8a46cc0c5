"""Multi-GPU is replicas only: every rank runs the whole workload, the job's
time is the slowest rank's, its value the sum over ranks, and no collective
touches the data path.  The cross-rank parts of bench.py run here on CPU as
two ranks over gloo (127.0.0.1)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            init_method=f"tcp://127.0.0.1:{port}")
    import bench
    got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5], world)
    Path(outdir, f"rank{rank}.json").write_text(json.dumps(got))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        assert json.loads((tmp_path / f"rank{r}.json").read_text()) == [2.0, 10.0, 0.5]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks([3, 4.5], 1) == [3.0, 4.5]


def test_reference_arm_under_torchrun_prints_once():
    """bench.py --impl reference with two ranks: rank 0 alone times the CPU
    path and prints one JSON line; the other rank exits 0 without work."""
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           str(ROOT / "bench.py"), "--gpus", "2", "--impl", "reference", "--steps", "1",
           "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] == 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0
