"""The multi-rank path of bench.py on CPU (gloo, world size 2).

The traversal shards without an exchange step, so N GPUs run N independent
replicas; the only collectives are the timing barrier and the max over ranks
of the elapsed time. These tests run that host logic with two gloo ranks.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import argparse

    import bench
    args = argparse.Namespace(impl="reference")
    w, r, _ = bench.dist_setup(args)
    assert (w, r) == (world, rank)
    bench.barrier(w)
    m = bench.reduce_max(float(rank + 1) * 1.5, w, "cpu")
    Path(out_dir, f"rank{rank}.txt").write_text(repr(m))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    assert [float((tmp_path / f"rank{r}.txt").read_text()) for r in (0, 1)] == [3.0, 3.0]


@pytest.mark.slow
def test_reference_arm_under_torchrun_prints_one_line(built):
    """`bench.py --impl reference` under torchrun with two ranks: rank 0 alone
    times the CPU restatement and prints one JSON line; rank 1 exits 0."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("reference", "port")
