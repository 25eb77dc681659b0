"""The N > 1 path of bench.py on the CPU with the gloo backend, world size 2: replicas with a
barrier, the max-over-ranks time, the aggregate over ranks, and the reference arm under
torchrun printing one JSON line from rank 0 while the other rank exits without work.
The path does not shard (replicas only), so there is no data-path collective to test."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import argparse

    import bench
    world_, rank_, local, pg = bench.dist_setup(argparse.Namespace(impl="reference"))
    ms = 100.0 + 50.0 * rank_  # rank 1 is the slower replica
    ms_max = bench.allmax(pg, ms)
    steps = 3
    value = world_ * steps / (ms_max / 1000.0)
    pg.barrier()
    (Path(out_dir) / f"rank{rank_}.json").write_text(
        json.dumps({"world": world_, "local": local, "ms_max": ms_max, "value": value}))
    pg.barrier()
    pg.destroy_process_group()


def test_two_replicas_take_the_slowest_time(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, free_port(), str(tmp_path)), nprocs=2, join=True)
    r = [json.loads((tmp_path / f"rank{k}.json").read_text()) for k in range(2)]
    for k in range(2):
        assert r[k]["world"] == 2 and r[k]["local"] == k
        assert r[k]["ms_max"] == 150.0  # both ranks see the slower replica's time
        assert r[k]["value"] == pytest.approx(2 * 3 / 0.150)  # units of both ranks / max time


def test_reference_arm_under_torchrun_prints_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--scale", "8"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
