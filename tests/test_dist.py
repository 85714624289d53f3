"""The multi-process path of bench.py on CPU (gloo, world size 2): rank
set-up from the launcher's environment, barrier, maximum over ranks, and
the reference arm under torch.distributed.run (rank 0 alone works and
prints).  The renderer path itself runs replicas with no collective."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local, pg = bench.dist_setup()
    bench.barrier(pg)
    m = bench.allmax(pg, 1.5 + r)
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"ws": ws, "rank": r, "local": local, "max": m}, f)
    pg.destroy_process_group()


def test_dist_setup_barrier_and_allmax(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_rank_main, args=(free_port(), str(tmp_path)), nprocs=2, join=True)
    for rank in (0, 1):
        d = json.load(open(tmp_path / f"r{rank}.json"))
        assert d == {"ws": 2, "rank": rank, "local": rank, "max": 2.5}


def test_reference_arm_under_torchrun():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--workload", "cube"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("reference", "port")
