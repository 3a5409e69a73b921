"""bench.py's multi-rank path on CPU (gloo, world size 2): the max-over-ranks timing and
barrier of the replica runs, and the reference arm under torchrun (rank 0 alone prints one
line; the other ranks exit 0 without work)."""
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


def _rank_main(rank, ws, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist(use_gpu=False)
    d.barrier()
    # per-rank step times: the job's time is the slowest rank's
    ms = 2.0 + rank
    sec = d.max(ms) / 1e3
    value = bench.replica_value(ws, 1000, sec)
    d.barrier()
    d.close()
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"sec": sec, "value": value}, f)


def test_dist_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    ws, port = 2, free_port()
    mp.start_processes(_rank_main, args=(ws, port, str(tmp_path)), nprocs=ws, join=True,
                       start_method="spawn")
    for r in range(ws):
        got = json.load(open(tmp_path / f"r{r}.json"))
        assert got["sec"] == pytest.approx(3.0e-3)       # max of 2 ms and 3 ms
        assert got["value"] == pytest.approx(2 * 1000 / 3.0e-3)


def test_reference_arm_two_ranks():
    """--impl reference under torchrun with two ranks on a small mesh: one JSON line."""
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--scale", "16"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port"
