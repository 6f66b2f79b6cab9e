"""The N > 1 paths of bench.py on CPU: gloo ranks, world size 2.

Replicas are independent, so the only cross-rank operations are the timing
barrier and the max over ranks; the reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "ATM_BENCH_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import bench

    r, w, local, pg = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(pg)
    # per-rank step times: the job time is the slowest rank's
    m = bench.max_over_ranks(1.5 + rank, pg)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(repr(m))
    pg.destroy_process_group()


def test_max_over_ranks_and_barrier_gloo(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    vals = [float(open(tmp_path / f"rank{r}.txt").read()) for r in range(2)]
    assert vals == [2.5, 2.5]


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("torch")
    env = dict(os.environ, ATM_BENCH_BACKEND="gloo", OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0"]
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["unit"] == "evals/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
