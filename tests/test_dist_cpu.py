"""The N > 1 replica path of bench.py on CPU with the gloo backend (world size 2): the reductions
that turn per-rank times and cell counts into the whole-job figure, and the launcher contract of the
reference arm (rank 0 alone runs and prints one line, the other ranks exit 0)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out):
    os.environ.update({"WORLD_SIZE": "2", "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    dist, r, ws, local = bench.dist_setup()
    assert dist is not None and r == rank and ws == 2 and local == rank
    bench.barrier(dist)
    mx = bench.dist_max(dist, 1.5 + rank)           # slowest rank's time
    sm = bench.dist_sum(dist, 1000.0 * (rank + 1))  # cells of all ranks
    bench.barrier(dist)
    out.put((rank, mx, sm))
    dist.destroy_process_group()


def test_bench_reductions_over_two_gloo_ranks():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.5, 3000.0), (1, 2.5, 3000.0)]


def test_reference_arm_under_torchrun_prints_one_line(oracle_lib):
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "1", "--shape", "32,16,16"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
