"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

bench.py --gpus N runs one replica of the batched workload per GPU (weak scaling, no data-path
collective): ranks meet at a barrier around the timed region and the timing is the maximum over
ranks.  This checks that rendezvous, barrier and max-reduction on CPU ranks, and that the
reference arm leaves non-zero ranks without work.
"""

import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch.distributed as dist

    import bench
    ws, r, local = bench.dist_init()
    bench.barrier(ws)
    slowest = bench.max_over_ranks(ws, float(10 * (rank + 1)), "cpu")
    bench.barrier(ws)
    q.put((r, ws, slowest))
    dist.destroy_process_group()


def test_two_rank_barrier_and_max_timing():
    import torch
    if torch.cuda.is_available():
        pytest.skip("runs the gloo path; a GPU box uses NCCL")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2, 20.0), (1, 2, 20.0)]


def test_reference_arm_nonzero_rank_does_no_work(monkeypatch):
    """Under torchrun only rank 0 of the reference arm runs; the others return at once."""
    import bench
    calls = []
    monkeypatch.setattr(bench, "dist_init", lambda: (2, 1, 1))
    monkeypatch.setattr(bench, "cpu_oracle_rate", lambda *a, **k: calls.append(a) or (1.0, 1.0))

    class A:
        steps, warmup = 3, 3
    assert bench.run_reference(A()) == 0
    assert calls == []


def test_bench_gpus_two_launches_two_ranks():
    """`bench.py --gpus 2` outside torchrun starts two ranks itself (gloo on a CPU host); the
    reference arm runs on rank 0 only and reports the run's world size."""
    import json
    import subprocess
    import sys
    import torch
    if torch.cuda.is_available():
        pytest.skip("runs the gloo path; a GPU box uses NCCL")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, env=env,
                       cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0


def test_bench_refuses_mismatched_world_size():
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, WORLD_SIZE="3")
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--impl", "reference"],
                       capture_output=True, text=True, timeout=120, env=env, cwd=root)
    assert r.returncode == 2 and "WORLD_SIZE" in r.stderr
