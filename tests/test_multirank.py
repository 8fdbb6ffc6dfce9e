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
