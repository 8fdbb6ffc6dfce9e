"""Benchmark of the nls time-stepping path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

One bench step = one complete solve of the workload: by default the batched form, 512 independent
solves (256 radial grids of 500-8192 nodes, 256 square grids of 64-512 per side; seeded
synthetic inputs) advanced 5000 RK4 steps each in complex64 by one graph-captured launch
sequence.  Throughput is node-steps/s (one node-step = one grid point advanced one full RK4
step).  The line also carries the plain complex128 GPU path on a sample of the same instances,
the relative L2 error of |psi|^2 and of the reservoir n against complex128 solves, a short
served stream (p50/p99), the roofline of the fused 2-D step kernel, the CPU oracle timed on the
host cores, the end-to-end figure through the host-buffer C ABI, and the SM clocks sampled
during the timed region.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "node-steps/s batched FP32 vs plain FP64 GPU at relL2≤1e-4; serve p50/p99 ms"
UNIT = "node-steps/s"
SOLVE_STEPS = 5000  # RK4 steps per solve of the batched mix (the --solve-steps default)
# Algorithmic HBM bytes per node-step of the fused single-pass 2-D step (complex64 state read and
# written once, float32 pump read once): 8 + 4 + 8.
BYTES_PER_NODE_STEP_C64 = 20


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# 2-D fused-step kernel of each tile shape (the C ABI's 2-D variant numbers)
SHAPE_KERNELS = {
    1: "rk4_2d_fused 64x64 region, 512 threads", 2: "rk4_2d_fused 128x32, 512 threads",
    3: "rk4_2d_fused 32x32, 256 threads", 4: "rk4_2d_fused 64x64, 1024 threads",
    5: "rk4_2d_fused 128x32, 1024 threads", 6: "rk4_2d_fused 64x(64+8K), 512 threads",
    7: "rk4_2d_fused 64x(64+8K), 768/640 threads", 8: "rk4_2d_reg 64x80, 16 warps x 5 rows",
    9: "rk4_2d_reg 64x96, 12 warps x 8 rows", 10: "rk4_2d_reg 64x96, 8 warps x 12 rows",
    11: "rk4_2d_reg 64x64, 16 warps x 4 rows", 12: "rk4_2d_reg 64x72, 8 warps x 9 rows",
    13: "rk4_2d_reg 64x72, 12 warps x 6 rows", 14: "rk4_2d_reg 64x80, 8 warps x 10 rows",
    15: "rk4_2d_stream, 64-column strips walked as a four-stage wavefront (cp.async row ring)",
}
DEFAULT_SHAPE_C64 = 15


def _traffic_per_node():
    """DRAM bytes per node per fused-step launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "rk4_2d_stream_c64_batch_mix.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_node_step:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clock/throttle sampling every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local


def launch_ranks(n: int) -> int:
    """--gpus N outside torchrun: start N ranks of this command (one per GPU, rendezvous on
    127.0.0.1) with torch.distributed.run and return its exit status; rank 0 prints the line."""
    import socket
    sk = socket.socket()
    sk.bind(("127.0.0.1", 0))
    port = sk.getsockname()[1]
    sk.close()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, value: float, device) -> float:
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ CPU oracle leg

def cpu_oracle_rate(specs, steps, threads):
    """node-steps/s of the float32 oracle (the reference algorithm, C++ restatement) over specs."""
    from oracle import oracle
    oracle.build()
    t0 = time.perf_counter()
    ns = 0
    for s in specs:
        oracle.solve(s.dt, s.dx, s.order, steps, s.pumping, s.coeffs, s.u0, dtype=np.float32,
                     threads=threads if s.dim == 2 else 1)
        ns += s.nodes * steps
    dt = time.perf_counter() - t0
    return ns / dt, dt


def oracle_sample(specs):
    """Bounded sample of the mix for the CPU leg: every 4th instance of each kind."""
    return [s for i, s in enumerate(specs) if i % 4 == 0]


def calibrated_steps(specs, threads, target_s=20.0, max_steps=2000):
    """RK4 steps per CPU sample so that one sample takes about target_s seconds."""
    steps = 1
    while True:   # grow the probe until it runs long enough to time
        _, t = cpu_oracle_rate(specs, steps, threads)
        if t > 0.25 or steps >= max_steps:
            break
        steps *= 4
    return int(min(max_steps, max(1, round(steps * target_s / max(t, 1e-6)))))


def run_reference(args):
    """--impl reference: the reference algorithm on the host cores (the oracle port), same metric."""
    ws, rank, local = dist_init()
    if rank != 0:
        return 0
    from nls_gb300 import workloads
    specs = oracle_sample(workloads.batch_mix())
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_oracle_rate(specs[:8], 1, threads)
    steps = calibrated_steps(specs, threads, target_s=15.0)
    rates, times = [], []
    for _ in range(args.steps):
        r, t = cpu_oracle_rate(specs, steps, threads)
        rates.append(r)
        times.append(t)
    value = float(np.mean(rates))
    sample = f"every 4th of the 512 mixed instances ({len(specs)} solves), {steps} RK4 steps each, float32"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(times) * 1e3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex64",
        "data": "synthetic (seeded)",
        "config": {"workload": "batch_mix", "instances": 512, "steps_per_solve": SOLVE_STEPS},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's Fortran cannot be compiled here (no Fortran compiler); the oracle's C++ "
                "restatement of nls/nls.f90 is timed instead",
    }
    print(json.dumps(line))
    return 0


def run_cpu(args):
    """--workload cpu: the reference algorithm (the float32 oracle, a C++ restatement of
    nls/nls.f90) on this host's cores for configs 0-2, on 1 thread (the reference is
    single-threaded) and on all cores (OpenMP over 2-D columns; a 1-D solve stays sequential),
    each a bounded sample of about 3 s of RK4 steps; one JSON line."""
    from nls_gb300 import workloads
    cores = os.cpu_count() or 1
    cases = [("config 0: 1-D 1000 nodes on [0,40], order 5, complex64", workloads.plain_1d()[0]),
             ("config 1: 2-D 256^2 on [-20,20]^2, order 3, complex64", workloads.plain_2d()[0]),
             ("config 2: 2-D 1024^2 on [-40,40]^2, order 5, complex64", workloads.precision_2d()[0])]
    out = []
    for name, spec in cases:
        for threads in sorted({1, cores}):
            if spec.dim == 1 and threads > 1:
                continue
            steps = calibrated_steps([spec], threads, target_s=3.0, max_steps=100000)
            rate, secs = cpu_oracle_rate([spec], steps, threads)
            out.append({"case": name, "threads": threads, "steps": steps, "seconds": secs,
                        "node_steps_per_s": rate})
    print(json.dumps({"workload": "cpu", "kind": "port", "cores": cores,
                      "note": "float32 oracle (the reference's algorithm and precision); the "
                              "reference's Fortran cannot be compiled here", "results": out}))
    return 0


# ------------------------------------------------------------------ GPU legs

def pinned_fields(b, specs):
    """The batch's pumps, initial states and outputs as three pinned (page-locked) host blocks in
    the batch's packed layout (``BatchSolver.layout``), inputs filled from the specs; returns the
    blocks and the per-instance views of the output block."""
    import torch
    _, _, pb, sb = b.layout()
    blocks = [torch.empty(int(nb), dtype=torch.uint8, pin_memory=True).numpy() for nb in (pb, sb, sb)]
    hP, hU, hO = blocks
    for s, p, u in zip(specs, b.packed_views(hP, "pump"), b.packed_views(hU, "state")):
        p[...] = np.asarray(s.pumping)
        u[...] = np.asarray(s.u0)
    return hP, hU, hO


def run_grid(args):
    """--workload grid1d|grid2d: one solve of one grid (profiling and single-solve roofline)."""
    import torch
    ws, rank, local = dist_init()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    from nls_gb300 import build as nbuild
    nbuild.build()
    from nls_gb300 import device as ndev
    from nls_gb300 import workloads
    dtype = np.complex128 if args.c128 else np.complex64
    if args.workload == "grid2d":
        s, _ = workloads.plain_2d(n=args.n, length=args.n * 0.15625, order=args.order)
    else:
        s, _ = workloads.plain_1d(n=args.n, length=args.n * 0.04, order=args.order)
    ct = torch.complex128 if args.c128 else torch.complex64
    rt = torch.float64 if args.c128 else torch.float32
    u = torch.tensor(np.ascontiguousarray(s.u0), dtype=ct, device=dev)
    P = torch.tensor(np.ascontiguousarray(s.pumping), dtype=rt, device=dev)
    kw = dict(order=s.order, dt=s.dt, dx=s.dx, coeffs=s.coeffs, variant=args.variant)
    for _ in range(args.warmup):
        ndev.solve_(u, P, iters=args.solve_steps, **kw)
    ext = ndev.stream(local)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(args.steps):
        ndev.solve_(u, P, iters=args.solve_steps, **kw)
    e1.record(ext)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    ns = float(s.nodes) * args.solve_steps * args.steps
    bpn = 40 if args.c128 else 20
    print(json.dumps({"workload": args.workload, "n": args.n, "order": args.order, "dtype": np.dtype(dtype).name,
                      "variant": args.variant, "node_steps_per_s": ns / (ms / 1e3),
                      "us_per_rk4_step": ms * 1e3 / (args.solve_steps * args.steps),
                      "algorithmic_GBps": ns * bpn / (ms / 1e3) / 1e9}))
    return 0


def run_precision(args):
    """--workload precision2d: 1024^2 on [-40, 40]^2, ring radius 15 width 2, order 5, dt 1e-5,
    50 000 complex64 steps with FP64 norm / chemical potential every 500 steps, then the relative
    L2 error of |psi|^2 and n against a complex128 run of the same problem."""
    import torch
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    from nls_gb300 import build as nbuild
    nbuild.build()
    from nls_gb300 import precision, workloads
    s, steps = workloads.precision_2d()
    if args.solve_steps != SOLVE_STEPS:
        steps = args.solve_steps
    res = precision.run(s, steps=steps, log_every=500, device=local)
    log = res["log"]
    print(json.dumps({
        "workload": "precision2d: 1024x1024 on [-40,40]^2, ring radius 15 width 2 amplitude 6, order 5, dt 1e-5, "
                    f"{steps} steps, complex64 state, FP64 diagnostics every 500 steps",
        "c64_node_steps_per_s": res["c64_node_steps_per_s"], "c64_seconds": res["c64_seconds"],
        "c128_node_steps_per_s": res["c128_node_steps_per_s"], "c128_seconds": res["c128_seconds"],
        "rel_l2_density": res["rel_l2_density"], "rel_l2_reservoir": res["rel_l2_reservoir"],
        "log_first": log[0], "log_last": log[-1], "log_entries": len(log),
        "norm_min": min(e["norm"] for e in log), "norm_max": max(e["norm"] for e in log)}))
    return 0


def run_serve(args):
    """--workload serve: a Poisson stream of requests (default 10 000 at 200 req/s) drawn from the
    mixed 1-D/2-D distribution with 1000-20000 steps each, complex64 state, 80 GB admission budget,
    continuously batched; p50/p99 latency and node-steps/s, next to sequential plain complex128
    solves of a sample of the same requests."""
    import torch
    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    from nls_gb300 import build as nbuild
    nbuild.build()
    from nls_gb300 import device as ndev
    from nls_gb300 import workloads
    from nls_gb300.serve import Pool, serve
    count = args.serve if args.serve > 0 else 10000
    reqs = workloads.serve_stream(count)
    tuned = None
    if args.autotune:
        # kernel variants tuned on the batched mix, which has the stream's size and parameter
        # distribution
        from nls_gb300 import autotune
        tuned = autotune.apply(workloads.batch_mix(), dtype=np.complex64, device=local, mode="batch")
        autotune.assign([spec for spec, _ in reqs], tuned)
    pool = Pool(dtype=np.complex64, budget_bytes=80 << 30, chunk_steps=args.chunk, device=local)
    st = serve(reqs, rate=200.0, pool=pool)
    pool.close()
    # sequential plain complex128 solves of a sample of the same requests
    dev = torch.device("cuda", local)
    plain_ns, plain_s = 0.0, 0.0
    for spec, steps in reqs[:: max(1, count // 24)][:24]:
        u = torch.tensor(np.ascontiguousarray(spec.u0), dtype=torch.complex128, device=dev)
        P = torch.tensor(np.ascontiguousarray(spec.pumping), dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        ndev.solve_(u, P, order=spec.order, dt=spec.dt, dx=spec.dx, coeffs=spec.coeffs, iters=steps)
        torch.cuda.synchronize(dev)
        plain_s += time.perf_counter() - t0
        plain_ns += float(spec.nodes) * steps
    lat = st["latency_s"]
    print(json.dumps({"workload": f"serve: {count} requests, Poisson 200/s, steps U[1000,20000], complex64, "
                                  f"80 GB budget, chunk {args.chunk} steps",
                      "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": float(np.mean(lat) * 1e3),
                      "max_ms": float(np.max(lat) * 1e3), "wall_s": st["wall_s"],
                      "node_steps_per_s": st["node_steps_per_s"], "node_steps": st["node_steps"],
                      "queue_p50_ms": st["queue_p50_ms"], "queue_p99_ms": st["queue_p99_ms"],
                      "gpu_busy_frac": st["gpu_busy_frac"],
                      "plain_c128_sequential_node_steps_per_s": plain_ns / plain_s,
                      "plain_c128_sample": "24 requests of the stream solved one after another",
                      "autotuned_variants": tuned}))
    return 0


# Algorithmic FP64 work of one node-step of the plain complex128 path (one RK4 step = four
# right-hand sides + the RK4 combinations), counted per node and stage: the operator row (1-D
# order 5: five complex-by-real multiply-adds, 20 flop; 2-D order 3: four neighbour sums and two
# weights per component, 12 flop), |u|^2 (3), the reservoir (multiply, add, divide: 3), a and b
# (4), the right-hand side (8) and the stage update plus accumulation (8).
FP64_FLOP_PER_NODE_STEP = {(1, 5): 4 * (20 + 3 + 3 + 4 + 8 + 8), (2, 3): 4 * (12 + 3 + 3 + 4 + 8 + 8)}


def measured_fp64_peak(dev):
    """FP64 FLOP/s of cuBLAS DGEMM (4096^3, best of 5) on this GPU: the FP64 denominator."""
    import torch
    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize(dev)
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2.0 * 4096 ** 3 / best


def plain_config_leg(spec, steps, dev, fp64_peak, threads):
    """One plain complex128 solve of a configuration, device-timed on resident tensors (CUDA events
    on the library's stream, after one warm-up solve), and end to end through the f2py-shaped
    call (host arrays in, host array out); relative L2 against the FP64 oracle outside the timed
    regions."""
    import torch
    from nls_gb300 import device as ndev
    from nls_gb300.native import nls
    from oracle import oracle
    u0 = np.asarray(spec.u0).T if spec.dim == 2 else np.asarray(spec.u0)
    P = np.asarray(spec.pumping).T if spec.dim == 2 else np.asarray(spec.pumping)
    Pt = torch.tensor(np.ascontiguousarray(P), dtype=torch.float64, device=dev)
    kw = dict(order=spec.order, dt=spec.dt, dx=spec.dx, coeffs=spec.coeffs)
    u = torch.tensor(np.ascontiguousarray(u0), dtype=torch.complex128, device=dev)
    ndev.solve_(u, Pt, iters=steps, **kw)                         # warm-up
    u = torch.tensor(np.ascontiguousarray(u0), dtype=torch.complex128, device=dev)
    ext = ndev.stream(dev.index or 0)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    ndev.solve_(u, Pt, iters=steps, **kw)
    e1.record(ext)
    e1.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    t0 = time.perf_counter()
    fn = nls.solve_nls if spec.dim == 1 else nls.solve_nls_2d
    got = fn(spec.dt, spec.dx, spec.order, steps, spec.pumping, spec.coeffs, spec.u0)
    e2e_sec = time.perf_counter() - t0
    want = oracle.solve(spec.dt, spec.dx, spec.order, steps, spec.pumping, spec.coeffs, spec.u0, dtype=np.float64,
                        threads=threads)
    rel = float(np.linalg.norm(got - want) / np.linalg.norm(want))
    dev_rel = float(np.linalg.norm((u.cpu().numpy().T if spec.dim == 2 else u.cpu().numpy()) - want)
                    / np.linalg.norm(want))
    ns = float(spec.nodes) * steps
    flop = FP64_FLOP_PER_NODE_STEP.get((spec.dim, spec.order))
    out = {"us_per_step": sec * 1e6 / steps, "node_steps_per_s": ns / sec, "seconds": sec,
           "e2e_node_steps_per_s": ns / e2e_sec, "rel_l2_vs_fp64_oracle": max(rel, dev_rel)}
    if flop and fp64_peak:
        achieved = ns * flop / sec
        out["fp64"] = {"flop_per_node_step": flop, "achieved_tflops": achieved / 1e12,
                       "peak_tflops": fp64_peak / 1e12, "frac": achieved / fp64_peak,
                       "peak_source": "cuBLAS DGEMM 4096^3 measured in this run"}
    return out


def run_ours(args):
    import torch
    ws, rank, local = dist_init()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    from nls_gb300 import build as nbuild
    nbuild.build()
    from nls_gb300 import device as ndev
    from nls_gb300 import workloads
    from nls_gb300.batch import BatchSolver
    from nls_gb300.native import nls

    specs = workloads.batch_mix()
    tuned = None
    if args.batch_variant is not None:
        for sp in specs:
            if sp.dim == 2:
                sp.variant = args.batch_variant
    elif args.autotune:
        from nls_gb300 import autotune
        tuned = autotune.apply(specs, dtype=np.complex64, device=local, mode="batch")
    total_nodes = sum(s.nodes for s in specs)
    nodes_2d = sum(s.nodes for s in specs if s.dim == 2)
    b = BatchSolver(specs, dtype=np.complex64, device=local)
    ext = ndev.stream(local)

    # warm-up: includes graph capture/instantiation for SOLVE_STEPS
    steps_per_solve = args.solve_steps
    for _ in range(args.warmup):
        b.run(steps_per_solve)
    b.synchronize()

    launches0 = ndev.launches(local)
    barrier(ws)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(ext)
        for _ in range(args.steps):
            b.run(steps_per_solve)
        e1.record(ext)
        e1.synchronize()
    torch.cuda.synchronize(dev)
    barrier(ws)
    ms = e0.elapsed_time(e1)
    gpu_launches = ndev.launches(local) - launches0
    ms = max_over_ranks(ws, ms, dev)
    node_steps = float(total_nodes) * steps_per_solve * args.steps * ws
    value = node_steps / (ms / 1e3)
    clocks = clk.summary()

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "complex64", "data": "synthetic (seeded)",
        "config": {"workload": "batch_mix: 256 radial grids (500-8192 nodes, order 5) + 256 square grids "
                               "(64-512 per side, order 3), 5000 RK4 steps each, complex64",
                   "instances": len(specs), "steps_per_solve": steps_per_solve, "total_nodes": total_nodes,
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                   "l2": "inputs larger than L2 (2-D states + pumps ~%.0f MB per step)" %
                         (nodes_2d * BYTES_PER_NODE_STEP_C64 / 1e6)},
        "gpu_launches": int(gpu_launches),
        "clocks": clocks,
    }
    if tuned:
        result["config"]["autotuned_variants"] = tuned
    if rank != 0:
        return 0
    if args.quick:
        print(json.dumps(result))
        return 0

    # ---- end to end through the host-buffer C ABI: upload u0 and P from pinned host memory,
    # solve, download every state into pinned host memory (right after the timed region, on the
    # same batch, before the other legs allocate)
    hP, hU, hO = pinned_fields(b, specs)
    h2d, d2h = hP.nbytes + hU.nbytes, hO.nbytes   # the copied blocks, 256-byte padding included
    e2e_times, phases = [], []
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for rep in range(1 + max(1, min(args.steps, 3))):   # the first pass is an untimed warm-up
        b.ctx.synchronize()
        t0 = time.perf_counter()
        b.set_packed(hP, hU)
        t1 = time.perf_counter()
        r0.record(ext)
        b.run(SOLVE_STEPS)
        r1.record(ext)
        b.get_packed(hO)
        t2 = time.perf_counter()
        if rep:
            e2e_times.append(t2 - t0)
            phases.append(((t1 - t0) * 1e3, r0.elapsed_time(r1), (t2 - t0) * 1e3))
    outs = b.packed_views(hO, "state")
    for i in (0, len(specs) // 2, len(specs) - 1):   # the packed download is the batch's state
        if not np.array_equal(outs[i], b.get(i)):
            raise RuntimeError(f"packed download differs from nls_batch_get for instance {i}")
    del outs
    e2e = float(total_nodes) * SOLVE_STEPS / float(np.mean(e2e_times))
    result["e2e"] = {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                     "path": "nls_batch_set_packed (pinned host blocks of every P and u0) -> nls_batch_run(5000) -> "
                             "nls_batch_get_packed (pinned host block of every u)",
                     "ms_upload_run_total": [[round(x, 2) for x in ph] for ph in phases]}
    del hP, hU, hO

    # ---- roofline of the fused 2-D step kernel (the dominant kernel), timed alone on its stream
    specs2 = [s for s in specs if s.dim == 2]
    b2 = BatchSolver(specs2, dtype=np.complex64, device=local)
    L = 200
    b2.run(L)
    b2.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ndev.launches(local)
    f0.record(ext)
    b2.run(L)
    f1.record(ext)
    f1.synchronize()
    l1 = ndev.launches(local)
    launch_s = f0.elapsed_time(f1) / 1e3 / L
    alg_bytes = BYTES_PER_NODE_STEP_C64 * nodes_2d
    peak, peak_kind = _peaks()
    achieved = alg_bytes / launch_s / 1e9
    tpn = _traffic_per_node()
    peak_source = ("MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)" if peak_kind == "measured" else
                   "fallback 6.8 TB/s (an earlier GB300 copy measurement; no MEASURED_PEAKS.json present)")
    result["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak, "traffic": (tpn * nodes_2d if tpn else None),
                          "kernel": "; ".join(sorted({SHAPE_KERNELS.get(v if v > 0 else DEFAULT_SHAPE_C64, str(v))
                                                      for v in (sp.variant for sp in specs2)}))
                                    + "; every 2-D instance in one work list",
                          "algorithmic_bytes_per_step": alg_bytes, "avg_step_us": launch_s * 1e6,
                          "steps_timed": L, "launches_timed": int(l1 - l0),
                          "note": "achieved = algorithmic bytes of the timed RK4 steps / their CUDA-event time "
                                  "(the streaming kernel runs up to 512 steps per launch on this list)",
                          "peak_source": peak_source}
    b2.close()

    # ---- accuracy of the batched complex64 results and the plain complex128 path on a sample
    sample_idx = list(range(0, 256, 32)) + list(range(256, 512, 32))
    import torch as T
    errs_d, errs_n = [], []
    plain_ns, plain_s = 0.0, 0.0
    # a fresh batch of the sample: exactly SOLVE_STEPS steps from u0
    bs = BatchSolver([specs[i] for i in sample_idx], dtype=np.complex64, device=local)
    bs.run(SOLVE_STEPS)
    bs.synchronize()
    for k, i in enumerate(sample_idx):
        s = specs[i]
        P64 = np.asfortranarray(s.pumping, dtype=np.float64) if s.dim == 2 else np.asarray(s.pumping, np.float64)
        u64 = np.asfortranarray(s.u0, dtype=np.complex128) if s.dim == 2 else np.asarray(s.u0, np.complex128)
        flat = lambda a: np.ravel(a, order="K")
        tu = T.tensor(flat(u64).copy(), device=dev)
        tP = T.tensor(flat(P64).copy(), device=dev)
        shp = (s.n, s.n) if s.dim == 2 else (s.n,)
        tu = tu.reshape(shp)
        tP = tP.reshape(shp)
        T.cuda.synchronize(dev)
        t0 = time.perf_counter()
        ndev.solve_(tu, tP, order=s.order, dt=s.dt, dx=s.dx, coeffs=s.coeffs, iters=SOLVE_STEPS)
        T.cuda.synchronize(dev)
        plain_s += time.perf_counter() - t0
        plain_ns += float(s.nodes) * SOLVE_STEPS
        got = bs.get(k)
        tg = T.tensor(np.ravel(got, order="K").copy(), device=dev).reshape(shp)
        d, r = ndev.density_errors(tg, tu, tP, s.coeffs)
        errs_d.append(d)
        errs_n.append(r)
    bs.close()
    plain_rate = plain_ns / plain_s
    result["plain_c128"] = {"value": plain_rate, "unit": UNIT,
                            "sample": f"{len(sample_idx)} of the 512 instances, sequential complex128 solves, "
                                      f"{SOLVE_STEPS} steps each (nls_solve_device)"}
    result["batched_over_plain"] = value / ws / plain_rate
    result["rel_l2_vs_c128"] = {"density_max": max(errs_d), "reservoir_max": max(errs_n),
                                "sample": f"same {len(sample_idx)} instances after {SOLVE_STEPS} steps"}

    # ---- the single-solve configurations: plain complex128 config 0 (1-D) and config 1 (2-D), and
    # the precision form on config 2, each against its FP64 reference
    if not args.no_configs:
        threads = os.cpu_count() or 1
        fp64_peak = measured_fp64_peak(dev)
        s0, st0 = workloads.plain_1d()
        result["plain_config0"] = dict(plain_config_leg(s0, st0, dev, fp64_peak, threads),
                                       config="1-D radial 1000 nodes on [0,40], order 5, dt 1e-4, 10 000 steps, "
                                              "complex128")
        s1, st1 = workloads.plain_2d()
        result["plain_config1"] = dict(plain_config_leg(s1, st1, dev, fp64_peak, threads),
                                       config="2-D 256^2 on [-20,20]^2, ring pump, order 3, dt 5e-5, 20 000 steps, "
                                              "complex128")
        from nls_gb300 import precision
        s2, st2 = workloads.precision_2d()
        res = precision.run(s2, steps=st2, log_every=500, device=local)
        result["precision_config2"] = {
            "config": "2-D 1024^2 on [-40,40]^2, ring radius 15 width 2, order 5, dt 1e-5, 50 000 steps; complex64 "
                      "state, FP64 norm and chemical potential every 500 steps, simulated time in FP64",
            "c64_node_steps_per_s": res["c64_node_steps_per_s"], "c64_seconds": res["c64_seconds"],
            "c128_node_steps_per_s": res["c128_node_steps_per_s"], "c128_seconds": res["c128_seconds"],
            "rel_l2_density": res["rel_l2_density"], "rel_l2_reservoir": res["rel_l2_reservoir"],
            "reference": "the plain complex128 GPU path on the same problem (pinned to the FP64 oracle at <= 1e-10 "
                         "by the test suite; the FP64 CPU oracle would need hours for 5e10 node-steps)",
            "log_entries": len(res["log"])}
        del res

    # ---- served stream (continuous batching) p50/p99
    if args.serve > 0:
        from nls_gb300.serve import Pool, serve
        reqs = workloads.serve_stream(args.serve)
        if tuned:
            from nls_gb300 import autotune
            autotune.assign([spec for spec, _ in reqs], tuned)
        pool = Pool(dtype=np.complex64, budget_bytes=80 << 30, chunk_steps=500, device=local)
        st = serve(reqs, rate=200.0, pool=pool)
        pool.close()
        offered = sum(float(sp.nodes) * k for sp, k in reqs) / float(
            np.cumsum(np.random.default_rng(7).exponential(1.0 / 200.0, size=len(reqs)))[-1])
        result["serve"] = {"requests": args.serve, "rate_per_s": 200.0, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                           "queue_p50_ms": st["queue_p50_ms"], "queue_p99_ms": st["queue_p99_ms"],
                           "node_steps_per_s": st["node_steps_per_s"], "offered_node_steps_per_s": offered,
                           "gpu_busy_frac": st["gpu_busy_frac"], "wall_s": st["wall_s"],
                           "budget_gb": 80, "chunk_steps": 500,
                           "stream": "Poisson arrivals (seed 7), steps U[1000, 20000], mixed 1-D/2-D sizes, complex64"}

    # ---- CPU oracle on the host cores (bounded sample)
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        samp = oracle_sample(specs)
        csteps = calibrated_steps(samp, threads)
        rate, secs = cpu_oracle_rate(samp, csteps, threads)
        result["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                  "sample": f"every 4th of the 512 instances ({len(samp)} solves) x {csteps} RK4 "
                                            f"steps, float32 C++ restatement of nls/nls.f90 (OpenMP over 2-D "
                                            f"columns), {secs:.1f} s"}
    print(json.dumps(result))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--serve", type=int, default=10000, help="requests in the served stream (0 = skip)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the plain config 0/1 and precision config 2 legs")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle leg")
    ap.add_argument("--quick", action="store_true",
                    help="timed batched solves only (no roofline, accuracy, e2e, serve or CPU legs)")
    ap.add_argument("--workload", choices=["batch", "grid1d", "grid2d", "precision2d", "serve", "cpu"],
                    default="batch")
    ap.add_argument("--chunk", type=int, default=500, help="serving pool chunk (RK4 steps per scheduling round)")
    ap.add_argument("--solve-steps", type=int, default=SOLVE_STEPS, help="RK4 steps per solve")
    ap.add_argument("--n", type=int, default=4096, help="grid size for grid1d/grid2d")
    ap.add_argument("--order", type=int, default=3, help="stencil order for grid1d/grid2d")
    ap.add_argument("--variant", type=int, default=-1, help="kernel variant for grid1d/grid2d")
    ap.add_argument("--c128", action="store_true", help="complex128 state for grid1d/grid2d")
    ap.add_argument("--batch-variant", type=int, default=None, help="2-D kernel variant for the batch")
    ap.add_argument("--autotune", action=argparse.BooleanOptionalAction, default=True,
                    help="choose kernel variants per size with the batch-throughput autotuner")
    args = ap.parse_args()
    ws_env = os.environ.get("WORLD_SIZE")
    if ws_env is None and args.gpus > 1:
        return launch_ranks(args.gpus)
    if ws_env is not None and int(ws_env) != args.gpus:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={ws_env}; launch one rank per GPU", file=sys.stderr)
        return 2
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "precision2d":
        return run_precision(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "cpu":
        return run_cpu(args)
    if args.workload != "batch":
        return run_grid(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
