"""Project-written autotuner for kernel shape and stage fusion.

For each (dimension, precision, stencil order, grid-size bucket) it times the candidate kernel
variants on a seeded instance of that size and keeps the fastest:

* 2-D: 0 = unfused (four stage launches per step, no halo recomputation), or a fused
  single-pass step: column-strip tiles (rk4_2d_fused) with region 64x64 / 512 threads (1),
  128x32 / 512 (2), 32x32 / 256 (3), 64x64 / 1024 (4), 128x32 / 1024 (5), 64x(64+8K) / 512 (6) or
  768/640 (7), or register-resident row-strip tiles (rk4_2d_reg, complex64) with region 64x80 /
  512 (8), 64x96 / 384 (9), 64x96 / 256 (10), 64x64 / 512 (11), 64x72 / 256 (12), 64x72 / 384 (13)
  or 64x80 / 256 (14), or the streaming wavefront over 64-column strips (rk4_2d_stream, complex64,
  15);
* 1-D: the resident kernel on 1, 2, 4, 8 or 16 CTAs of a cluster, or 0 = unfused stage kernels.

Two objectives: ``mode="single"`` times one solve of the size (latency of a lone solve), and
``mode="batch"`` times a batch of copies large enough to fill the GPU (throughput per node-step,
what a batched or served mix cares about: a shape with less halo recomputation wins there even
when it exposes fewer tiles per grid).  For a batch, ``apply`` also times the batch's own 2-D
specs under one shared shape (one persistent launch per step instead of one per shape) against
the per-size choices and keeps the faster, then refines the 1-D cluster sizes on the batch itself
(one pass of coordinate descent over the size buckets, largest first): inside a mix the 1-D grids
share the GPU with the 2-D steps, so the fewest CTAs per grid often cost the batch least.  Per-size results are cached per GPU name in a JSON
file (``NLS_GB300_TUNE_CACHE`` or ``~/.cache/nls_gb300/autotune.json``); ``apply(specs, dtype,
mode)`` fills ``Spec.variant``.  Timings use CUDA events on the library's stream.
"""

from __future__ import annotations

import copy
import json
import os
import threading

import numpy as np

_lock = threading.Lock()


def _cache_path():
    return os.environ.get("NLS_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "nls_gb300", "autotune.json"))


def bucket(n: int) -> int:
    """Size bucket: the next power of two (for 2-D, of the side)."""
    b = 1
    while b < n:
        b *= 2
    return b


def feasible_1d(n: int, cl: int, order: int, dtype) -> bool:
    """The resident 1-D kernels' size rule: a segment of ceil(n / cl) nodes fits the CTA's limit
    (4096 nodes complex64, 2048 complex128), a cluster also holding 8K halo nodes, K = (order-1)/2."""
    if cl == 0:
        return True                      # unfused stage kernels: any size
    K = (order - 1) // 2
    lim = 4096 if np.dtype(dtype) == np.dtype(np.complex64) else 2048
    seg = -(-n // cl)
    if cl == 1:
        return 2 * K <= seg <= lim
    return 1 < cl <= 16 and seg >= 4 * K and seg + 8 * K <= lim


def candidates(dim: int, dtype, n: int, order: int = 5):
    c64 = np.dtype(dtype) == np.dtype(np.complex64)
    if dim == 2:
        return [15, 10, 12, 13, 14, 9, 8, 11, 6, 1, 7, 2, 3, 4, 5, 0] if c64 else [0, 3]
    return [cl for cl in (1, 2, 4, 8, 16) if feasible_1d(n, cl, order, dtype)] + [0]


def _time_variant(dim, n, order, dtype, variant, steps, device):
    import torch

    from . import device as ndev
    from . import workloads
    if dim == 2:
        s, _ = workloads.plain_2d(n=n, length=n * 0.15625, order=order)
    else:
        s, _ = workloads.plain_1d(n=n, length=n * 0.04, order=order)
    ct = torch.complex64 if np.dtype(dtype) == np.dtype(np.complex64) else torch.complex128
    rt = torch.float32 if ct == torch.complex64 else torch.float64
    u = torch.tensor(np.ascontiguousarray(s.u0), dtype=ct, device=f"cuda:{device}")
    P = torch.tensor(np.ascontiguousarray(s.pumping), dtype=rt, device=f"cuda:{device}")
    kw = dict(order=order, dt=s.dt, dx=s.dx, coeffs=s.coeffs, variant=variant)
    ndev.solve_(u, P, iters=steps, **kw)           # warm-up (graph instantiation, attributes)
    ext = ndev.stream(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    ndev.solve_(u, P, iters=steps, **kw)
    e1.record(ext)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def _time_batch(dim, n, order, dtype, variant, steps, device):
    """ms per node-step of a batch of copies of this size with the given variant."""
    import torch

    from . import device as ndev
    from . import workloads
    from .batch import BatchSolver
    if dim == 2:
        s, _ = workloads.plain_2d(n=n, length=n * 0.15625, order=order)
    else:
        s, _ = workloads.plain_1d(n=n, length=n * 0.04, order=order)
    s.variant = variant
    copies = max(1, min(512, (8 << 20) // max(1, s.nodes)))
    b = BatchSolver([s] * copies, dtype=dtype, device=device)
    try:
        b.run(steps)
        ext = ndev.stream(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        b.run(steps)
        e1.record(ext)
        e1.synchronize()
        return e0.elapsed_time(e1) / (steps * copies * s.nodes)
    finally:
        b.close()


def tune(dim: int, n: int, order: int, dtype=np.complex64, steps: int = 128, device: int = 0,
         mode: str = "single"):
    """Fastest variant for this case (cached)."""
    import torch
    name = torch.cuda.get_device_name(device)
    key = f"{name}|{mode}|{dim}|{np.dtype(dtype).name}|{order}|{bucket(n)}"
    path = _cache_path()
    with _lock:
        cache = {}
        if os.path.exists(path):
            try:
                with open(path) as f:
                    cache = json.load(f)
            except (OSError, ValueError):
                cache = {}
        if key in cache:
            return int(cache[key]["variant"])
    times = {}
    nb = bucket(n)
    timer = _time_batch if mode == "batch" else _time_variant
    for v in candidates(dim, dtype, nb, order):
        if mode == "batch" and v == 0:
            continue          # the unfused path is a single-solve fallback
        try:
            times[v] = timer(dim, nb, order, dtype, v, steps, device)
        except ValueError:
            continue
    best = min(times, key=times.get)
    with _lock:
        cache[key] = {"variant": int(best), "ms_per_step": {str(k): t for k, t in times.items()}}
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, path)
    return int(best)


def _time_mix(specs, dtype, variant, steps, device):
    """ms per node-step of one batch of exactly these specs with the 2-D variant forced."""
    trial = []
    for s in specs:
        t = copy.copy(s)
        t.variant = variant
        trial.append(t)
    return _time_mix_assigned(trial, dtype, steps, device)


def tune_mix(specs, dtype=np.complex64, steps: int = 32, device: int = 0):
    """One 2-D tile shape for a whole batch of 2-D specs of one stencil order, timed on that batch.

    All of the batch's 2-D tiles then go to a single persistent launch per step, which balances
    better over the SMs than one launch per shape."""
    times = {}
    n_max = max(s.n for s in specs)
    for v in candidates(2, dtype, bucket(n_max)):
        if v == 0:
            continue
        try:
            times[v] = _time_mix(specs, dtype, v, steps, device)
        except ValueError:
            continue
    best = min(times, key=times.get)
    return int(best), times


def apply(specs, dtype=np.complex64, device: int = 0, mode: str = "batch"):
    """Set each Spec.variant from the tuned choice; returns the choices.

    1-D specs: the fastest cluster size of their size bucket; in ``batch`` mode then refined on
    the batch itself.  2-D specs: per size bucket in ``single`` mode; in ``batch`` mode one shape
    per stencil order, timed on the batch itself (``tune_mix``), unless the per-bucket choices
    together time faster on it."""
    memo = {}
    out = {}
    two_d = {}
    for s in specs:
        if s.dim == 2 and mode == "batch":
            two_d.setdefault(s.order, []).append(s)
            continue
        k = (s.dim, s.order, bucket(s.n))
        if k not in memo:
            memo[k] = tune(s.dim, s.n, s.order, dtype=dtype, device=device, mode=mode)
        s.variant = memo[k]
    for order, group in sorted(two_d.items()):
        best, times = tune_mix(group, dtype=dtype, device=device)
        # per-bucket choices as one more candidate
        per = {}
        for s in group:
            k = (order, bucket(s.n))
            if k not in per:
                per[k] = tune(2, s.n, order, dtype=dtype, device=device, mode="batch")
        trial = [copy.copy(s) for s in group]
        for t in trial:
            t.variant = per[(order, bucket(t.n))]
        t_per = _time_mix_assigned(trial, dtype, 32, device)
        if t_per < times[best]:
            for s in group:
                s.variant = per[(order, bucket(s.n))]
            for (o, b), v in sorted(per.items()):
                out[f"2d/o{o}/n<={b}"] = v
        else:
            for s in group:
                s.variant = best
            out[f"2d/o{order}/mix"] = best
    # 1-D in a batch: the per-size choices above maximise the throughput of a GPU full of copies
    # of one grid, which favours wide clusters; inside a mix the 1-D grids share the SMs with the
    # 2-D steps and fewer CTAs per grid can cost less SM time.  One pass of coordinate descent on
    # the batch itself, largest size bucket first, over that bucket's cluster sizes.
    if mode == "batch" and any(s.dim == 1 for s in specs):
        keys = sorted({(s.order, bucket(s.n)) for s in specs if s.dim == 1}, key=lambda k: -k[1])
        best_t = _time_mix_assigned([copy.copy(s) for s in specs], dtype, 32, device)
        for order, b in keys:
            group = [s for s in specs if s.dim == 1 and s.order == order and bucket(s.n) == b]
            for v in candidates(1, dtype, b, order):
                if v == 0 or v == group[0].variant:
                    continue
                trial = [copy.copy(s) for s in specs]
                for t in trial:
                    if t.dim == 1 and t.order == order and bucket(t.n) == b:
                        t.variant = v
                try:
                    t_v = _time_mix_assigned(trial, dtype, 32, device)
                except ValueError:
                    continue
                if t_v < best_t:
                    best_t = t_v
                    for s in group:
                        s.variant = v
                    memo[(1, order, b)] = v
    for (d, o, b), v in sorted(memo.items()):
        out[f"{d}d/o{o}/n<={b}"] = v
    return out


def _time_mix_assigned(specs, dtype, steps, device):
    """ms per node-step of one batch of these specs with their own variants."""
    import torch

    from . import device as ndev
    from .batch import BatchSolver
    b = BatchSolver(specs, dtype=dtype, device=device)
    try:
        b.run(steps)
        ext = ndev.stream(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        b.run(steps)
        e1.record(ext)
        e1.synchronize()
        return e0.elapsed_time(e1) / (steps * sum(s.nodes for s in specs))
    finally:
        b.close()


def assign(specs, choices):
    """Apply the choices ``apply`` returned (for one population) to other specs of the same
    population, e.g. the requests of a served stream: per size bucket, or the shared 2-D shape of
    a stencil order ("2d/o3/mix").  Specs with no matching choice keep their variant.
    A 1-D cluster size chosen on one size of a bucket that does not fit another size of it
    becomes the smallest larger cluster that fits (or the built-in choice)."""
    for s in specs:
        key = f"{s.dim}d/o{s.order}/n<={bucket(s.n)}"
        mix = f"{s.dim}d/o{s.order}/mix"
        if key in choices:
            s.variant = int(choices[key])
        elif mix in choices:
            s.variant = int(choices[mix])
        if s.dim == 1 and s.variant > 0 and not feasible_1d(s.n, s.variant, s.order, np.complex64):
            fit = [cl for cl in (1, 2, 4, 8, 16) if cl > s.variant and feasible_1d(s.n, cl, s.order, np.complex64)]
            s.variant = fit[0] if fit else -1
    return specs
