"""Serving form: continuous batching of solve requests under an HBM admission budget.

The reference serves many solves through schedulr, an HTTP pull queue whose workers each run one
solve at a time on the CPU (schedulr/schedulr.py:48-154, schedulr/workr.py:88-102).  Here one
process owns the GPU: ``Pool`` admits requests while slots and budget are free, keeps every
admitted state resident, and each chunk advances all of them by up to ``chunk_steps`` steps in
one batched launch sequence; up to two chunks are in flight, admissions upload on a copy stream
while chunks run, a request that arrives while others run joins at the next chunk boundary and a
finished one leaves, freeing its memory for the queue.  Per-request
arithmetic never depends on what else is in the pool, so a result is the same alone and in the
mix.
"""

from __future__ import annotations

import ctypes
import time
from collections import deque

import numpy as np

from . import _lib
from .batch import Spec


class Pool:
    def __init__(self, dtype=np.complex64, budget_bytes: int = 80 << 30, max_slots: int = 2048,
                 chunk_steps: int = 250, device: int = 0, keep_inputs: bool = False):
        """keep_inputs: remember each admitted request (its Spec and step count) so that
        ``take_with_accuracy`` can report the result against a complex128 companion solve."""
        self.device = device
        self.keep_inputs = keep_inputs
        self._requests = {}
        self.code = _lib.dtype_code(dtype)
        self.ctype, self.rtype = _lib.np_types(self.code)
        self.ctx = _lib.default_context(device)
        self.chunk_steps = chunk_steps
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().nls_pool_create(self.ctx.handle, self.code, int(budget_bytes), int(max_slots),
                                              int(chunk_steps), ctypes.byref(h)), "nls_pool_create", self.ctx.handle)
        self.handle = h
        self._shapes = {}

    def admit(self, spec: Spec, steps: int, tag: int):
        """Returns the slot, or None when the pool has no room for this request now."""
        P = np.asfortranarray(spec.pumping, dtype=self.rtype) if spec.dim == 2 else \
            np.ascontiguousarray(spec.pumping, dtype=self.rtype)
        U = np.asfortranarray(spec.u0, dtype=self.ctype) if spec.dim == 2 else \
            np.ascontiguousarray(spec.u0, dtype=self.ctype)
        pr = spec.problem()
        slot = ctypes.c_int(-1)
        st = _lib.lib().nls_pool_admit(self.handle, ctypes.byref(pr), _lib.ptr(P), _lib.ptr(U), int(steps), int(tag),
                                       ctypes.byref(slot))
        if st == _lib.NLS_ERR_BUSY:
            return None
        _lib.check(st, "nls_pool_admit", self.ctx.handle)
        self._shapes[int(tag)] = (spec.n, spec.dim)
        if self.keep_inputs:
            self._requests[int(tag)] = (spec, int(steps))
        return slot.value

    def step(self) -> int:
        """Launch the next chunk (if fewer than two are in flight) and wait for the oldest one."""
        done = ctypes.c_int(0)
        _lib.check(_lib.lib().nls_pool_step(self.handle, ctypes.byref(done)), "nls_pool_step", self.ctx.handle)
        return done.value

    def launch(self) -> bool:
        """Enqueue the next chunk without waiting; False when two are in flight or nothing is left."""
        got = ctypes.c_int(0)
        _lib.check(_lib.lib().nls_pool_launch(self.handle, ctypes.byref(got)), "nls_pool_launch", self.ctx.handle)
        return bool(got.value)

    def wait(self) -> int:
        """Block until the oldest chunk in flight completes; the number of requests it finished."""
        done = ctypes.c_int(0)
        _lib.check(_lib.lib().nls_pool_wait(self.handle, ctypes.byref(done)), "nls_pool_wait", self.ctx.handle)
        return done.value

    def ready(self) -> bool:
        """True when the oldest chunk in flight has completed (or none is in flight)."""
        r = ctypes.c_int(0)
        _lib.check(_lib.lib().nls_pool_ready(self.handle, ctypes.byref(r)), "nls_pool_ready", self.ctx.handle)
        return bool(r.value)

    def info(self):
        """(chunks in flight, device milliseconds of all completed chunks)."""
        f, ms = ctypes.c_int(0), ctypes.c_double(0.0)
        _lib.check(_lib.lib().nls_pool_info(self.handle, ctypes.byref(f), ctypes.byref(ms)), "nls_pool_info",
                   self.ctx.handle)
        return f.value, ms.value

    def take(self):
        """Tag of the earliest finished request (its state is dropped), or None."""
        tag = ctypes.c_int64()
        st = _lib.lib().nls_pool_take(self.handle, ctypes.byref(tag), None, 0)
        if st == _lib.NLS_ERR_NOT_READY:
            return None
        _lib.check(st, "nls_pool_take", self.ctx.handle)
        return int(tag.value)

    def take_with_state(self):
        """(tag, final state) of the earliest finished request, or None."""
        tag = ctypes.c_int64()
        # a buffer large enough for any admitted request
        n_max = max((n * n if d == 2 else n) for (n, d) in self._shapes.values()) if self._shapes else 1
        buf = np.empty(n_max, dtype=self.ctype)
        st = _lib.lib().nls_pool_take(self.handle, ctypes.byref(tag), _lib.ptr(buf), buf.nbytes)
        if st == _lib.NLS_ERR_NOT_READY:
            return None
        _lib.check(st, "nls_pool_take", self.ctx.handle)
        n, d = self._shapes.pop(int(tag.value))
        if d == 1:
            return int(tag.value), buf[:n].copy()
        return int(tag.value), buf[: n * n].reshape((n, n), order="F").copy()

    def take_with_accuracy(self):
        """(tag, final state, (rel-L2 |psi|^2, rel-L2 n)) of the earliest finished request, the
        errors against a complex128 companion solve of the same request; or None.  Needs
        keep_inputs=True."""
        from . import device as ndev
        if not self.keep_inputs:
            raise ValueError("take_with_accuracy() needs Pool(..., keep_inputs=True)")
        got = self.take_with_state()
        if got is None:
            return None
        tag, state = got
        spec, steps = self._requests.pop(tag)
        return tag, state, ndev.companion_errors(state, spec, steps, self.device)

    def status(self):
        a, b = ctypes.c_int(), ctypes.c_size_t()
        _lib.check(_lib.lib().nls_pool_status(self.handle, ctypes.byref(a), ctypes.byref(b)), "nls_pool_status",
                   self.ctx.handle)
        return a.value, b.value

    def close(self):
        if self.handle:
            _lib.lib().nls_pool_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def serve(requests, rate: float, pool: Pool, seed: int = 7, keep_results: bool = False, clock=time.perf_counter):
    """Replay a Poisson stream of (Spec, steps) requests at `rate` per second through `pool`.

    The loop keeps the GPU fed: up to two chunks are in flight; while the oldest one runs, new
    arrivals are admitted (their uploads overlap the running chunk and join the next one) and
    finished requests are taken.  Returns per-request latency (completion minus arrival, seconds)
    with p50/p99, the queueing delay (admission minus arrival) with p50/p99, the wall time,
    node-steps/s over the whole stream, the GPU-busy fraction (device time of the chunks over the
    wall time) and results by tag if keep_results."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(requests))
    arrival = np.cumsum(gaps)
    queue = deque()
    nxt = 0
    lat = np.full(len(requests), np.nan)
    qdelay = np.full(len(requests), np.nan)
    results = {}
    done = 0
    t0 = clock()
    node_steps = 0.0

    def admit_arrivals():
        nonlocal nxt
        now = clock() - t0
        while nxt < len(requests) and arrival[nxt] <= now:
            queue.append(nxt)
            nxt += 1
        while queue:
            i = queue[0]
            spec, steps = requests[i]
            if pool.admit(spec, steps, i) is None:
                active, in_use = pool.status()
                if active == 0 and in_use == 0 and pool.info()[0] == 0:
                    raise RuntimeError(f"request {i} does not fit the pool even when it is empty")
                break
            qdelay[i] = clock() - t0 - arrival[i]
            queue.popleft()

    def take_finished():
        nonlocal done, node_steps
        while True:
            got = pool.take_with_state() if keep_results else pool.take()
            if got is None:
                break
            tag = got[0] if keep_results else got
            if keep_results:
                results[tag] = got[1]
            lat[tag] = clock() - t0 - arrival[tag]
            spec, steps = requests[tag]
            node_steps += float(spec.nodes) * steps
            done += 1

    while done < len(requests):
        admit_arrivals()
        while pool.launch():
            pass
        take_finished()
        if pool.info()[0] == 0:
            if not queue and nxt < len(requests):
                wait = arrival[nxt] - (clock() - t0)
                if wait > 0:
                    time.sleep(min(wait, 0.002))
            continue
        # the oldest chunk runs: admit arrivals meanwhile, then collect it
        while not pool.ready():
            admit_arrivals()
            time.sleep(0.0002)
        pool.wait()
        take_finished()
    wall = clock() - t0
    busy_ms = pool.info()[1]
    return {
        "latency_s": lat,
        "p50_ms": float(np.percentile(lat, 50) * 1e3),
        "p99_ms": float(np.percentile(lat, 99) * 1e3),
        "queue_p50_ms": float(np.percentile(qdelay, 50) * 1e3),
        "queue_p99_ms": float(np.percentile(qdelay, 99) * 1e3),
        "wall_s": wall,
        "node_steps": node_steps,
        "node_steps_per_s": node_steps / wall,
        "gpu_busy_frac": busy_ms / 1e3 / wall,
        "results": results,
    }
