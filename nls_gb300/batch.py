"""Batched form: many independent solves advanced together by one CUDA graph.

The reference solves one configuration per call and farms many configurations out to separate
processes (benchmark/benchmark.py:21-76; schedulr/workr.py:39-66).  ``BatchSolver`` keeps every
instance resident on the GPU -- radial 1-D grids in shared-memory resident kernels, 2-D grids in
fused-step tile kernels over one work list -- and ``run(steps)`` replays a cached graph.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib


@dataclass
class Spec:
    """One solve: dim 1 (radial, n nodes) or 2 (n x n), stencil order, steps sizes, coefficients."""
    dim: int
    n: int
    order: int
    dt: float
    dx: float
    coeffs: np.ndarray
    variant: int = -1
    pumping: np.ndarray = field(default=None, repr=False)
    u0: np.ndarray = field(default=None, repr=False)

    def problem(self) -> _lib.Problem:
        return _lib.make_problem(self.dim, self.n, self.order, self.dt, self.dx, self.coeffs, self.variant)

    @property
    def nodes(self) -> int:
        return self.n if self.dim == 1 else self.n * self.n


class BatchSolver:
    def __init__(self, specs, dtype=np.complex64, device: int = 0):
        self.code = _lib.dtype_code(dtype)
        self.ctype, self.rtype = _lib.np_types(self.code)
        self.ctx = _lib.default_context(device)
        self.specs = list(specs)
        arr = (_lib.Problem * len(self.specs))(*[s.problem() for s in self.specs])
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().nls_batch_create(self.ctx.handle, self.code, len(self.specs), arr, ctypes.byref(h)),
                   "nls_batch_create", self.ctx.handle)
        self.handle = h
        for i, s in enumerate(self.specs):
            if s.pumping is not None and s.u0 is not None:
                self.set(i, s.pumping, s.u0)

    def _field(self, i, a, dt):
        s = self.specs[i]
        a = np.asarray(a)
        if a.size != s.nodes:
            raise ValueError(f"instance {i}: expected {s.nodes} values, got {a.size}")
        return np.asfortranarray(a, dtype=dt) if s.dim == 2 else np.ascontiguousarray(a, dtype=dt)

    def set(self, i: int, pumping, u0):
        P = self._field(i, pumping, self.rtype)
        U = self._field(i, u0, self.ctype)
        _lib.check(_lib.lib().nls_batch_set(self.handle, i, _lib.ptr(P), _lib.ptr(U)), "nls_batch_set",
                   self.ctx.handle)

    def run(self, steps: int):
        _lib.check(_lib.lib().nls_batch_run(self.handle, int(steps)), "nls_batch_run", self.ctx.handle)

    def synchronize(self):
        self.ctx.synchronize()

    def get(self, i: int, out: np.ndarray = None) -> np.ndarray:
        """State of instance i; into ``out`` if given (the instance's shape and complex dtype,
        Fortran order in 2-D, e.g. a view of pinned host memory), else into a new array."""
        s = self.specs[i]
        shape = (s.n, s.n) if s.dim == 2 else (s.n,)
        if out is None:
            out = np.empty(shape, dtype=self.ctype, order="F" if s.dim == 2 else "C")
        elif (out.shape != shape or out.dtype != self.ctype or
              not (out.flags.f_contiguous if s.dim == 2 else out.flags.c_contiguous)):
            raise ValueError(f"instance {i}: out must be {shape} {np.dtype(self.ctype).name}, "
                             f"{'Fortran' if s.dim == 2 else 'C'} order")
        _lib.check(_lib.lib().nls_batch_get(self.handle, i, _lib.ptr(out)), "nls_batch_get", self.ctx.handle)
        return out

    def state_pointer(self, i: int):
        u, p = ctypes.c_void_p(), ctypes.c_void_p()
        _lib.check(_lib.lib().nls_batch_state(self.handle, i, ctypes.byref(u), ctypes.byref(p)), "nls_batch_state",
                   self.ctx.handle)
        return u.value, p.value

    def info(self, steps: int):
        l, n = ctypes.c_int64(), ctypes.c_int64()
        _lib.check(_lib.lib().nls_batch_info(self.handle, int(steps), ctypes.byref(l), ctypes.byref(n)),
                   "nls_batch_info", self.ctx.handle)
        return l.value, n.value

    def close(self):
        if self.handle:
            _lib.lib().nls_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
