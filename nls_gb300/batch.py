"""Batched form: many independent solves advanced together by one CUDA graph.

The reference solves one configuration per call and farms many configurations out to separate
processes (benchmark/benchmark.py:21-76; schedulr/workr.py:39-66).  ``BatchSolver`` keeps every
instance resident on the GPU -- radial 1-D grids in resident (register or shared-memory) kernels,
2-D grids in fused-step tile kernels over one work list -- and ``run(steps)`` replays a cached
graph.
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
    """keep_inputs: keep host copies of every instance's pump and initial state as the caller
    gave them (before the conversion to the working precision) and count the steps run since, so
    ``accuracy`` can report each result against a complex128 companion solve."""

    def __init__(self, specs, dtype=np.complex64, device: int = 0, keep_inputs: bool = False):
        self.device = device
        self.keep_inputs = keep_inputs
        self._inputs = {}
        self._steps = [0] * len(specs)
        self.code = _lib.dtype_code(dtype)
        self.ctype, self.rtype = _lib.np_types(self.code)
        self.ctx = _lib.default_context(device)
        self.specs = list(specs)
        arr = (_lib.Problem * len(self.specs))(*[s.problem() for s in self.specs])
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().nls_batch_create(self.ctx.handle, self.code, len(self.specs), arr, ctypes.byref(h)),
                   "nls_batch_create", self.ctx.handle)
        self.handle = h
        have = [i for i, s in enumerate(self.specs) if s.pumping is not None and s.u0 is not None]
        if len(have) == len(self.specs):
            self.set_many([s.pumping for s in self.specs], [s.u0 for s in self.specs])
        else:
            for i in have:
                self.set(i, self.specs[i].pumping, self.specs[i].u0)

    def _field(self, i, a, dt):
        s = self.specs[i]
        a = np.asarray(a)
        if a.size != s.nodes:
            raise ValueError(f"instance {i}: expected {s.nodes} values, got {a.size}")
        return np.asfortranarray(a, dtype=dt) if s.dim == 2 else np.ascontiguousarray(a, dtype=dt)

    def _record(self, i, pumping, u0):
        self._steps[i] = 0
        if self.keep_inputs:
            self._inputs[i] = (np.array(pumping, dtype=np.float64), np.array(u0, dtype=np.complex128))

    def set(self, i: int, pumping, u0):
        P = self._field(i, pumping, self.rtype)
        U = self._field(i, u0, self.ctype)
        _lib.check(_lib.lib().nls_batch_set(self.handle, i, _lib.ptr(P), _lib.ptr(U)), "nls_batch_set",
                   self.ctx.handle)
        self._record(i, pumping, u0)

    def run(self, steps: int):
        _lib.check(_lib.lib().nls_batch_run(self.handle, int(steps)), "nls_batch_run", self.ctx.handle)
        self._steps = [k + int(steps) for k in self._steps]

    def accuracy(self, indices=None):
        """Per-result relative L2 errors (|psi|^2, reservoir n) of the listed instances (all by
        default) against complex128 companion solves from their last uploaded inputs (as given,
        before the conversion to the working precision) over the steps run since, reduced in FP64
        on the device.  Needs keep_inputs=True."""
        from dataclasses import replace

        from . import device as ndev
        if not self.keep_inputs:
            raise ValueError("accuracy() needs BatchSolver(..., keep_inputs=True)")
        self.synchronize()
        out = []
        for i in (range(len(self.specs)) if indices is None else indices):
            P, U = self._inputs[i]
            spec = replace(self.specs[i], pumping=P, u0=U)
            u_ptr, _ = self.state_pointer(i)
            out.append(ndev.companion_errors(u_ptr, spec, self._steps[i], self.device))
        return out

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

    def set_many(self, pumpings, u0s, first: int = 0):
        """``set`` for instances first, first+1, ... in one call: every upload is queued and the
        call waits once.  The arrays must stay alive until it returns (it blocks)."""
        if len(pumpings) != len(u0s):
            raise ValueError("pumpings and u0s differ in length")
        count = len(u0s)
        if first < 0 or first + count > len(self.specs):
            raise ValueError("instance range out of bounds")
        Ps = [self._field(first + k, pumpings[k], self.rtype) for k in range(count)]
        Us = [self._field(first + k, u0s[k], self.ctype) for k in range(count)]
        pp = (ctypes.c_void_p * max(count, 1))(*[a.ctypes.data for a in Ps])
        pu = (ctypes.c_void_p * max(count, 1))(*[a.ctypes.data for a in Us])
        _lib.check(_lib.lib().nls_batch_set_many(self.handle, first, count, pp, pu), "nls_batch_set_many",
                   self.ctx.handle)
        for k in range(count):
            self._record(first + k, pumpings[k], u0s[k])

    def get_many(self, outs=None, first: int = 0, count: int = None):
        """``get`` for instances first, first+1, ... in one call (one wait).  ``outs``: arrays as
        ``get``'s ``out`` (e.g. views of pinned host memory), or None for new arrays."""
        if outs is None:
            count = len(self.specs) - first if count is None else count
            outs = [None] * count
        count = len(outs)
        if first < 0 or first + count > len(self.specs):
            raise ValueError("instance range out of bounds")
        res = []
        for k, out in enumerate(outs):
            s = self.specs[first + k]
            shape = (s.n, s.n) if s.dim == 2 else (s.n,)
            if out is None:
                out = np.empty(shape, dtype=self.ctype, order="F" if s.dim == 2 else "C")
            elif (out.shape != shape or out.dtype != self.ctype or
                  not (out.flags.f_contiguous if s.dim == 2 else out.flags.c_contiguous)):
                raise ValueError(f"instance {first + k}: out must be {shape} {np.dtype(self.ctype).name}, "
                                 f"{'Fortran' if s.dim == 2 else 'C'} order")
            res.append(out)
        pu = (ctypes.c_void_p * max(count, 1))(*[a.ctypes.data for a in res])
        _lib.check(_lib.lib().nls_batch_get_many(self.handle, first, count, pu), "nls_batch_get_many",
                   self.ctx.handle)
        return res

    def layout(self):
        """Packed host layout: (pump offsets, state offsets, pump block bytes, state block bytes);
        instance k's pump / state at those byte offsets of one block each."""
        n = len(self.specs)
        po, so = np.zeros(max(n, 1), np.int64), np.zeros(max(n, 1), np.int64)
        pb, sb = ctypes.c_int64(), ctypes.c_int64()
        _lib.check(_lib.lib().nls_batch_layout(self.handle, _lib.ptr(po), _lib.ptr(so), ctypes.byref(pb),
                                               ctypes.byref(sb)), "nls_batch_layout", self.ctx.handle)
        return po[:n], so[:n], pb.value, sb.value

    def packed_views(self, block: np.ndarray, field: str):
        """Per-instance arrays viewing a packed block (``field`` "pump" or "state"): the shapes,
        dtypes and orders ``set``/``get`` use, sharing the block's memory."""
        po, so, pb, sb = self.layout()
        offs, need, dt = (po, pb, self.rtype) if field == "pump" else (so, sb, self.ctype)
        if block.dtype != np.uint8 or block.ndim != 1 or block.nbytes < need:
            raise ValueError(f"{field} block must be a flat uint8 array of at least {need} bytes")
        out = []
        for s, o in zip(self.specs, offs):
            shape = (s.n, s.n) if s.dim == 2 else (s.n,)
            out.append(np.ndarray(shape, dtype=dt, buffer=block, offset=int(o), order="F" if s.dim == 2 else "C"))
        return out

    def _block(self, block, need, what):
        if (not isinstance(block, np.ndarray) or block.dtype != np.uint8 or block.ndim != 1
                or not block.flags.c_contiguous or block.nbytes < need):
            raise ValueError(f"{what} must be a flat contiguous uint8 array of at least {need} bytes")
        return block

    def set_packed(self, pump_block: np.ndarray, state_block: np.ndarray):
        """Upload every pump and initial state from two packed blocks (``layout``); one wait."""
        _, _, pb, sb = self.layout()
        P = self._block(pump_block, pb, "pump block")
        U = self._block(state_block, sb, "state block")
        _lib.check(_lib.lib().nls_batch_set_packed(self.handle, _lib.ptr(P), _lib.ptr(U)), "nls_batch_set_packed",
                   self.ctx.handle)
        for i, (p, u) in enumerate(zip(self.packed_views(P, "pump"), self.packed_views(U, "state"))):
            self._record(i, p, u)

    def get_packed(self, out: np.ndarray = None) -> np.ndarray:
        """Every current state into one packed block (``layout``; a new one if ``out`` is None)."""
        _, _, _, sb = self.layout()
        out = np.empty(sb, np.uint8) if out is None else self._block(out, sb, "out")
        _lib.check(_lib.lib().nls_batch_get_packed(self.handle, _lib.ptr(out)), "nls_batch_get_packed",
                   self.ctx.handle)
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
