"""ctypes binding of libnls_gb300.so (the C ABI declared in include/nls_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is present, every solver
entry point raises.  Host-only helpers (operator construction, version) work without a GPU.
"""

from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libnls_gb300.so")

NLS_OK = 0
NLS_ERR_INVALID = 1
NLS_ERR_ORDER = 2
NLS_ERR_CUDA = 3
NLS_ERR_NONFINITE = 4
NLS_ERR_TIMEOUT = 5
NLS_ERR_NOMEM = 6
NLS_ERR_BUSY = 7
NLS_ERR_NOT_READY = 8
NLS_ERR_TOO_LARGE = 9
NLS_NOALLOC_MAX_NODES = 262144

NLS_C128 = 0
NLS_C64 = 1

_STATUS_NAMES = {
    NLS_ERR_INVALID: "invalid argument",
    NLS_ERR_ORDER: "unsupported order",
    NLS_ERR_CUDA: "CUDA error",
    NLS_ERR_NONFINITE: "non-finite result",
    NLS_ERR_TIMEOUT: "timeout",
    NLS_ERR_NOMEM: "out of device memory",
    NLS_ERR_BUSY: "busy",
    NLS_ERR_NOT_READY: "not ready",
    NLS_ERR_TOO_LARGE: "grid too large for the allocation-free entry point",
}

# Every symbol include/nls_gb300.h declares, with (restype, argtypes).
_p, _i, _d, _i64, _sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64, ctypes.c_size_t
_pi, _pd, _pi64, _psz = (ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                         ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_size_t))


class Problem(ctypes.Structure):
    """Mirror of `nls_problem`."""
    _fields_ = [("dim", ctypes.c_int), ("n", ctypes.c_int), ("order", ctypes.c_int),
                ("variant", ctypes.c_int), ("dt", ctypes.c_double), ("dx", ctypes.c_double),
                ("coeffs", ctypes.c_double * 23)]


_pp = ctypes.POINTER(Problem)

SIGNATURES = {
    "nls_version": (_i, [_pi, _pi, _pi]),
    "nls_make_laplacian": (_i, [_i, _i, _d, _p]),
    "nls_make_laplacian_2d": (_i, [_i, _i, _d, _p, _p]),
    "nls_ctx_create": (_i, [_i, ctypes.POINTER(_p)]),
    "nls_ctx_destroy": (_i, [_p]),
    "nls_ctx_stream": (_i, [_p, ctypes.POINTER(_p)]),
    "nls_ctx_synchronize": (_i, [_p]),
    "nls_last_error": (ctypes.c_char_p, [_p]),
    "nls_ctx_launch_count": (_i64, [_p]),
    "nls_solve_1d": (_i, [_p, _i, _d, _d, _i, _i, _i, _p, _p, _p, _p]),
    "nls_solve_2d": (_i, [_p, _i, _d, _d, _i, _i, _i, _p, _p, _p, _p]),
    "nls_solve_device": (_i, [_p, _i, _pp, _i64, _p, _p]),
    "nls_chemical_potential_1d": (_i, [_p, _i, _d, _i, _p, _p, _p, _pd, _pd]),
    "nls_chemical_potential_2d": (_i, [_p, _i, _d, _i, _p, _p, _p, _pd]),
    "nls_chemical_potential_device": (_i, [_p, _i, _pp, _p, _p, _pd, _pd]),
    "nls_norm_device": (_i, [_p, _i, _i64, _p, _pd, _pi64]),
    "nls_damping_integral_device": (_i, [_p, _i, _pp, _p, _p, _pd]),
    "nls_density_error_device": (_i, [_p, _i, _i64, _p, _p, _p, _d, _d, _d, _pd, _pd]),
    "nls_batch_create": (_i, [_p, _i, _i, _pp, ctypes.POINTER(_p)]),
    "nls_batch_set": (_i, [_p, _i, _p, _p]),
    "nls_batch_run": (_i, [_p, _i64]),
    "nls_batch_get": (_i, [_p, _i, _p]),
    "nls_batch_set_many": (_i, [_p, _i, _i, _p, _p]),
    "nls_batch_get_many": (_i, [_p, _i, _i, _p]),
    "nls_batch_layout": (_i, [_p, _p, _p, _p, _p]),
    "nls_batch_set_packed": (_i, [_p, _p, _p]),
    "nls_batch_get_packed": (_i, [_p, _p]),
    "nls_batch_state": (_i, [_p, _i, ctypes.POINTER(_p), ctypes.POINTER(_p)]),
    "nls_batch_info": (_i, [_p, _i64, _pi64, _pi64]),
    "nls_batch_destroy": (_i, [_p]),
    "nls_pool_create": (_i, [_p, _i, _sz, _i, _i, ctypes.POINTER(_p)]),
    "nls_pool_admit": (_i, [_p, _pp, _p, _p, _i64, _i64, _pi]),
    "nls_pool_step": (_i, [_p, _pi]),
    "nls_pool_launch": (_i, [_p, _pi]),
    "nls_pool_wait": (_i, [_p, _pi]),
    "nls_pool_ready": (_i, [_p, _pi]),
    "nls_pool_info": (_i, [_p, _pi, _pd]),
    "nls_pool_take": (_i, [_p, _pi64, _p, _sz]),
    "nls_pool_status": (_i, [_p, _pi, _psz]),
    "nls_pool_destroy": (_i, [_p]),
    "nls_solve_2d_noalloc": (_i, [_i, _pp, _i64, _p, _p, _p]),
    "nls_test_set_tile_tx_extra": (_i, [_i, ctypes.c_uint]),
    "nls_test_set_stream_dep_extra": (_i, [_i, ctypes.c_uint]),
    "nls_test_set_stream_steps_per_launch": (_i, [_i]),
}

_lib = None
_lock = threading.Lock()


class NativeError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: {_STATUS_NAMES.get(status, 'status %d' % status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


def lib() -> ctypes.CDLL:
    """Load libnls_gb300.so (built by nls_gb300.build); raises if it is absent."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: run `python -m nls_gb300.build` "
                                   "(the solver has no CPU fallback)")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(status: int, where: str, ctx=None):
    if status != NLS_OK:
        detail = ""
        if ctx is not None:
            raw = lib().nls_last_error(ctx)
            detail = raw.decode() if raw else ""
        if status == NLS_ERR_INVALID or status == NLS_ERR_ORDER:
            raise ValueError(NativeError(status, where, detail))
        raise NativeError(status, where, detail)


class Context:
    """An nls_ctx on one CUDA device (its own non-blocking stream)."""

    def __init__(self, device: int = 0):
        self.device = device
        h = ctypes.c_void_p()
        st = lib().nls_ctx_create(device, ctypes.byref(h))
        if st != NLS_OK:
            raise NativeError(st, "nls_ctx_create", "no usable CUDA device")
        self.handle = h

    def close(self):
        if self.handle:
            lib().nls_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        check(lib().nls_ctx_stream(self.handle, ctypes.byref(s)), "nls_ctx_stream", self.handle)
        return s.value or 0

    def synchronize(self):
        check(lib().nls_ctx_synchronize(self.handle), "nls_ctx_synchronize", self.handle)

    @property
    def launches(self) -> int:
        return int(lib().nls_ctx_launch_count(self.handle))


_default = {}


def default_context(device: int = 0) -> Context:
    with _lock:
        ctx = _default.get(device)
    if ctx is None:
        ctx = Context(device)
        with _lock:
            _default.setdefault(device, ctx)
            ctx = _default[device]
    return ctx


def dtype_code(dtype) -> int:
    """complex64/float32 -> the single-precision form; everything else -> the complex128 path."""
    dt = np.dtype(dtype)
    return NLS_C64 if dt in (np.dtype(np.complex64), np.dtype(np.float32)) else NLS_C128


def np_types(code: int):
    return (np.complex128, np.float64) if code == NLS_C128 else (np.complex64, np.float32)


def ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def make_problem(dim, n, order, dt, dx, coeffs, variant=-1) -> Problem:
    c = np.asarray(coeffs, dtype=np.float64).ravel()
    if c.size != 23:
        raise ValueError("coeffs must have exactly 23 entries (coeffs(1..23) of the reference)")
    pr = Problem()
    pr.dim, pr.n, pr.order, pr.variant = int(dim), int(n), int(order), int(variant)
    pr.dt, pr.dx = float(dt), float(dx)
    for i in range(23):
        pr.coeffs[i] = float(c[i])
    return pr
