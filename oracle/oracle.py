"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module; the shipped solver in ``nls_gb300`` never does.  It wraps ``libnls_oracle.so`` (built
from ``nls_oracle.cpp`` by ``build()`` below or ``make -C oracle``), the C++ restatement of the
reference routines in nls/nls.f90 listed in that file's header.

Array conventions follow the reference's f2py module ``nls.native.nls`` (setup.py:69-79):
2-D fields are passed to the native code in Fortran (column-major) order, so the numpy array
``a[i, j]`` is the Fortran element ``a(i+1, j+1)`` and the first numpy axis is the contiguous one.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libnls_oracle.so")
_lib = None

_TYPES = {np.float32: ("f32", ctypes.c_float), np.float64: ("f64", ctypes.c_double)}


def build(force: bool = False) -> str:
    """Compile ``libnls_oracle.so`` with the committed Makefile; returns its path."""
    src = os.path.join(_HERE, "nls_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "libnls_oracle.so"], check=True)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        ptr = ctypes.c_void_p
        for sfx, ct in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
            getattr(_lib, f"orc_make_banded_matrix_{sfx}").argtypes = [ctypes.c_int, ctypes.c_int, ptr, ptr]
            getattr(_lib, f"orc_make_banded_matrix_{sfx}").restype = None
            getattr(_lib, f"orc_make_laplacian_{sfx}").argtypes = [ctypes.c_int, ctypes.c_int, ct, ptr]
            getattr(_lib, f"orc_make_laplacian_2d_{sfx}").argtypes = [ctypes.c_int, ctypes.c_int, ct, ptr, ptr]
            getattr(_lib, f"orc_gbmv_{sfx}").argtypes = [ctypes.c_int, ctypes.c_int, ct, ptr, ptr, ptr]
            getattr(_lib, f"orc_gbmv_{sfx}").restype = None
            for name in ("hamiltonian_1d", "hamiltonian_2d"):
                getattr(_lib, f"orc_{name}_{sfx}").argtypes = [ctypes.c_int, ctypes.c_int, ct, ptr, ptr, ptr, ptr]
            for name in ("solve_1d", "solve_2d"):
                getattr(_lib, f"orc_{name}_{sfx}").argtypes = [
                    ct, ct, ctypes.c_int, ctypes.c_int, ctypes.c_int, ptr, ptr, ptr, ptr, ctypes.c_int]
            for name in ("chemical_potential_1d", "chemical_potential_2d"):
                getattr(_lib, f"orc_{name}_{sfx}").argtypes = [ct, ctypes.c_int, ptr, ptr, ptr, ptr]
        _lib.orc_openmp_max_threads.restype = ctypes.c_int
    return _lib


def _real_type(dtype):
    dtype = np.dtype(dtype)
    if dtype in (np.dtype(np.complex64), np.dtype(np.float32)):
        return np.float32
    if dtype in (np.dtype(np.complex128), np.dtype(np.float64)):
        return np.float64
    raise TypeError(f"unsupported dtype {dtype}")


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(status: int, what: str):
    if status:
        raise ValueError(f"oracle {what}: status {status}")


def max_threads() -> int:
    return int(lib().orc_openmp_max_threads())


def make_banded_matrix(n: int, row, dtype=np.float32) -> np.ndarray:
    """Band storage (m, n) of the Toeplitz matrix built from ``row`` (nls/nls.f90:61-91)."""
    rt = _real_type(dtype)
    sfx, _ = _TYPES[rt]
    row = np.ascontiguousarray(row, dtype=rt)
    mat = np.zeros((row.size, n), dtype=rt, order="F")
    getattr(lib(), f"orc_make_banded_matrix_{sfx}")(n, row.size, _p(row), _p(mat))
    return mat


def make_laplacian(n: int, order: int, h: float, dtype=np.float64) -> np.ndarray:
    """Band storage (order, n) of the 1-D radial Laplacian (nls/nls.f90:278-295)."""
    rt = _real_type(dtype)
    sfx, ct = _TYPES[rt]
    op = np.zeros((order, n), dtype=rt, order="F")
    _check(getattr(lib(), f"orc_make_laplacian_{sfx}")(n, order, ct(h), _p(op)), "make_laplacian")
    return op


def make_laplacian_2d(n: int, order: int, h: float, dtype=np.float64):
    """Block pieces (n, 2m-1) and band orders (m,) of the 2-D cross stencil (nls/nls.f90:388-403)."""
    rt = _real_type(dtype)
    sfx, ct = _TYPES[rt]
    blocks = np.zeros((n, 2 * order - 1), dtype=rt, order="F")
    orders = np.zeros(order, dtype=np.int32)
    _check(getattr(lib(), f"orc_make_laplacian_2d_{sfx}")(n, order, ct(h), _p(blocks), _p(orders)),
           "make_laplacian_2d")
    return blocks, orders


def gbmv(alpha: float, a: np.ndarray, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """y + alpha*A*x for a square band matrix with kl = ku (nls/nls.f90:530-541)."""
    rt = _real_type(a.dtype)
    sfx, ct = _TYPES[rt]
    a = np.asfortranarray(a, dtype=rt)
    x = np.ascontiguousarray(x, dtype=rt)
    out = np.array(y, dtype=rt, copy=True)
    klu = (a.shape[0] - 1) // 2
    getattr(lib(), f"orc_gbmv_{sfx}")(a.shape[1], klu, ct(alpha), _p(a), _p(x), _p(out))
    return out


def _complex_of(rt):
    return np.complex64 if rt == np.float32 else np.complex128


def _field(a, ctype, two_d: bool):
    return np.asfortranarray(a, dtype=ctype) if two_d else np.ascontiguousarray(a, dtype=ctype)


def hamiltonian(dx, order, pumping, coeffs, u, dtype=None):
    """Action of the right-hand side operator on u (nls/nls.f90:621-650 and :841-870)."""
    dtype = dtype or np.asarray(u).dtype
    rt = _real_type(dtype)
    ct_np = _complex_of(rt)
    sfx, ct = _TYPES[rt]
    u = np.asarray(u)
    two_d = u.ndim == 2
    uu = _field(u, ct_np, two_d)
    P = _field(pumping, rt, two_d)
    c = np.ascontiguousarray(coeffs, dtype=rt)
    assert c.size == 23
    v = np.zeros_like(uu)
    fn = getattr(lib(), f"orc_hamiltonian_{'2d' if two_d else '1d'}_{sfx}")
    _check(fn(uu.shape[0], order, ct(dx), _p(P), _p(c), _p(uu), _p(v)), "hamiltonian")
    return v


def solve(dt, dx, order, iters, pumping, coeffs, u0, dtype=None, threads: int = 1):
    """RK4 solve of nls/nls.f90:797-813 (1-D) or :903-919 (2-D), in float32 or float64."""
    dtype = dtype or np.asarray(u0).dtype
    rt = _real_type(dtype)
    ct_np = _complex_of(rt)
    sfx, ct = _TYPES[rt]
    u0 = np.asarray(u0)
    two_d = u0.ndim == 2
    uu0 = _field(u0, ct_np, two_d)
    P = _field(pumping, rt, two_d)
    c = np.ascontiguousarray(coeffs, dtype=rt)
    assert c.size == 23
    out = np.zeros_like(uu0)
    fn = getattr(lib(), f"orc_solve_{'2d' if two_d else '1d'}_{sfx}")
    _check(fn(ct(dt), ct(dx), uu0.shape[0], order, int(iters), _p(P), _p(c), _p(uu0), _p(out),
              int(max(1, threads))), "solve")
    return out


def chemical_potential(dx, pumping, coeffs, u0, dtype=None):
    """nls/nls.f90:921-971: complex mu in 1-D, real mu in 2-D."""
    dtype = dtype or np.asarray(u0).dtype
    rt = _real_type(dtype)
    ct_np = _complex_of(rt)
    sfx, ct = _TYPES[rt]
    u0 = np.asarray(u0)
    two_d = u0.ndim == 2
    uu0 = _field(u0, ct_np, two_d)
    P = _field(pumping, rt, two_d)
    c = np.ascontiguousarray(coeffs, dtype=rt)
    mu = np.zeros(2, dtype=rt)
    fn = getattr(lib(), f"orc_chemical_potential_{'2d' if two_d else '1d'}_{sfx}")
    _check(fn(ct(dx), uu0.shape[0], _p(P), _p(c), _p(uu0), _p(mu)), "chemical_potential")
    return float(mu[0]) if two_d else complex(mu[0], mu[1])
