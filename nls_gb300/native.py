"""Drop-in for the reference's f2py module: ``from nls_gb300.native import nls``.

The reference builds ``nls.native`` from nls/nls.f90 with f2py (setup.py:69-79) and its Python
layer calls the Fortran module object ``nls`` (nls/solver.py:9, 65-69, 79-83).  ``nls`` here has
the same routine names, positional argument order, optional trailing ``n`` and return values:

    u  = nls.solve_nls(dt, dx, order, iters, pumping, coeffs, u0, [n])      nls/nls.f90:797-813
    u  = nls.solve_nls_1d(...)                                             nls/nls.f90:815-827
    u  = nls.solve_nls_2d(dt, dx, order, iters, pumping, coeffs, u0, [n])   nls/nls.f90:903-919
    mu = nls.chemical_potential_1d(dx, pumping, coeffs, u0, [n])           nls/nls.f90:921-948
    mu = nls.chemical_potential_2d(dx, pumping, coeffs, u0, [n])           nls/nls.f90:950-971
    op = nls.make_laplacian(n, m, h)                                       nls/nls.f90:278-295
    major, minor, patch = nls.version()                                    nls/nls.f90:29-37

Behaviour kept from f2py: inputs are copied (2-D arrays into Fortran order, so the first numpy
axis is the contiguous one, as in the reference), ``n`` defaults to ``len(pumping)`` and must
match it, ``coeffs`` must hold 23 values, a new output array is returned and nothing is kept
between calls; shape errors raise ``ValueError``.  Documented difference: precision follows
``u0``'s dtype -- complex64 (or float32) input runs the complex64 form, anything else runs the
complex128 path, where f2py would silently cast to complex64.  Every call runs on the GPU
through libnls_gb300.so; there is no CPU fallback.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _prep(pumping, coeffs, u0, n, two_d: bool):
    code = _lib.dtype_code(np.asarray(u0).dtype)
    ct, rt = _lib.np_types(code)
    P = np.asarray(pumping)
    U = np.asarray(u0)
    if two_d:
        if P.ndim != 2 or P.shape[0] != P.shape[1]:
            raise ValueError("pumping must be a square (n, n) array")
        if U.shape != P.shape:
            raise ValueError("u0 must have the shape of pumping")
    else:
        if P.ndim != 1:
            raise ValueError("pumping must be a 1-D array")
        if U.shape != P.shape:
            raise ValueError("u0 must have the shape of pumping")
    if n is None:
        n = P.shape[0]
    if int(n) != P.shape[0]:
        raise ValueError(f"n={n} does not match shape(pumping, 0)={P.shape[0]}")
    c = np.ascontiguousarray(coeffs, dtype=np.float64).ravel()
    if c.size != 23:
        raise ValueError("coeffs must have exactly 23 entries")
    if two_d:
        P = np.asfortranarray(P, dtype=rt)
        U = np.asfortranarray(U, dtype=ct)
    else:
        P = np.ascontiguousarray(P, dtype=rt)
        U = np.ascontiguousarray(U, dtype=ct)
    return code, int(n), P, c, U


class _NativeModule:
    """The Fortran module object `nls` of the reference's extension, backed by the GPU."""

    def __init__(self, device: int = 0):
        self.device = device

    def _ctx(self):
        return _lib.default_context(self.device)

    def version(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.lib().nls_version(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)), "version")
        return a.value, b.value, c.value

    def make_laplacian(self, n, m, h):
        """Band storage (m, n) of the radial Laplacian, float64, Fortran order."""
        op = np.zeros((int(m), int(n)), dtype=np.float64, order="F")
        _lib.check(_lib.lib().nls_make_laplacian(int(n), int(m), float(h), _lib.ptr(op)), "make_laplacian")
        return op

    def make_laplacian_2d(self, n, m, h):
        """Block pieces (n, 2m-1) and band orders (m,) of the 2-D cross stencil (orders 3, 5)."""
        blocks = np.zeros((int(n), 2 * int(m) - 1), dtype=np.float64, order="F")
        orders = np.zeros(int(m), dtype=np.int32)
        _lib.check(_lib.lib().nls_make_laplacian_2d(int(n), int(m), float(h), _lib.ptr(blocks), _lib.ptr(orders)),
                   "make_laplacian_2d")
        return blocks, orders

    def _solve(self, dim, dt, dx, order, iters, pumping, coeffs, u0, n):
        code, n, P, c, U = _prep(pumping, coeffs, u0, n, dim == 2)
        out = np.empty_like(U, order="F" if dim == 2 else "C")
        ctx = self._ctx()
        fn = _lib.lib().nls_solve_1d if dim == 1 else _lib.lib().nls_solve_2d
        st = fn(ctx.handle, code, float(dt), float(dx), n, int(order), int(iters), _lib.ptr(c), _lib.ptr(P),
                _lib.ptr(U), _lib.ptr(out))
        _lib.check(st, "solve_nls" if dim == 1 else "solve_nls_2d", ctx.handle)
        return out

    def solve_nls(self, dt, dx, order, iters, pumping, coeffs, u0, n=None):
        return self._solve(1, dt, dx, order, iters, pumping, coeffs, u0, n)

    def solve_nls_1d(self, dt, dx, order, iters, pumping, coeffs, u0, n=None):
        return self._solve(1, dt, dx, order, iters, pumping, coeffs, u0, n)

    def solve_nls_2d(self, dt, dx, order, iters, pumping, coeffs, u0, n=None):
        return self._solve(2, dt, dx, order, iters, pumping, coeffs, u0, n)

    def chemical_potential_1d(self, dx, pumping, coeffs, u0, n=None):
        code, n, P, c, U = _prep(pumping, coeffs, u0, n, False)
        re, im = ctypes.c_double(), ctypes.c_double()
        ctx = self._ctx()
        st = _lib.lib().nls_chemical_potential_1d(ctx.handle, code, float(dx), n, _lib.ptr(c), _lib.ptr(P),
                                                  _lib.ptr(U), ctypes.byref(re), ctypes.byref(im))
        _lib.check(st, "chemical_potential_1d", ctx.handle)
        return complex(re.value, im.value)

    def chemical_potential_2d(self, dx, pumping, coeffs, u0, n=None):
        code, n, P, c, U = _prep(pumping, coeffs, u0, n, True)
        mu = ctypes.c_double()
        ctx = self._ctx()
        st = _lib.lib().nls_chemical_potential_2d(ctx.handle, code, float(dx), n, _lib.ptr(c), _lib.ptr(P),
                                                  _lib.ptr(U), ctypes.byref(mu))
        _lib.check(st, "chemical_potential_2d", ctx.handle)
        return mu.value


nls = _NativeModule()

__all__ = ["nls"]
