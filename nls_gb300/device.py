"""Device-resident solves on torch CUDA tensors (resume without re-upload).

The reference resumes a run by ``model.setInitialSolution(prev)`` followed by ``solve(k)``
(nls/animation.py:65-66, tools/check.py:35-36), which re-sends the state through f2py each time.
Here the state stays on the GPU: ``solve_(u, P, ...)`` advances the complex tensor ``u`` in place.
Work runs on the library context's stream; the calls order themselves after torch's current
stream and make it wait for the result, so ordinary torch code can use ``u`` right after.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib


def _ext_stream(ctx: _lib.Context) -> torch.cuda.ExternalStream:
    s = getattr(ctx, "_torch_stream", None)
    if s is None:
        s = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", ctx.device))
        ctx._torch_stream = s
    return s


def context(device: int = 0) -> _lib.Context:
    return _lib.default_context(device)


def stream(device: int = 0) -> torch.cuda.ExternalStream:
    """The torch view of the stream every kernel of this library is launched on."""
    return _ext_stream(context(device))


def _code_of(u: torch.Tensor) -> int:
    if u.dtype == torch.complex128:
        return _lib.NLS_C128
    if u.dtype == torch.complex64:
        return _lib.NLS_C64
    raise TypeError("state must be complex64 or complex128")


def solve_(u: torch.Tensor, P: torch.Tensor, *, order: int, dt: float, dx: float, coeffs, iters: int,
           variant: int = -1) -> torch.Tensor:
    """Advance u (shape (n,) for the radial model or (n, n) for the 2-D model) by iters RK4 steps.

    For 2-D, memory order follows the reference's Fortran arrays: the last torch dimension is
    the contiguous one and plays the role of the Fortran first index (the cross stencils are
    symmetric, so this only fixes the order of floating-point operations)."""
    if not u.is_cuda or not P.is_cuda:
        raise ValueError("u and P must be CUDA tensors")
    if not u.is_contiguous() or not P.is_contiguous():
        raise ValueError("u and P must be contiguous")
    code = _code_of(u)
    want_p = torch.float64 if code == _lib.NLS_C128 else torch.float32
    if P.dtype != want_p or P.shape != u.shape:
        raise ValueError(f"P must be {want_p} with the shape of u")
    dim = u.dim()
    if dim not in (1, 2) or (dim == 2 and u.shape[0] != u.shape[1]):
        raise ValueError("u must be (n,) or (n, n)")
    ctx = context(u.device.index or 0)
    pr = _lib.make_problem(dim, u.shape[0], order, dt, dx, coeffs, variant)
    ext = _ext_stream(ctx)
    ext.wait_stream(torch.cuda.current_stream(u.device))
    st = _lib.lib().nls_solve_device(ctx.handle, code, ctypes.byref(pr), int(iters),
                                     ctypes.c_void_p(P.data_ptr()), ctypes.c_void_p(u.data_ptr()))
    _lib.check(st, "nls_solve_device", ctx.handle)
    torch.cuda.current_stream(u.device).wait_stream(ext)
    u.record_stream(ext)
    P.record_stream(ext)
    return u


def norm(u: torch.Tensor) -> float:
    """FP64 sum of |u|^2 over all nodes; raises if any component is non-finite."""
    ctx = context(u.device.index or 0)
    ext = _ext_stream(ctx)
    ext.wait_stream(torch.cuda.current_stream(u.device))
    s = ctypes.c_double()
    bad = ctypes.c_int64()
    st = _lib.lib().nls_norm_device(ctx.handle, _code_of(u), u.numel(), ctypes.c_void_p(u.data_ptr()),
                                    ctypes.byref(s), ctypes.byref(bad))
    _lib.check(st, "nls_norm_device", ctx.handle)
    return s.value


def chemical_potential(u: torch.Tensor, P: torch.Tensor, *, dx: float, coeffs) -> complex:
    """FP64 chemical potential mu = i<u, H u>/<u, u> of a device state (order-5 operator, radial
    weight in 1-D), as chemical_potential_1d/2d of the reference (nls/nls.f90:921-971)."""
    ctx = context(u.device.index or 0)
    ext = _ext_stream(ctx)
    ext.wait_stream(torch.cuda.current_stream(u.device))
    pr = _lib.make_problem(u.dim(), u.shape[0], 5, 0.0, dx, coeffs)
    re, im = ctypes.c_double(), ctypes.c_double()
    st = _lib.lib().nls_chemical_potential_device(ctx.handle, _code_of(u), ctypes.byref(pr),
                                                  ctypes.c_void_p(P.data_ptr()), ctypes.c_void_p(u.data_ptr()),
                                                  ctypes.byref(re), ctypes.byref(im))
    _lib.check(st, "nls_chemical_potential_device", ctx.handle)
    return complex(re.value, im.value)


def damping_integral(u: torch.Tensor, P: torch.Tensor, *, dx: float, coeffs) -> float:
    """FP64 damping integral of a device state, as Solution.getDampingIntegral (nls/model.py:350-365):
    rectangle rule of (n - 1)|u|^2 with n = c12 P / (c13 + c14 |u|^2), radial weight 2 pi r dx on
    linspace(0, n dx, n) in 1-D, dx^2 in 2-D."""
    ctx = context(u.device.index or 0)
    ext = _ext_stream(ctx)
    ext.wait_stream(torch.cuda.current_stream(u.device))
    pr = _lib.make_problem(u.dim(), u.shape[0], 5, 0.0, dx, coeffs)
    out = ctypes.c_double()
    st = _lib.lib().nls_damping_integral_device(ctx.handle, _code_of(u), ctypes.byref(pr),
                                                ctypes.c_void_p(P.data_ptr()), ctypes.c_void_p(u.data_ptr()),
                                                ctypes.byref(out))
    _lib.check(st, "nls_damping_integral_device", ctx.handle)
    return out.value


def density_errors(u: torch.Tensor, u_ref: torch.Tensor, P64: torch.Tensor, coeffs):
    """Relative L2 errors of |u|^2 and of the reservoir n against a complex128 reference."""
    if u_ref.dtype != torch.complex128 or P64.dtype != torch.float64:
        raise ValueError("reference must be complex128 with a float64 pump")
    c = np.asarray(coeffs, dtype=np.float64)
    ctx = context(u.device.index or 0)
    ext = _ext_stream(ctx)
    ext.wait_stream(torch.cuda.current_stream(u.device))
    d, r = ctypes.c_double(), ctypes.c_double()
    st = _lib.lib().nls_density_error_device(ctx.handle, _code_of(u), u.numel(), ctypes.c_void_p(u.data_ptr()),
                                             ctypes.c_void_p(u_ref.data_ptr()), ctypes.c_void_p(P64.data_ptr()),
                                             float(c[11]), float(c[12]), float(c[13]), ctypes.byref(d),
                                             ctypes.byref(r))
    _lib.check(st, "nls_density_error_device", ctx.handle)
    return d.value, r.value


def launches(device: int = 0) -> int:
    """Kernel launches issued so far by this process's context on the device."""
    return context(device).launches


def companion_errors(state, spec, steps: int, device: int = 0):
    """Relative L2 errors of |psi|^2 and of the reservoir n of a result against a complex128
    companion solve of the same problem (the plain path, pinned to the FP64 oracle) from the
    spec's pump and initial state over the same number of steps, reduced in FP64 on the device.

    ``state`` is the result as a host array (the spec's shape; Fortran order in 2-D, as the batch
    and pool return it) or a raw device pointer to a complex64 result in that memory order."""
    dev = torch.device("cuda", device)
    shape = (spec.n, spec.n) if spec.dim == 2 else (spec.n,)
    order = "F" if spec.dim == 2 else "C"
    u64 = torch.tensor(np.ravel(np.asarray(spec.u0, dtype=np.complex128), order=order).copy(),
                       device=dev).reshape(shape)
    P64 = torch.tensor(np.ravel(np.asarray(spec.pumping, dtype=np.float64), order=order).copy(),
                       device=dev).reshape(shape)
    solve_(u64, P64, order=spec.order, dt=spec.dt, dx=spec.dx, coeffs=spec.coeffs, iters=int(steps))
    if isinstance(state, np.ndarray):
        code = _lib.dtype_code(state.dtype)
        ct = torch.complex64 if code == _lib.NLS_C64 else torch.complex128
        t = torch.tensor(np.ravel(state, order=order).copy(), dtype=ct, device=dev)
        ptr = t.data_ptr()
    else:
        code, t, ptr = _lib.NLS_C64, None, int(state)
    c = np.asarray(spec.coeffs, dtype=np.float64)
    ctx = context(device)
    ext = _ext_stream(ctx)
    ext.wait_stream(torch.cuda.current_stream(dev))
    d, r = ctypes.c_double(), ctypes.c_double()
    st = _lib.lib().nls_density_error_device(ctx.handle, code, spec.nodes, ctypes.c_void_p(ptr),
                                             ctypes.c_void_p(u64.data_ptr()), ctypes.c_void_p(P64.data_ptr()),
                                             float(c[11]), float(c[12]), float(c[13]), ctypes.byref(d),
                                             ctypes.byref(r))
    _lib.check(st, "nls_density_error_device", ctx.handle)
    return d.value, r.value
