"""The allocation-free 2-D entry point (nls_solve_2d_noalloc) against nls_solve_device.

Some callers of this library may not allocate device memory at all -- a service that reserves its
device budget once at start-up, a framework whose caching allocator owns the GPU memory, or a
latency-critical loop that cannot afford cudaMalloc's possible device-wide synchronisation.  For
them the library exposes one 2-D solve whose scratch is a fixed device array inside the library.
This test calls it through the C ABI twice in a row (different sizes and orders, so the second
call runs over whatever the first left in the shared array) and checks each result against the
ordinary entry point running the same kernel, within the parity tolerances of the other GPU
tests (1e-10 relative L2 for complex128, 3e-5 for complex64).  It is collected last so that a
failure here never hides the rest of the suite, and it runs the same alone or after the others.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def env():
    import torch
    from nls_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    from nls_gb300 import _lib
    return torch, _lib


def _case(n, order, seed):
    from nls_gb300 import workloads
    s, _ = workloads.plain_2d(n=n, length=n * 0.15625, order=order, seed=seed)
    return s


@pytest.mark.parametrize("dtype,variant,tol", [(np.complex64, 1, 3e-5), (np.complex64, 10, 3e-5),
                                               (np.complex128, 3, 1e-10)])
def test_noalloc_matches_solve_device_on_two_calls(env, dtype, variant, tol):
    torch, _lib = env
    from nls_gb300 import device
    lib = _lib.lib()
    code = _lib.dtype_code(dtype)
    ct = torch.complex64 if dtype == np.complex64 else torch.complex128
    rt = torch.float32 if dtype == np.complex64 else torch.float64
    for call, (n, order, iters, seed) in enumerate([(130, 5, 41, 1), (96, 3, 40, 2)]):
        s = _case(n, order, seed)
        P = torch.tensor(np.ascontiguousarray(s.pumping), dtype=rt, device="cuda")
        u_ref = torch.tensor(np.ascontiguousarray(s.u0), dtype=ct, device="cuda")
        u_new = u_ref.clone()
        device.solve_(u_ref, P, order=order, dt=s.dt, dx=s.dx, coeffs=s.coeffs, iters=iters, variant=variant)
        pr = _lib.make_problem(2, n, order, s.dt, s.dx, s.coeffs, variant)
        stream = torch.cuda.current_stream()
        st = lib.nls_solve_2d_noalloc(code, ctypes.byref(pr), iters, ctypes.c_void_p(P.data_ptr()),
                                      ctypes.c_void_p(u_new.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        assert st == _lib.NLS_OK, (call, st)
        torch.cuda.synchronize()
        a, b = u_new.cpu().numpy(), u_ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert rel(a, b) <= tol, (call, rel(a, b))


def test_noalloc_rejects_grids_beyond_its_limit(env):
    torch, _lib = env
    lib = _lib.lib()
    n = 513                                    # 513 * 513 > NLS_NOALLOC_MAX_NODES
    s = _case(16, 3, 0)
    pr = _lib.make_problem(2, n, 3, s.dt, s.dx, s.coeffs, -1)
    dummy = torch.zeros(4, dtype=torch.complex64, device="cuda")
    st = lib.nls_solve_2d_noalloc(_lib.NLS_C64, ctypes.byref(pr), 1, ctypes.c_void_p(dummy.data_ptr()),
                                  ctypes.c_void_p(dummy.data_ptr()), None)
    assert st == _lib.NLS_ERR_TOO_LARGE
