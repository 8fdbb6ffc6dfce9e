"""Second, independent restatement of the reference path on top of scipy's BLAS ?gbmv (TEST INFRASTRUCTURE).

The reference multiplies by its band operators through BLAS ``sgbmv`` (nls/nls.f90:540), an
unpinned third-party routine (``-lblas`` in setup.py:75-77 and nls/makefile:49; MKL in
nls/makefile:47).  scipy 1.18 ships the same routine (``scipy.linalg.blas.sgbmv/dgbmv``, backed by
its bundled OpenBLAS), so this module rebuilds the operators with numpy, following
nls/nls.f90:61-403 statement by statement, and performs every banded product through scipy's
?gbmv exactly as ``rgbmv``/``rbbmv_o3``/``rbbmv_o5`` call it (nls/nls.f90:408-541).  It is slow
(one BLAS call per block column in 2-D, as in the reference) and meant for small grids: it pins
the C++ oracle in ``nls_oracle.cpp`` and produces the committed golden fixtures.
"""

from __future__ import annotations

import numpy as np
from scipy.linalg import blas


def _gbmv(rt):
    return blas.sgbmv if rt == np.float32 else blas.dgbmv


def make_banded_matrix(n, row, rt=np.float32):
    """nls/nls.f90:61-91: mat(k+1+i-j, j) = A(i, j) for A(i, i+d) = row(k+1-d)."""
    row = np.asarray(row, dtype=rt)
    m = row.size
    k = (m - 1) // 2
    mat = np.zeros((m, n), dtype=rt, order="F")
    for j in range(1, k + 1):                       # left triangle (1-based j)
        mat[k + 1 - j:, j - 1] = row[k + 1 - j:]
    for j in range(k + 1, n - k + 1):               # body
        mat[:, j - 1] = row
    for j in range(1, k + 1):                       # right triangle
        col = n - k + j
        mat[: m - j, col - 1] = row[: m - j]
        mat[m - j:, col - 1] = 0
    return mat


def _finish_radial(L1, L2, h, rt):
    m, n = L1.shape
    for i in range(1, (m + 1) // 2 + 1):            # clear_first_row_of_derivative
        L1[i - 1, (m + 1) // 2 - i] = 0
    for i in range(1, m + 1):                       # divide_derivative_on_radius
        for j in range(1, n + 1):
            row = i + j - (m + 3) // 2
            if row > 0:
                L1[i - 1, j - 1] = L1[i - 1, j - 1] / (rt(row) * h)
    return (L1 + L2).astype(rt)


def make_laplacian(n, order, h, rt=np.float32):
    """nls/nls.f90:132-295 (orders 3, 5, 7)."""
    h = rt(h)
    if order == 3:
        dx1, dx2 = rt(2) * h, rt(1) * (h * h)
        r1, r2 = [1, 0, -1], [1, -2, 1]
    elif order == 5:
        dx1, dx2 = rt(12) * h, rt(12) * (h * h)
        r1, r2 = [-1, 8, 0, -8, 1], [-1, 16, -30, 16, -1]
    elif order == 7:
        dx1, dx2 = rt(60) * h, rt(180) * (h * h)
        r1, r2 = [1, -9, 45, 0, -45, 9, -1], [2, -27, 270, -490, 270, -27, 2]
    else:
        raise ValueError("order must be 3, 5 or 7")
    L1 = make_banded_matrix(n, np.array(r1, dtype=rt) / dx1, rt)
    L2 = make_banded_matrix(n, np.array(r2, dtype=rt) / dx2, rt)
    # Fortran (band_row, column), 1-based -> numpy [band_row-1, column-1]
    if order == 3:
        L2[1, 0] = rt(2) * L2[1, 0]
        L2[0, 1] = rt(4) * L2[0, 1]
    elif order == 5:
        L1[2, 1] = L1[2, 1] + rt(1) / dx1
        L2[2, 1] = L2[2, 1] - rt(1) / dx2
        L2[2, 0] = rt(2) * L2[2, 0]
        L2[1, 1] = rt(4) * L2[1, 1]
        L2[0, 2] = rt(4) * L2[0, 2]
    else:
        L1[3, 1] = L1[3, 1] + rt(9) / dx1
        L1[2, 2] = L1[2, 2] - rt(1) / dx1
        L1[4, 1] = L1[4, 1] - rt(1) / dx1
        L2[3, 0] = rt(2) * L2[3, 0]
        L2[2, 1] = rt(4) * L2[2, 1]
        L2[1, 2] = rt(4) * L2[1, 2]
        L2[0, 3] = rt(4) * L2[0, 3]
        L2[3, 1] = L2[3, 1] - rt(27) / dx2
        L2[2, 2] = L2[2, 2] + rt(2) / dx2
        L2[4, 1] = L2[4, 1] + rt(2) / dx2
    return _finish_radial(L1, L2, h, rt)


def make_laplacian_2d(n, order, h, rt=np.float32):
    """nls/nls.f90:297-351: list of (band matrix, klu, column offset) in the reference's call order."""
    h = rt(h)
    if order == 3:
        dx2 = rt(1) * (h * h)
        s = make_banded_matrix(n, [rt(1) / dx2], rt)
        mid = make_banded_matrix(n, np.array([1, -4, 1], dtype=rt) / dx2, rt)
        # rbbmv_o3 (nls/nls.f90:421-431): left block on x col i-1, middle on col i, right on i+1
        return [(s, 0, -1), (mid, 1, 0), (s.copy(), 0, +1)]
    if order == 5:
        dx2 = rt(12) * (h * h)
        a = make_banded_matrix(n, [rt(-1) / dx2], rt)
        b = make_banded_matrix(n, [rt(16) / dx2], rt)
        mid = make_banded_matrix(n, np.array([-1, 16, -60, 16, -1], dtype=rt) / dx2, rt)
        # rbbmv_o5 (nls/nls.f90:447-465): right2, right1, middle, left1, left2
        return [(a, 0, +2), (b, 0, +1), (mid, 2, 0), (b.copy(), 0, -1), (a.copy(), 0, -2)]
    raise ValueError("2-D order must be 3 or 5")


def _rgbmv(x, y, sign, op, klu, rt):
    n = x.size
    return _gbmv(rt)(n, n, klu, klu, sign, op, x, beta=rt(1), y=y)


def hamiltonian_1d(op, pumping, coeffs, u, rt):
    """nls/nls.f90:621-650 with revervoir :570-581."""
    c = np.asarray(coeffs, dtype=rt)
    ur, ui = u.real.astype(rt), u.imag.astype(rt)
    s = ur * ur + ui * ui
    r = c[11] * pumping / (c[12] + c[13] * s)
    vr = (c[2] * r - c[3]) * ur + (c[4] * s + c[5] * r) * ui
    vi = (c[2] * r - c[3]) * ui - (c[4] * s + c[5] * r) * ur
    klu = (op.shape[0] - 1) // 2
    vr = _rgbmv(ui, vr, rt(-1), op, klu, rt)
    vi = _rgbmv(ur, vi, rt(+1), op, klu, rt)
    return (vr + 1j * vi).astype(np.complex64 if rt == np.float32 else np.complex128)


def hamiltonian_2d(pieces, pumping, coeffs, u, rt):
    """nls/nls.f90:841-870; u and pumping are (n, n) with axis 0 the contiguous Fortran axis."""
    c = np.asarray(coeffs, dtype=rt)
    ur, ui = u.real.astype(rt), u.imag.astype(rt)
    s = ur * ur + ui * ui
    r = c[11] * pumping / (c[12] + c[13] * s)
    vr = (c[2] * r - c[3]) * ur + (c[4] * s + c[5] * r) * ui
    vi = (c[2] * r - c[3]) * ui - (c[4] * s + c[5] * r) * ur
    n = u.shape[0]
    for x, y, sign in ((ui, vr, rt(-1)), (ur, vi, rt(+1))):
        for band, klu, off in pieces:
            for col in range(n):                    # Fortran column col+1 of y
                src = col + off
                if 0 <= src < n:
                    y[:, col] = _rgbmv(np.ascontiguousarray(x[:, src]), np.ascontiguousarray(y[:, col]),
                                       sign, band, klu, rt)
    return (vr + 1j * vi).astype(np.complex64 if rt == np.float32 else np.complex128)


def solve(dt, dx, order, iters, pumping, coeffs, u0, rt=np.float32):
    """RK4 of nls/nls.f90:705-734 / :873-901 in the reference's operation order."""
    ct = np.complex64 if rt == np.float32 else np.complex128
    u = np.array(u0, dtype=ct)
    P = np.asarray(pumping, dtype=rt)
    dt = rt(dt)
    if u.ndim == 1:
        op = make_laplacian(u.size, order, dx, rt)
        H = lambda v: hamiltonian_1d(op, P, coeffs, v, rt)
    else:
        pieces = make_laplacian_2d(u.shape[0], order, dx, rt)
        H = lambda v: hamiltonian_2d(pieces, P, coeffs, v, rt)
    two, six = rt(2), rt(6)

    def axpy(a, k, scale_mul, scale_div):
        re = a.real + (k.real * scale_mul) / scale_div
        im = a.imag + (k.imag * scale_mul) / scale_div
        return (re + 1j * im).astype(ct)

    for _ in range(int(iters)):
        k1 = H(u)
        k2 = H(axpy(u, k1, dt, two))
        k3 = H(axpy(u, k2, dt, two))
        k4 = H(axpy(u, k3, dt, rt(1)))
        sre = ((k1.real + two * k2.real) + two * k3.real) + k4.real
        sim = ((k1.imag + two * k2.imag) + two * k3.imag) + k4.imag
        u = ((u.real + (sre * dt) / six) + 1j * (u.imag + (sim * dt) / six)).astype(ct)
    return u
