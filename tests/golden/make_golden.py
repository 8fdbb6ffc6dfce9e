"""Regenerate the committed golden fixtures in this directory.

Run from the repository root in a checkout that has the reference source tree available:

    python tests/golden/make_golden.py [--reference PATH_TO_DASKOL_NLS]

Two kinds of fixture are written.

* ``kat_test_nls_f95.json`` -- the two valid known-answer tests of the reference's Fortran unit
  tests, read as text from test/test_nls.f95: the band storage of row (1..5) for n = 7
  (test_make_banded_matrix, :36-76) and the banded matvec of the identity rows
  (test_rgbmv, :151-202).  The stale order-5 Laplacian answer of :102-108 is deliberately not
  extracted (its /24h^2 normalisation is not what nls/nls.f90 computes).
* ``restatement_small.npz`` -- small end-to-end solves and operators produced by
  ``oracle/blas_oracle.py``, the restatement that multiplies through scipy's BLAS ?gbmv like the
  reference does.  The reference itself cannot be compiled or imported here (Fortran, Python 2),
  so these pin the C++ oracle and the GPU path to the BLAS-based restatement.
"""

from __future__ import annotations

import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import blas_oracle  # noqa: E402


def _fortran_array_literals(src: str, name: str):
    """Return the integer lists of every `name = ... (/ ... /)` assignment in src, in order."""
    out = []
    pat = re.compile(r"\b" + name + r"\s*=\s*(?:transpose\()?(?:reshape\()?\(/(.*?)/\)", re.S)
    for m in pat.finditer(src):
        body = m.group(1).replace("&", " ")
        out.append([int(float(t)) for t in re.split(r"[,\s]+", body.strip()) if t])
    return out


def kat_from_reference(ref_root: str) -> dict:
    path = os.path.join(ref_root, "test", "test_nls.f95")
    src = open(path).read()
    # test_make_banded_matrix: row, ans = reshape((/...), shape(ans)) with ans(m=5, n=7)
    start = src.index("subroutine test_make_banded_matrix")
    end = src.index("end subroutine test_make_banded_matrix")
    body = src[start:end]
    row = _fortran_array_literals(body, "row")[0]
    ans = _fortran_array_literals(body, "ans")[0]
    m, n = 5, 7
    band = np.array(ans, dtype=np.int64).reshape((n, m)).T        # column-major fill of (m, n)
    # test_rgbmv: z = transpose(reshape((/...), shape(z))) -> z(i, :) is the i-th listed row
    start = src.index("subroutine test_rgbmv")
    end = src.index("end subroutine test_rgbmv")
    body = src[start:end]
    row2 = _fortran_array_literals(body, "row")[0]
    z = np.array(_fortran_array_literals(body, "z")[0], dtype=np.int64).reshape((7, 7))
    return {
        "source": "test/test_nls.f95:36-76 and :151-202",
        "make_banded_matrix": {"n": n, "m": m, "row": row, "band_fortran_m_by_n": band.tolist()},
        "rgbmv": {"n": 7, "klu": 2, "sign": 1.0, "row": row2,
                  "x": "identity rows x(i, :) = e_i, y initially zero",
                  "z_rows": z.tolist()},
    }


def config0_coeffs():
    """c3 = R/2, c4 = gamma/2, c5 = g, c6 = 2 g_R, c12 = 1, c13 = gamma_R, c14 = R (0-based index k-1)."""
    c = np.zeros(23)
    c[0] = c[1] = 1.0
    c[2], c[3], c[4], c[5] = 0.5, 0.25, 1.0, 4.0
    c[11], c[12], c[13] = 1.0, 1.0, 1.0
    return c


def restatement_fixtures() -> dict:
    rng = np.random.default_rng(20260)
    out = {}
    coeffs = config0_coeffs()
    out["coeffs"] = coeffs
    for order in (3, 5, 7):
        for rt, tag in ((np.float32, "f32"), (np.float64, "f64")):
            out[f"op1d_o{order}_{tag}"] = blas_oracle.make_laplacian(9, order, 0.1, rt)
    # 1-D solves: n = 16, radial grid r = i*dx, Gaussian pump
    n, dx, dt, iters = 16, 0.25, 1.0e-3, 25
    x = np.linspace(0.0, n * dx, n)
    P1 = 4.0 * np.exp(-x ** 2 / 8.0)
    u1 = 0.1 * (rng.standard_normal(n) + 1j * rng.standard_normal(n))
    out["p1d"], out["u1d_0"] = P1, u1
    for order in (3, 5, 7):
        for rt, tag in ((np.float32, "f32"), (np.float64, "f64")):
            out[f"u1d_o{order}_{tag}"] = blas_oracle.solve(dt, dx, order, iters, P1, coeffs, u1, rt)
    # 2-D solves: n = 12 on [-L/2, L/2]^2, ring pump; axis 0 is the contiguous Fortran axis
    n2, dx2, dt2, iters2 = 12, 0.5, 1.0e-3, 10
    g = np.linspace(-n2 * dx2 / 2, n2 * dx2 / 2, n2)
    X, Y = np.meshgrid(g, g)
    rr = np.sqrt(X ** 2 + Y ** 2)
    P2 = 6.0 * (np.exp(-(rr - 2.0) ** 2 / 2.0) + np.exp(-(rr + 2.0) ** 2 / 2.0))
    u2 = 0.1 * (rng.standard_normal((n2, n2)) + 1j * rng.standard_normal((n2, n2)))
    out["p2d"], out["u2d_0"] = P2, u2
    for order in (3, 5):
        for rt, tag in ((np.float32, "f32"), (np.float64, "f64")):
            out[f"u2d_o{order}_{tag}"] = blas_oracle.solve(dt2, dx2, order, iters2, P2, coeffs, u2, rt)
    out["params"] = np.array([n, dx, dt, iters, n2, dx2, dt2, iters2])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("NLS_REFERENCE_ROOT"), required="NLS_REFERENCE_ROOT" not in os.environ,
                    help="checkout of daskol/nls whose test/test_nls.f95 holds the known-answer tests "
                         "(or set NLS_REFERENCE_ROOT)")
    args = ap.parse_args()
    kat = kat_from_reference(args.reference)
    with open(os.path.join(HERE, "kat_test_nls_f95.json"), "w") as f:
        json.dump(kat, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "restatement_small.npz"), **restatement_fixtures())
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
