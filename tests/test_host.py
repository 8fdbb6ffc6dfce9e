"""CPU tests of the host side: the C-ABI library loads and exports the header's symbols, the
host operator builders match the oracle bit for bit, and the Python API keeps the reference's
conventions.  No kernel is launched here."""

import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from nls_gb300 import build
    build.build()
    from nls_gb300 import _lib
    return _lib.lib()


def header_symbols():
    src = open(os.path.join(ROOT, "include", "nls_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nls_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib):
    names = header_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    from nls_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == names


def test_version(lib):
    from nls_gb300.native import nls
    assert nls.version() == (0, 2, 0)


@pytest.mark.parametrize("order", [3, 5, 7])
@pytest.mark.parametrize("n", [7, 8, 33, 1000])
def test_make_laplacian_matches_oracle_bitwise(lib, oracle_lib, order, n):
    from nls_gb300.native import nls
    for h in (0.04, 0.1, 0.15625):
        a = nls.make_laplacian(n, order, h)
        b = oracle_lib.make_laplacian(n, order, h, np.float64)
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("order", [3, 5])
def test_make_laplacian_2d_matches_oracle_bitwise(lib, oracle_lib, order):
    from nls_gb300.native import nls
    for n in (5, 9, 64):
        a, oa = nls.make_laplacian_2d(n, order, 0.15625)
        b, ob = oracle_lib.make_laplacian_2d(n, order, 0.15625, np.float64)
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(oa, ob)


def test_invalid_order_rejected_on_host(lib):
    from nls_gb300.native import nls
    with pytest.raises(ValueError):
        nls.make_laplacian(10, 4, 0.1)
    with pytest.raises(ValueError):
        nls.make_laplacian_2d(10, 7, 0.1)


def test_context_without_gpu_fails_cleanly(lib):
    """With no CUDA device the context call returns a status instead of crashing."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = lib.nls_ctx_create(0, ctypes.byref(h))
    assert st != 0 and not h.value


def test_solver_refuses_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from nls_gb300 import _lib
    from nls_gb300.native import nls
    _lib._default.clear()
    n = 16
    with pytest.raises(RuntimeError):
        nls.solve_nls(1e-3, 0.1, 5, 1, np.ones(n), np.zeros(23), np.ones(n, complex))


def test_argument_checks_before_any_gpu_work(lib):
    from nls_gb300.native import nls
    with pytest.raises(ValueError):
        nls.solve_nls(1e-3, 0.1, 5, 1, np.ones(16), np.zeros(22), np.ones(16, complex))
    with pytest.raises(ValueError):
        nls.solve_nls(1e-3, 0.1, 5, 1, np.ones(16), np.zeros(23), np.ones(15, complex))
    with pytest.raises(ValueError):
        nls.solve_nls(1e-3, 0.1, 5, 1, np.ones(16), np.zeros(23), np.ones(16, complex), 17)
    with pytest.raises(ValueError):
        nls.solve_nls_2d(1e-3, 0.1, 3, 1, np.ones((4, 5)), np.zeros(23), np.ones((4, 5), complex))


def test_model_defaults_and_coefficients():
    from nls_gb300 import Model1D, Model2D, Problem
    m1 = Problem().model()
    assert isinstance(m1, Model1D)
    assert (m1.dx, m1.dt, m1.order, m1.num_nodes, m1.num_iters) == (0.1, 1e-3, 5, 1000, 100000)
    m2 = Problem().model(model="2d")
    assert isinstance(m2, Model2D)
    assert (m2.order, m2.num_nodes, m2.num_iters) == (3, 40, 1000)
    o = m1.originals
    phi0 = np.sqrt(o["gamma"] / (2 * o["g"]))
    n0 = 2.0 / (o["R"] * phi0)
    c = m1.getCoefficients()
    assert c.size == 23
    np.testing.assert_allclose(c[:5], 1.0)
    np.testing.assert_allclose(c[5], 4 * o["tilde_g"] / o["R"])
    np.testing.assert_allclose(c[11], 1.0 / (n0 * o["gamma_R"]))
    np.testing.assert_allclose(c[12], 1.0)
    np.testing.assert_allclose(c[13], o["R"] * phi0 ** 2 / o["gamma_R"])


def test_pump_grid_convention():
    """The pump grid spacing is n*dx/(n-1) while the Laplacian uses dx (nls/model.py:220-232)."""
    from nls_gb300 import GaussianPumping1D, GaussianRingPumping2D, Problem
    m = Problem().model(num_nodes=11, dx=0.5, pumping=GaussianPumping1D(power=4.0, variation=2.0))
    x = np.linspace(0, 5.5, 11)
    np.testing.assert_allclose(m.getPumping(), 4.0 * np.exp(-x ** 2 / 8.0))
    m2 = Problem().model(model="2d", num_nodes=9, dx=1.0,
                         pumping=GaussianRingPumping2D(power=6.0, radius=2.0, variation=1.0))
    g = np.linspace(-4.5, 4.5, 9)
    X, Y = np.meshgrid(g, g)
    r = np.sqrt(X ** 2 + Y ** 2)
    want = 6.0 * (np.exp(-(r - 2) ** 2 / 2) + np.exp(-(r + 2) ** 2 / 2))
    np.testing.assert_allclose(m2.getPumping(), want)


def test_pumping_algebra_matches_reference_semantics():
    from nls_gb300.pumping import (GaussianElipticPumping2D, GaussianPumping, OpMulPumping,
                                   RectangularRingPumping1D)
    a, b = GaussianPumping(power=2.0), GaussianPumping(power=1.0, x0=1.0)
    x, y = np.linspace(-2, 2, 5), np.zeros(5)
    np.testing.assert_allclose((a + b)(x, y), a(x, y) + b(x, y))
    np.testing.assert_allclose((a - b)(x, y), a(x, y) - b(x, y))
    with pytest.raises(NotImplementedError):
        OpMulPumping(a, b)(x, y)
    rr = RectangularRingPumping1D(power=3.0, radius=2.0, width=1.0)
    np.testing.assert_allclose(rr(np.array([-2.0, 0.0, 2.4, 3.0])), [3.0, 0.0, 3.0, 0.0])
    e = GaussianElipticPumping2D(power=1.0, variation=2.0, a=1.0, b=1.0)
    r = 1.5
    np.testing.assert_allclose(e(np.array([r]), np.array([0.0])),
                               np.exp(-(1 - r) ** 2 / 4.0) + np.exp(-(1 + r) ** 2 / 4.0))


def test_solution_reservoir_density_and_mat_roundtrip(tmp_path):
    from nls_gb300 import GaussianPumping1D, Problem, Solution
    m = Problem().model(num_nodes=16, dx=0.25, pumping=GaussianPumping1D(power=2.0))
    rng = np.random.default_rng(0)
    psi = rng.standard_normal(16) + 1j * rng.standard_normal(16)
    s = Solution(m, psi)
    c = m.coeffs
    np.testing.assert_allclose(s.getDensity(), np.abs(psi) ** 2)
    np.testing.assert_allclose(s.getReservoir(), c[11] * m.getPumping() / (c[12] + c[13] * np.abs(psi) ** 2))
    f = str(tmp_path / "m.mat")
    m.store(f)
    m2 = Problem().model(filename=f)
    assert m2.num_nodes == 16 and m2.order == 5
    np.testing.assert_allclose(m2.coeffs, m.coeffs)
    np.testing.assert_allclose(m2.getPumping(), m.getPumping())
    s.setElapsedTime(1.5)
    f2 = str(tmp_path / "s.mat")
    s.store(f2)
    s2 = Solution(m2).restore(f2)
    np.testing.assert_allclose(s2.getSolution(), psi)
    assert s2.getElapsedTime() == 1.5


def test_autotune_assign_maps_choices_to_other_specs():
    """Choices tuned on one population are applied by size bucket, or by the shared 2-D shape."""
    from nls_gb300 import autotune
    from nls_gb300 import workloads as w
    specs = [w.mix_instance(i, 1, with_data=False) for i in range(4)] + \
            [w.mix_instance(10 + i, 2, with_data=False) for i in range(4)]
    choices = {f"1d/o5/n<={autotune.bucket(s.n)}": 4 for s in specs if s.dim == 1}
    choices["2d/o3/mix"] = 12
    autotune.assign(specs, choices)
    assert all(s.variant == (4 if s.dim == 1 else 12) for s in specs)


def test_autotune_batch_refines_1d_cluster_sizes_on_the_batch(monkeypatch):
    """Batch mode starts the 1-D specs from the per-size choice and keeps, per size bucket, the
    cluster size that times fastest on the whole batch (fake timings, no GPU)."""
    from nls_gb300 import autotune
    from nls_gb300 import workloads as w
    specs = [w.mix_instance(i, 1, with_data=False) for i in range(40)] + \
            [w.mix_instance(100 + i, 2, with_data=False) for i in range(3)]
    assert any(s.n > 4096 for s in specs if s.dim == 1) and any(s.n <= 4096 for s in specs if s.dim == 1)

    def best(n):
        return 1 if n <= 4096 else 4

    def cost(s):
        order = [1, 2, 4, 8, 16] if s.n <= 4096 else [4, 2, 8, 16]
        return 1.0 + order.index(s.variant) if s.variant in order else 100.0

    calls = []
    monkeypatch.setattr(autotune, "tune", lambda dim, n, order, **kw: 16 if dim == 1 else 12)
    monkeypatch.setattr(autotune, "tune_mix", lambda group, **kw: (12, {12: 1.0}))

    def fake_time(trial, dtype, steps, device):
        calls.append(1)
        return 50.0 + sum(cost(t) for t in trial if t.dim == 1)

    monkeypatch.setattr(autotune, "_time_mix_assigned", fake_time)
    out = autotune.apply(specs, dtype=np.complex64, mode="batch")
    for s in specs:
        if s.dim == 1:
            assert s.variant == best(s.n), (s.n, s.variant)
            assert out[f"1d/o{s.order}/n<={autotune.bucket(s.n)}"] == s.variant
        else:
            assert s.variant == 12
    assert calls
    # single mode keeps the per-size choice
    single = [w.mix_instance(i, 1, with_data=False) for i in range(5)]
    autotune.apply(single, dtype=np.complex64, mode="single")
    assert all(s.variant == 16 for s in single)


def test_native_alias_binds_the_gpu_module_object():
    """The documented drop-in alias: with ``sys.modules["nls.native"]`` set to ``nls_gb300.native``,
    the reference's ``from .native import nls`` (nls/solver.py:9) binds the GPU module object."""
    import sys
    import types
    import nls_gb300.native
    saved = {k: sys.modules.get(k) for k in ("nls", "nls.native")}
    try:
        pkg = types.ModuleType("nls")
        pkg.__path__ = []
        sys.modules["nls"] = pkg
        sys.modules["nls.native"] = nls_gb300.native
        from nls.native import nls as bound  # noqa: E402
        assert bound is nls_gb300.native.nls
        assert callable(bound.solve_nls) and callable(bound.solve_nls_2d)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


def test_job_intake_table_and_http_routes():
    """schedulr's job contract in process and over HTTP on 127.0.0.1 (no GPU work)."""
    import json
    import urllib.request
    from nls_gb300.intake import JobQueue, job_model, serve_http
    q = JobQueue()
    ids = q.post_jobs([json.dumps({"power": 2.5}), {"power": 3.0, "num_nodes": 32, "num_iters": 10}])
    assert ids == [1, 2] and q.pending() == 2
    m = job_model(q.job(2).description)
    assert (m.num_nodes, m.num_iters, m.order, m.dx) == (32, 10, 5, 0.2)
    assert np.asarray(m.getInitialSolution()).shape == (32, 32)
    m1 = job_model(q.job(1).description)
    assert (m1.num_nodes, m1.num_iters, m1.dt) == (200, 2000, 2e-3)
    xm = 20.0 / 199                                    # nearest grid point to the pump centre
    np.testing.assert_allclose(m1.getPumping().max(), 2.5 * np.exp(-2 * xm ** 2 / (2 * 25.0)), rtol=1e-12)
    srv = serve_http(q, port=0)
    port = srv.server_address[1]
    try:
        def call(method, path, body=None):
            data = json.dumps(body).encode() if body is not None else None
            req = urllib.request.Request(f"http://127.0.0.1:{port}{path}", data=data, method=method,
                                         headers={"Content-Type": "application/json"})
            with urllib.request.urlopen(req) as r:
                raw = r.read()
                return r.status, (json.loads(raw) if raw else None)
        assert call("POST", "/api/jobs", {"jobs": [json.dumps({"power": 1.0})]})[0] == 201
        st, job = call("GET", "/api/job", {"worker_id": 7})
        assert st == 200 and job["job_id"] == 1
        st, listing = call("GET", "/api/jobs")
        assert st == 200 and [j["id"] for j in listing["jobs"]] == [1]
        assert call("POST", "/api/job", {"worker_id": 7, "job_id": 1})[0] == 204
        assert q.job(1).state == "done" and q.pending() == 2
    finally:
        srv.shutdown()


def test_autotune_assign_respects_1d_size_limits():
    """A cluster size tuned on one size of a bucket is not applied where it does not fit."""
    from nls_gb300 import autotune
    from nls_gb300.batch import Spec
    specs = [Spec(1, n, 5, 1e-4, 0.04, np.zeros(23)) for n in (4500, 8192, 6000)]
    autotune.assign(specs, {"1d/o5/n<=8192": 2})
    assert [s.variant for s in specs] == [2, 4, 2]
    for s in specs:
        assert autotune.feasible_1d(s.n, s.variant, 5, np.complex64)
    assert not autotune.feasible_1d(8192, 2, 5, np.complex64) and autotune.feasible_1d(4096, 1, 5, np.complex64)
