"""GPU parity: every kernel path of libnls_gb300.so against the CPU oracle.

Tolerances (relative L2 over the whole field):
* complex128 path vs the float64 oracle: <= 1e-10 (the drop-in contract);
* complex64 form vs the float32 oracle: <= 3e-5; vs the float64 oracle on |psi|^2 and on the
  reservoir n: <= 1e-4 (the precision form's contract);
* batched, served and resumed results vs single solves on the same kernel path: bit-identical.
"""

import os

import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.fixture(scope="module")
def gpu():
    import torch
    from nls_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from nls_gb300 import _lib
    _lib.lib()
    return torch


def _spec_1d(n, order, seed=0, dt=1e-4, dx=0.04):
    from nls_gb300 import workloads as w
    s, _ = w.plain_1d(n=n, length=n * dx, order=order, dt=dt, seed=seed)
    return s


def _spec_2d(n, order, seed=0, dt=5e-5, dx=0.15625):
    from nls_gb300 import workloads as w
    s, _ = w.plain_2d(n=n, length=n * dx, order=order, dt=dt, seed=seed)
    return s


def _device_solve(torch, s, iters, dtype, variant):
    from nls_gb300 import device
    ct = torch.complex128 if dtype == np.complex128 else torch.complex64
    rt = torch.float64 if dtype == np.complex128 else torch.float32
    # 2-D: torch row-major (n, n) with the last index contiguous == Fortran-order numpy memory
    u0 = np.asarray(s.u0).T if s.dim == 2 else s.u0
    P = np.asarray(s.pumping).T if s.dim == 2 else s.pumping
    u = torch.tensor(np.ascontiguousarray(u0), dtype=ct, device="cuda")
    Pt = torch.tensor(np.ascontiguousarray(P), dtype=rt, device="cuda")
    device.solve_(u, Pt, order=s.order, dt=s.dt, dx=s.dx, coeffs=s.coeffs, iters=iters, variant=variant)
    out = u.cpu().numpy()
    return out.T if s.dim == 2 else out


# ------------------------------------------------------------------ complex128 drop-in path

@pytest.mark.parametrize("order", [3, 5, 7])
@pytest.mark.parametrize("variant", [-1, 1, 2, 4, 16, 0])
def test_1d_c128_matches_oracle(gpu, oracle_lib, order, variant):
    s = _spec_1d(257, order)
    iters = 300
    want = oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=np.float64)
    got = _device_solve(gpu, s, iters, np.complex128, variant)
    assert rel(got, want) <= 1e-10


def test_1d_plain_config_full(gpu, oracle_lib):
    """1000 nodes on [0, 40], order 5, dt 1e-4, 10 000 steps, through the f2py-shaped API."""
    from nls_gb300 import workloads as w
    from nls_gb300.native import nls
    s, steps = w.plain_1d()
    want = oracle_lib.solve(s.dt, s.dx, s.order, steps, s.pumping, s.coeffs, s.u0, dtype=np.float64)
    got = nls.solve_nls(s.dt, s.dx, s.order, steps, s.pumping, s.coeffs, s.u0)
    assert got.dtype == np.complex128
    assert rel(got, want) <= 1e-10


@pytest.mark.parametrize("order", [3, 5])
@pytest.mark.parametrize("variant", [-1, 0, 3])
@pytest.mark.parametrize("n", [61, 100])
def test_2d_c128_matches_oracle(gpu, oracle_lib, order, variant, n):
    s = _spec_2d(n, order)
    iters = 130
    want = oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=np.float64)
    got = _device_solve(gpu, s, iters, np.complex128, variant)
    assert rel(got, want) <= 1e-10


def test_2d_plain_config_full(gpu, oracle_lib):
    """256 x 256 on [-20, 20]^2, ring pump, order 3, dt 5e-5, 20 000 steps via solve_nls_2d."""
    from nls_gb300 import workloads as w
    from nls_gb300.native import nls
    s, steps = w.plain_2d()
    got = nls.solve_nls_2d(s.dt, s.dx, s.order, steps, s.pumping, s.coeffs, s.u0)
    want = oracle_lib.solve(s.dt, s.dx, s.order, steps, s.pumping, s.coeffs, s.u0, dtype=np.float64,
                            threads=os.cpu_count() or 1)
    assert rel(got, want) <= 1e-10


def test_golden_restatement_fixtures(gpu):
    """GPU against the scipy-BLAS restatement fixtures (both precisions)."""
    from nls_gb300.native import nls
    fx = dict(np.load(os.path.join(GOLDEN, "restatement_small.npz")))
    n, dx, dt, iters, n2, dx2, dt2, iters2 = fx["params"]
    for order in (3, 5, 7):
        got = nls.solve_nls(dt, dx, order, int(iters), fx["p1d"], fx["coeffs"], fx["u1d_0"])
        assert rel(got, fx[f"u1d_o{order}_f64"]) <= 1e-10
        got = nls.solve_nls(dt, dx, order, int(iters), fx["p1d"], fx["coeffs"], fx["u1d_0"].astype(np.complex64))
        assert rel(got, fx[f"u1d_o{order}_f32"]) <= 3e-5
    for order in (3, 5):
        got = nls.solve_nls_2d(dt2, dx2, order, int(iters2), fx["p2d"], fx["coeffs"], fx["u2d_0"])
        assert rel(got, fx[f"u2d_o{order}_f64"]) <= 1e-10
        got = nls.solve_nls_2d(dt2, dx2, order, int(iters2), fx["p2d"], fx["coeffs"], fx["u2d_0"].astype(np.complex64))
        assert rel(got, fx[f"u2d_o{order}_f32"]) <= 3e-5


def test_chemical_potential_matches_oracle(gpu, oracle_lib):
    from nls_gb300.native import nls
    s = _spec_1d(300, 5)
    u = s.u0 * 100 + 0.05
    mu = nls.chemical_potential_1d(s.dx, s.pumping, s.coeffs, u)
    want = oracle_lib.chemical_potential(s.dx, s.pumping, s.coeffs, u, dtype=np.float64)
    assert abs(mu - want) <= 1e-10 * abs(want)
    s2 = _spec_2d(48, 5)
    u2 = s2.u0 * 100 + 0.05
    mu2 = nls.chemical_potential_2d(s2.dx, s2.pumping, s2.coeffs, u2)
    want2 = oracle_lib.chemical_potential(s2.dx, s2.pumping, s2.coeffs, u2, dtype=np.float64)
    assert abs(mu2 - want2) <= 1e-10 * abs(want2)


# ------------------------------------------------------------------ complex64 precision form

@pytest.mark.parametrize("order", [3, 5, 7])
@pytest.mark.parametrize("variant", [-1, 1, 2, 0])
def test_1d_c64_vs_oracles(gpu, oracle_lib, order, variant):
    s = _spec_1d(700, order)
    iters = 2000
    want32 = oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=np.float32)
    want64 = oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=np.float64)
    got = _device_solve(gpu, s, iters, np.complex64, variant)
    assert rel(got, want32) <= 3e-5
    assert rel(np.abs(got) ** 2, np.abs(want64) ** 2) <= 1e-4


_ORACLE_2D = {}


def _oracle_2d_pair(oracle_lib, s, order, iters):
    """FP32 and FP64 oracle results of a 2-D case, computed once per (size, order, steps)."""
    key = (s.u0.shape[0], order, iters)
    if key not in _ORACLE_2D:
        _ORACLE_2D[key] = tuple(
            oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=dt, threads=8)
            for dt in (np.float32, np.float64))
    return _ORACLE_2D[key]


# n = 150: plain global loads (rows not 16-byte multiples); n = 152: the TMA tile path
@pytest.mark.parametrize("n", [150, 152])
@pytest.mark.parametrize("order", [3, 5])
@pytest.mark.parametrize("variant", [-1, 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15])
def test_2d_c64_vs_oracles(gpu, oracle_lib, order, variant, n):
    s = _spec_2d(n, order)
    iters = 400
    want32, want64 = _oracle_2d_pair(oracle_lib, s, order, iters)
    got = _device_solve(gpu, s, iters, np.complex64, variant)
    assert rel(got, want32) <= 3e-5
    d64 = np.abs(want64) ** 2
    assert rel(np.abs(got) ** 2, d64) <= 1e-4
    c = s.coeffs
    n_got = c[11] * s.pumping / (c[12] + c[13] * np.abs(got) ** 2)
    n_want = c[11] * s.pumping / (c[12] + c[13] * d64)
    assert rel(n_got, n_want) <= 1e-4


def test_device_error_reductions(gpu):
    import torch
    from nls_gb300 import device
    rng = np.random.default_rng(1)
    a = rng.standard_normal(5000) + 1j * rng.standard_normal(5000)
    b = a * (1 + 1e-3 * rng.standard_normal(5000))
    P = rng.random(5000)
    c = np.zeros(23)
    c[11], c[12], c[13] = 1.0, 1.0, 0.7
    ta = torch.tensor(a.astype(np.complex64), device="cuda")
    tb = torch.tensor(b, device="cuda")
    tP = torch.tensor(P, device="cuda")
    d, r = device.density_errors(ta, tb, tP, c)
    a32 = a.astype(np.complex64).astype(np.complex128)
    np.testing.assert_allclose(d, rel(np.abs(a32) ** 2, np.abs(b) ** 2), rtol=1e-9)
    na = P / (1 + 0.7 * np.abs(a32) ** 2)
    nb = P / (1 + 0.7 * np.abs(b) ** 2)
    np.testing.assert_allclose(r, rel(na, nb), rtol=1e-9)
    np.testing.assert_allclose(device.norm(tb), np.sum(np.abs(b) ** 2), rtol=1e-12)


def test_nonfinite_state_is_reported(gpu):
    import torch
    from nls_gb300 import _lib, device
    u = torch.zeros(1000, dtype=torch.complex128, device="cuda")
    u[17] = complex(float("nan"), 0.0)
    with pytest.raises(_lib.NativeError) as ei:
        device.norm(u)
    assert ei.value.status == _lib.NLS_ERR_NONFINITE


# ------------------------------------------------------------------ edge cases

def test_edge_sizes_and_iteration_counts(gpu, oracle_lib):
    from nls_gb300.native import nls
    for order in (3, 5, 7):
        s = _spec_1d(order, order, dx=0.3)            # smallest grid the operator allows
        for iters in (0, 1, 7):
            want = oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=np.float64)
            got = nls.solve_nls(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0)
            assert rel(got, want) <= 1e-10 if np.linalg.norm(want) else np.array_equal(got, want)
    for order in (3, 5):
        for n in (order, 33, 57):
            s = _spec_2d(n, order)
            for iters in (0, 1, 65):
                want = oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=np.float64)
                got = nls.solve_nls_2d(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0)
                assert rel(got, want) <= 1e-10


def test_invalid_arguments_raise(gpu):
    from nls_gb300.native import nls
    s = _spec_1d(64, 5)
    with pytest.raises(ValueError):
        nls.solve_nls(s.dt, s.dx, 4, 10, s.pumping, s.coeffs, s.u0)
    s2 = _spec_2d(16, 3)
    with pytest.raises(ValueError):
        nls.solve_nls_2d(s2.dt, s2.dx, 7, 10, s2.pumping, s2.coeffs, s2.u0)


# ------------------------------------------------------------------ resume, batch, pool

@pytest.mark.parametrize("dim,variant,dtype", [(1, -1, np.complex128), (1, 0, np.complex64),
                                               (2, 1, np.complex64), (2, 8, np.complex64), (2, 15, np.complex64),
                                               (2, 0, np.complex128), (2, 3, np.complex128)])
def test_resume_is_bitwise(gpu, dim, variant, dtype):
    """One solve of N steps equals k solves of N/k steps from the device-resident state."""
    import torch
    from nls_gb300 import device
    s = _spec_1d(300, 5) if dim == 1 else _spec_2d(90, 3)
    ct = torch.complex128 if dtype == np.complex128 else torch.complex64
    rt = torch.float64 if dtype == np.complex128 else torch.float32
    P = torch.tensor(np.ascontiguousarray(s.pumping), dtype=rt, device="cuda")
    u1 = torch.tensor(np.ascontiguousarray(s.u0), dtype=ct, device="cuda")
    u2 = u1.clone()
    device.solve_(u1, P, order=s.order, dt=s.dt, dx=s.dx, coeffs=s.coeffs, iters=195, variant=variant)
    for _ in range(3):
        device.solve_(u2, P, order=s.order, dt=s.dt, dx=s.dx, coeffs=s.coeffs, iters=65, variant=variant)
    assert torch.equal(u1, u2)


def _mixed_specs(dtype):
    from nls_gb300 import workloads as w
    specs = [w.mix_instance(i, 1) for i in range(5)] + [w.mix_instance(10 + i, 2) for i in range(6)]
    # include sizes that are not multiples of any tile and the smallest allowed sides
    extra = _spec_2d(37, 3)
    extra.variant = 3
    specs.append(extra)
    return specs


@pytest.mark.parametrize("dtype,shape2d", [(np.complex64, -1), (np.complex64, 12), (np.complex64, 9),
                                            (np.complex64, 15), (np.complex128, -1)])
def test_batch_matches_single_solves(gpu, dtype, shape2d):
    from nls_gb300.batch import BatchSolver
    specs = _mixed_specs(dtype)
    if shape2d > 0:
        for s in specs[:-1]:          # the last one keeps its own 32x32 tile: two 2-D groups
            if s.dim == 2:
                s.variant = shape2d
    b = BatchSolver(specs, dtype=dtype)
    b.run(57)
    b.run(20)
    for i, s in enumerate(specs):
        got = b.get(i)
        want = _device_solve(gpu, s, 77, dtype, s.variant)
        assert np.array_equal(got, want.astype(got.dtype)), i


def test_batch_set_get_many_match_per_instance(gpu):
    """The one-wait bulk upload and download equal per-instance set/get bit for bit, on a
    sub-range and on the whole batch."""
    from nls_gb300.batch import BatchSolver
    specs = _mixed_specs(np.complex64)
    a = BatchSolver(specs, dtype=np.complex64)
    b = BatchSolver([copy.copy(s) for s in specs], dtype=np.complex64)
    rng = np.random.default_rng(5)
    newP, newU = [], []
    for s in specs:
        shape = (s.n, s.n) if s.dim == 2 else (s.n,)
        newP.append(rng.uniform(0.5, 2.0, shape).astype(np.float32))
        newU.append((rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64) * 0.1)
    lo, hi = 1, len(specs) - 1
    for i in range(lo, hi):
        a.set(i, newP[i], newU[i])
    b.set_many(newP[lo:hi], newU[lo:hi], first=lo)
    a.run(33)
    b.run(33)
    whole = b.get_many()
    part = b.get_many([np.empty_like(whole[i], order="F" if specs[i].dim == 2 else "C")
                       for i in range(lo, hi)], first=lo)
    for i in range(len(specs)):
        want = a.get(i)
        assert np.array_equal(whole[i], want), i
        if lo <= i < hi:
            assert np.array_equal(part[i - lo], want), i
    with pytest.raises(ValueError):
        b.get_many(first=len(specs) - 1, outs=[None, None])


@pytest.mark.parametrize("steps", [34, 33])   # 2-D states end in the first / second buffer
def test_batch_packed_layout_matches_per_instance(gpu, steps):
    """Packed blocks: offsets in instance order, 256-byte aligned and padded; the packed upload and
    download equal per-instance set/get bit for bit, whichever state buffer is current."""
    from nls_gb300.batch import BatchSolver
    specs = _mixed_specs(np.complex64)
    a = BatchSolver(specs, dtype=np.complex64)
    b = BatchSolver([copy.copy(s) for s in specs], dtype=np.complex64)
    po, so, pb, sb = b.layout()
    for offs, total, item in ((po, pb, 4), (so, sb, 8)):
        ends = [o + s.nodes * item for o, s in zip(offs, specs)]
        assert offs[0] == 0 and all(o % 256 == 0 for o in offs)
        assert all(e <= o2 for e, o2 in zip(ends[:-1], offs[1:])) and ends[-1] <= total
        assert all(o2 - e < 256 for e, o2 in zip(ends[:-1], list(offs[1:]))) and total - ends[-1] < 256
    rng = np.random.default_rng(9)
    hP, hU = np.zeros(pb, np.uint8), np.zeros(sb, np.uint8)
    for i, (p, u) in enumerate(zip(b.packed_views(hP, "pump"), b.packed_views(hU, "state"))):
        p[...] = rng.uniform(0.5, 2.0, p.shape)
        u[...] = (rng.normal(size=u.shape) + 1j * rng.normal(size=u.shape)) * 0.1
        a.set(i, p, u)
    b.set_packed(hP, hU)
    a.run(steps)
    b.run(steps)
    out = b.get_packed()
    for i, got in enumerate(b.packed_views(out, "state")):
        assert np.array_equal(got, a.get(i)), i
    # a second packed upload over states that sit in the second buffer, then one more run
    b.set_packed(hP, hU)
    for i, (p, u) in enumerate(zip(b.packed_views(hP, "pump"), b.packed_views(hU, "state"))):
        a.set(i, p, u)
    a.run(5)
    b.run(5)
    for i, got in enumerate(b.packed_views(b.get_packed(), "state")):
        assert np.array_equal(got, a.get(i)), i
    with pytest.raises(ValueError):
        b.set_packed(hP[:-1], hU)


@pytest.mark.parametrize("variant2d", [-1, 15])
def test_pool_same_alone_and_in_the_mix(gpu, variant2d):
    from nls_gb300 import workloads as w
    from nls_gb300.serve import Pool
    target = w.mix_instance(3, 2, variant=variant2d)
    target1 = w.mix_instance(4, 1)
    alone = Pool(budget_bytes=1 << 30, chunk_steps=40)
    alone.admit(target, 123, 0)
    alone.admit(target1, 77, 1)
    while alone.status()[0]:
        alone.step()
    ra = dict([alone.take_with_state(), alone.take_with_state()])
    mix = Pool(budget_bytes=1 << 30, chunk_steps=40)
    others = [w.mix_instance(20 + i, 1 + (i % 2), variant=variant2d if i % 2 else -1) for i in range(8)]
    for k, o in enumerate(others[:4]):
        mix.admit(o, 50 + 13 * k, 100 + k)
    mix.step()                                   # the target arrives while others run
    mix.admit(target, 123, 0)
    for k, o in enumerate(others[4:]):
        mix.admit(o, 90 + 7 * k, 200 + k)
    mix.step()
    mix.admit(target1, 77, 1)
    rm = {}
    while True:
        got = mix.take_with_state()
        if got is not None:
            rm[got[0]] = got[1]
            continue
        if mix.status()[0] == 0:
            break
        mix.step()
    assert np.array_equal(ra[0], rm[0])
    assert np.array_equal(ra[1], rm[1])
    # and equal to a plain single solve on the same kernel
    want = _device_solve(gpu, target, 123, np.complex64, variant2d)
    assert np.array_equal(rm[0], want)


def test_precision_form_with_fp64_diagnostics(gpu, oracle_lib):
    """complex64 solve with FP64 norm/chemical-potential logging, checked against complex128."""
    from nls_gb300 import precision, workloads
    s, _ = workloads.precision_2d(n=192, length=192 * 0.078125)
    res = precision.run(s, steps=1200, log_every=500)
    assert [e["step"] for e in res["log"]] == [500, 1000, 1200]
    assert all(np.isfinite(e["norm"]) and np.isfinite(e["mu"]) for e in res["log"])
    assert abs(res["log"][-1]["t"] - 1200 * s.dt) < 1e-15
    assert res["rel_l2_density"] <= 1e-4 and res["rel_l2_reservoir"] <= 1e-4
    # the FP64 diagnostics agree with the oracle's chemical potential of the final state
    u = res["state"].cpu().numpy().T.astype(np.complex128)
    want = oracle_lib.chemical_potential(s.dx, s.pumping, s.coeffs, u, dtype=np.float64)
    assert abs(res["log"][-1]["mu"] - want) <= 1e-5 * abs(want)
    np.testing.assert_allclose(res["log"][-1]["norm"], np.sum(np.abs(u) ** 2) * s.dx ** 2, rtol=1e-12)


def test_autotune_batch_mode_assigns_valid_variants(gpu, tmp_path, monkeypatch):
    """Batch-mode tuning gives every spec a candidate variant, and the tuned batch matches single solves."""
    from nls_gb300 import autotune
    from nls_gb300 import workloads as w
    from nls_gb300.batch import BatchSolver
    monkeypatch.setenv("NLS_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    specs = [w.mix_instance(i, 1) for i in range(3)] + [w.mix_instance(10 + i, 2) for i in range(4)]
    got = autotune.apply(specs, dtype=np.complex64, mode="batch")
    assert got
    for s in specs:
        assert s.variant in autotune.candidates(s.dim, np.complex64, autotune.bucket(s.n))
    b = BatchSolver(specs, dtype=np.complex64)
    b.run(30)
    for i, s in enumerate(specs):
        want = _device_solve(gpu, s, 30, np.complex64, s.variant)
        assert np.array_equal(b.get(i), want.astype(np.complex64)), i


@pytest.mark.parametrize("variant", [8, 10, 12, 15])
@pytest.mark.parametrize("order", [3, 5])
@pytest.mark.parametrize("n", [5, 33, 64, 65, 97, 120, 121, 128, 200])
def test_2d_c64_register_tiles_small_and_ragged(gpu, oracle_lib, variant, order, n):
    """Register-resident tiles on grids smaller than one region, odd sides (plain loads) and
    multiples of 4 (TMA), against the FP32 oracle."""
    if n < order:
        pytest.skip("grid smaller than the stencil")
    s = _spec_2d(n, order)
    iters = 60
    want32 = oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=np.float32)
    got = _device_solve(gpu, s, iters, np.complex64, variant)
    assert rel(got, want32) <= 3e-5


def test_tile_wait_timeout_is_reported_and_the_context_recovers(gpu, oracle_lib):
    """A tile barrier armed for more bytes than its copies bring never completes: the bounded wait
    gives up (about a second), the solve reports NLS_ERR_TIMEOUT, and the next solve is correct."""
    from nls_gb300 import _lib, device
    s = _spec_2d(152, 3)                          # 152 = multiple of 4: the TMA path
    assert _lib.lib().nls_test_set_tile_tx_extra(0, 16) == _lib.NLS_OK
    try:
        # the device-pointer solve only enqueues; the context's synchronize reports the expiry
        _device_solve(gpu, s, 1, np.complex64, 10)
        with pytest.raises(_lib.NativeError) as err:
            device.context(0).synchronize()
        assert err.value.status == _lib.NLS_ERR_TIMEOUT
    finally:
        assert _lib.lib().nls_test_set_tile_tx_extra(0, 0) == _lib.NLS_OK
    got = _device_solve(gpu, s, 40, np.complex64, 10)
    want = oracle_lib.solve(s.dt, s.dx, 3, 40, s.pumping, s.coeffs, s.u0, dtype=np.float32)
    assert rel(got, want) <= 3e-5


@pytest.fixture
def stream_mode():
    """Sets the streaming kernel's launch schedule (test control) for lists set up afterwards:
    1 = several RK4 steps per launch wherever the grids take the paired form, 2 = one step per
    launch; restores the automatic choice afterwards."""
    from nls_gb300 import _lib

    def set_mode(m):
        assert _lib.lib().nls_test_set_stream_steps_per_launch(m) == _lib.NLS_OK
    yield set_mode
    set_mode(0)


@pytest.mark.parametrize("order,n", [(3, 1000), (5, 516), (3, 130), (3, 64)])
def test_2d_c64_stream_several_steps_per_launch_equal_single_steps(gpu, stream_mode, order, n):
    """The streaming step with many RK4 steps per launch (an item of step t + 1 starts once the
    items of step t it reads from or overwrites have published) equals one launch per step bit for
    bit, at both orders (grids of even side: the paired form)."""
    from nls_gb300 import device
    s = _spec_2d(n, order)
    iters = 37                                   # odd: the state ends in the scratch buffer
    u0 = gpu.tensor(np.ascontiguousarray(np.asarray(s.u0).T), dtype=gpu.complex64, device="cuda")
    P = gpu.tensor(np.ascontiguousarray(np.asarray(s.pumping).T), dtype=gpu.float32, device="cuda")
    kw = dict(order=order, dt=s.dt, dx=s.dx, coeffs=s.coeffs, variant=15)
    stream_mode(1)
    a = u0.clone()
    device.solve_(a, P, iters=iters, **kw)
    stream_mode(2)
    b = u0.clone()
    device.solve_(b, P, iters=iters, **kw)
    gpu.cuda.synchronize()
    assert gpu.equal(a, b)


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_stream_schedules_match_single_solves(gpu, stream_mode, mode):
    """A batch whose square grids share the streaming kernel, run with several steps per launch (1)
    and one step per launch (2), equals single solves bit for bit."""
    from nls_gb300.batch import BatchSolver
    specs = _mixed_specs(np.complex64)
    for s in specs[:-1]:
        if s.dim == 2:
            s.variant = 15
    stream_mode(mode)
    b = BatchSolver(specs, dtype=np.complex64)
    b.run(57)
    b.run(20)
    stream_mode(2)
    for i, s in enumerate(specs):
        want = _device_solve(gpu, s, 77, np.complex64, s.variant)
        assert np.array_equal(b.get(i), want), i


def test_batch_and_pool_stream_mixed_forms_match_single_solves(gpu):
    """Square grids of odd and even sides in one streaming group (both the paired and the per-node
    form launch every step, over one work list) in a batch and in the pool equal single solves."""
    from nls_gb300.batch import BatchSolver
    from nls_gb300.serve import Pool
    specs = []
    for k, n in enumerate((64, 97, 130, 33, 256, 121)):
        s = _spec_2d(n, 3, seed=40 + k)
        s.variant = 15
        specs.append(s)
    b = BatchSolver(specs, dtype=np.complex64)
    b.run(23)
    pool = Pool(budget_bytes=1 << 30, chunk_steps=10)
    for tag, s in enumerate(specs):
        pool.admit(s, 23 + tag, tag)
    got = {}
    while True:
        r = pool.take_with_state()
        if r is not None:
            got[r[0]] = r[1]
            continue
        if pool.status()[0] == 0:
            break
        pool.step()
    for i, s in enumerate(specs):
        assert np.array_equal(b.get(i), _device_solve(gpu, s, 23, np.complex64, 15)), i
        assert np.array_equal(got[i], _device_solve(gpu, s, 23 + i, np.complex64, 15)), i


def test_pool_stream_several_steps_per_launch_match_single_solves(gpu, stream_mode):
    """Pool chunks of the streaming kernel with several steps per launch, requests of different
    step counts (a request stops at its own count inside a launch), equal single solves."""
    from nls_gb300 import workloads as w
    from nls_gb300.serve import Pool
    stream_mode(1)
    reqs = [(w.mix_instance(30 + i, 2, variant=15), 35 + 11 * i) for i in range(5)]
    pool = Pool(budget_bytes=1 << 30, chunk_steps=40)
    for tag, (spec, steps) in enumerate(reqs):
        pool.admit(spec, steps, tag)
    got = {}
    while True:
        r = pool.take_with_state()
        if r is not None:
            got[r[0]] = r[1]
            continue
        if pool.status()[0] == 0:
            break
        pool.step()
    stream_mode(2)
    for tag, (spec, steps) in enumerate(reqs):
        want = _device_solve(gpu, spec, steps, np.complex64, 15)
        assert np.array_equal(got[tag], want), tag


def test_stream_dependency_wait_timeout_is_reported_and_the_context_recovers(gpu, oracle_lib, stream_mode):
    """A launch of several streaming steps whose dependency waits can never be met (test control):
    the first bounded wait gives up (about a second), the others stop waiting, the context's
    synchronize reports NLS_ERR_TIMEOUT, and the next solve is correct."""
    from nls_gb300 import _lib, device
    s = _spec_2d(256, 3)
    stream_mode(1)
    assert _lib.lib().nls_test_set_stream_dep_extra(0, 1 << 30) == _lib.NLS_OK
    try:
        _device_solve(gpu, s, 3, np.complex64, 15)
        with pytest.raises(_lib.NativeError) as err:
            device.context(0).synchronize()
        assert err.value.status == _lib.NLS_ERR_TIMEOUT
    finally:
        assert _lib.lib().nls_test_set_stream_dep_extra(0, 0) == _lib.NLS_OK
    got = _device_solve(gpu, s, 40, np.complex64, 15)
    want = oracle_lib.solve(s.dt, s.dx, 3, 40, s.pumping, s.coeffs, s.u0, dtype=np.float32)
    assert rel(got, want) <= 3e-5


@pytest.mark.parametrize("order", [3, 5])
def test_2d_c64_stream_4096_full_size(gpu, oracle_lib, order):
    """A 4096^2 grid on the streaming step at full size: at order 3 its work list is topped up to
    exactly one item per resident warp (strips of different segment counts), and launches follow
    each other as programmatic dependent launches; against the FP32 oracle."""
    s = _spec_2d(4096, order)
    iters = 6
    want32 = oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=np.float32,
                              threads=os.cpu_count() or 1)
    got = _device_solve(gpu, s, iters, np.complex64, 15)
    assert rel(got, want32) <= 3e-5


def test_1d_c64_register_cluster_single_solve(gpu, oracle_lib):
    """An 8192-node radial grid alone on the register-resident cluster kernel (default cluster
    size) against the FP32 oracle."""
    s = _spec_1d(8192, 5)
    iters = 500
    want32 = oracle_lib.solve(s.dt, s.dx, 5, iters, s.pumping, s.coeffs, s.u0, dtype=np.float32)
    got = _device_solve(gpu, s, iters, np.complex64, -1)
    assert rel(got, want32) <= 3e-5


@pytest.mark.parametrize("order,n", [(3, 1000), (5, 1000), (3, 1030), (5, 515)])
def test_2d_c64_stream_large_grids(gpu, oracle_lib, order, n):
    """The streaming step on grids of many strips and row segments (segment warm-up and drain,
    interior and edge strips, odd sides on the plain-load path) against the FP32 oracle."""
    s = _spec_2d(n, order)
    iters = 40
    want32 = oracle_lib.solve(s.dt, s.dx, order, iters, s.pumping, s.coeffs, s.u0, dtype=np.float32,
                              threads=os.cpu_count() or 1)
    got = _device_solve(gpu, s, iters, np.complex64, 15)
    assert rel(got, want32) <= 3e-5


def test_pipelined_serving_matches_single_solves(gpu):
    """serve(): two chunks in flight, admissions on the copy stream while chunks run, takes while
    the next chunk runs -- every request's result equals its single solve bit for bit."""
    from nls_gb300 import workloads as w
    from nls_gb300.serve import Pool, serve
    reqs = []
    for i in range(14):
        spec = w.mix_instance(300 + i, 1 + (i % 2), variant=15 if i % 4 == 1 else -1)
        reqs.append((spec, 30 + 17 * i))
    pool = Pool(budget_bytes=1 << 30, chunk_steps=25)
    st = serve(reqs, rate=400.0, pool=pool, keep_results=True)
    assert len(st["results"]) == len(reqs)
    assert 0.0 < st["gpu_busy_frac"] <= 1.0 and np.isfinite(st["queue_p99_ms"])
    for tag, (spec, steps) in enumerate(reqs):
        want = _device_solve(gpu, spec, steps, np.complex64, spec.variant)
        got = st["results"][tag]
        assert np.array_equal(got, want.astype(got.dtype)), tag
    pool.close()


def test_pool_launch_wait_protocol(gpu):
    """Two chunks in flight at most; wait() completes the oldest; requests taken while a chunk runs."""
    from nls_gb300 import workloads as w
    from nls_gb300.serve import Pool
    pool = Pool(budget_bytes=1 << 30, chunk_steps=10)
    a, b = w.mix_instance(7, 2), w.mix_instance(8, 1)
    pool.admit(a, 10, 0)
    pool.admit(b, 35, 1)
    assert pool.launch() and pool.launch() and not pool.launch()
    assert pool.info()[0] == 2
    assert pool.wait() == 1                      # the first chunk finishes request 0
    got = pool.take_with_state()                 # taken while the second chunk runs
    assert got is not None and got[0] == 0
    assert pool.launch()                         # steps 20..30 of request 1
    while pool.info()[0]:
        pool.wait()
    assert pool.launch() and pool.wait() == 1    # steps 30..35
    got1 = pool.take_with_state()
    assert got1[0] == 1
    assert np.array_equal(got[1], _device_solve(gpu, a, 10, np.complex64, -1))
    assert np.array_equal(got1[1], _device_solve(gpu, b, 35, np.complex64, -1))
    assert not pool.launch() and pool.wait() == 0 and pool.ready()
    pool.close()


def test_per_result_accuracy_of_batch_and_pool(gpu):
    """Opt-in per-result relative L2 of |psi|^2 and n against complex128 companion solves: the
    batch's figures equal a direct computation, and the batch's and the pool's meet the precision
    form's 1e-4."""
    from nls_gb300 import workloads as w
    from nls_gb300.batch import BatchSolver
    from nls_gb300.serve import Pool
    specs = [w.mix_instance(40 + i, 1 + (i % 2)) for i in range(4)]
    b = BatchSolver(specs, dtype=np.complex64, keep_inputs=True)
    b.run(60)
    b.run(40)
    acc = b.accuracy()
    for i, s in enumerate(specs):
        got = b.get(i)
        d, r = acc[i]
        assert 0.0 < d <= 1e-4 and 0.0 <= r <= 1e-4, (i, d, r)
        u64 = _device_solve(gpu, s, 100, np.complex128, -1)
        dd = rel(np.abs(got.astype(np.complex128)) ** 2, np.abs(u64) ** 2)
        assert abs(dd - d) <= 1e-6 * dd, (i, dd, d)
    pool = Pool(budget_bytes=1 << 30, chunk_steps=30, keep_inputs=True)
    for i, s in enumerate(specs):
        pool.admit(s, 50 + 10 * i, i)
    seen = 0
    while seen < len(specs):
        pool.step()
        while True:
            got = pool.take_with_accuracy()
            if got is None:
                break
            tag, state, (d, r) = got
            assert 0.0 < d <= 1e-4 and r <= 1e-4, (tag, d, r)
            seen += 1
    pool.close()
