"""GPU parity of the drop-in call chain and of the 1-D complex64 cluster kernels.

The reference's user-facing path is ``Model.solve`` (nls/model.py:252-255) ->
``AbstractSolver.__call__`` (nls/solver.py:21-38) -> ``nls.solve_nls`` / ``nls.solve_nls_2d``
of the f2py module, and ``Solver1D/2D.chemicalPotential`` (nls/solver.py:40-45, 65-69, 79-83)
-> ``chemical_potential_1d/2d``.  Here the same chain runs through ``nls_gb300`` on the GPU and
its results are compared with the FP64 oracle on exactly the inputs the chain passes down (the
model's pump grid with its n*dx/(n-1) spacing, nls/model.py:220-232, its coefficient vector and
its initial state -- the real default ``u0 = 0.1``, nls/model.py:86-102, selects the complex128
path).  Tolerances: complex128 <= 1e-10 relative L2; complex64 <= 3e-5 against the FP32 oracle
and <= 1e-4 on |psi|^2 against the FP64 oracle.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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


def _config0_model(**kw):
    from nls_gb300 import Problem
    from nls_gb300.pumping import GaussianPumping1D
    args = dict(model="1d", dx=0.04, dt=1e-4, num_nodes=1000, num_iters=10000, order=5,
                pumping=GaussianPumping1D(power=4.0, variation=2.0))
    args.update(kw)
    return Problem().model(**args)


def _config1_model(**kw):
    from nls_gb300 import Problem
    from nls_gb300.pumping import GaussianRingPumping2D
    args = dict(model="2d", dx=40.0 / 256, dt=5e-5, num_nodes=256, num_iters=20000, order=3,
                pumping=GaussianRingPumping2D(power=6.0, radius=8.0, variation=1.0))
    args.update(kw)
    return Problem().model(**args)


def _oracle_of(oracle_lib, model, iters, dtype, threads=1):
    return oracle_lib.solve(model.getTimeStep(), model.getSpatialStep(), model.getApproximationOrder(), iters,
                            model.getPumping(), model.getCoefficients(), model.getInitialSolution(),
                            dtype=dtype, threads=threads)


def test_problem_model_solve_1d_config0(gpu, oracle_lib):
    """Problem().model('1d', config-0 parameters).solve() with the real default u0 = 0.1."""
    from nls_gb300.model import Model1D, Solution
    from nls_gb300.solver import Solver1D
    model = _config0_model()
    assert isinstance(model, Model1D) and isinstance(model.getSolver(), Solver1D)
    assert np.asarray(model.getInitialSolution()).dtype == np.float64
    sol = model.solve()
    assert isinstance(sol, Solution) and sol.getElapsedTime() > 0
    got = sol.getSolution()
    assert got.dtype == np.complex128 and got.shape == (1000,)
    want = _oracle_of(oracle_lib, model, 10000, np.float64)
    assert np.all(np.isfinite(got))
    assert rel(got, want) <= 1e-10
    # chemicalPotential through the solver facade and through the model
    mu = model.getChemicalPotential(sol)
    mu_want = oracle_lib.chemical_potential(model.getSpatialStep(), model.getPumping(), model.getCoefficients(),
                                            got, dtype=np.float64)
    assert isinstance(mu, complex)
    assert abs(mu - mu_want) <= 1e-10 * abs(mu_want)
    assert model.getSolver().chemicalPotential(got) == mu


def test_problem_model_solve_2d_config1(gpu, oracle_lib):
    """Problem().model('2d', config-1 parameters).solve() with the real default u0 = 0.1."""
    import os
    from nls_gb300.model import Model2D
    from nls_gb300.solver import Solver2D
    model = _config1_model()
    assert isinstance(model, Model2D) and isinstance(model.getSolver(), Solver2D)
    sol = model.solve()
    got = sol.getSolution()
    assert got.dtype == np.complex128 and got.shape == (256, 256)
    want = _oracle_of(oracle_lib, model, 20000, np.float64, threads=os.cpu_count() or 1)
    assert rel(got, want) <= 1e-10
    mu = model.getChemicalPotential(sol)
    mu_want = oracle_lib.chemical_potential(model.getSpatialStep(), model.getPumping(), model.getCoefficients(),
                                            got, dtype=np.float64)
    assert isinstance(mu, float)
    assert abs(mu - mu_want) <= 1e-10 * abs(mu_want)


@pytest.mark.parametrize("dim", [1, 2])
def test_problem_model_solve_complex64(gpu, oracle_lib, dim):
    """A complex64 initial state selects the precision form through the same chain."""
    rng = np.random.default_rng(3)
    if dim == 1:
        u0 = (0.1 + 1e-3 * (rng.standard_normal(1000) + 1j * rng.standard_normal(1000))).astype(np.complex64)
        model = _config0_model(u0=u0, num_iters=2000)
    else:
        u0 = (0.1 + 1e-3 * (rng.standard_normal((96, 96)) + 1j * rng.standard_normal((96, 96)))).astype(np.complex64)
        model = _config1_model(u0=u0, num_nodes=96, num_iters=600)
    got = model.solve().getSolution()
    assert got.dtype == np.complex64
    iters = model.getNumberOfIterations()
    want32 = _oracle_of(oracle_lib, model, iters, np.float32)
    want64 = _oracle_of(oracle_lib, model, iters, np.float64)
    assert rel(got, want32) <= 3e-5
    assert rel(np.abs(got) ** 2, np.abs(want64) ** 2) <= 1e-4


def test_solution_integrals_of_a_gpu_solution(gpu):
    """getDampingIntegral / getParticleNumber on a GPU-solved state against numpy restatements of
    nls/model.py:350-365 (rectangle rule, radial weight 2 pi r dx on linspace(0, n dx, n)) and of
    the reference's Simpson particle number (nls/model.py:216-217)."""
    from scipy.integrate import simpson
    for model in (_config0_model(num_iters=500), _config1_model(num_nodes=64, num_iters=300)):
        sol = model.solve()
        u = sol.getSolution()
        c = model.getCoefficients()
        P = model.getPumping()
        dens = np.abs(u) ** 2
        res = c[11] * P / (c[12] + c[13] * dens)
        dx = model.getSpatialStep()
        if u.ndim == 1:
            r = np.linspace(0, u.size * dx, u.size)
            want = 2 * np.pi * np.sum((res - 1.0) * dens * r * dx)
        else:
            want = np.sum((res - 1.0) * dens * dx ** 2)
        assert abs(sol.getDampingIntegral() - want) <= 1e-12 * max(1.0, abs(want))
        np.testing.assert_allclose(sol.getReservoir(), res, rtol=1e-14)
        model.solution = u          # the reference reads model.solution (nls/model.py:216-217)
        np.testing.assert_allclose(model.getParticleNumber(), simpson(dens, dx=dx), rtol=1e-13, atol=0)


# ------------------------------------------------------------------ 1-D complex64 clusters

def _feasible_c64(n, cl, K):
    """The resident 1-D kernels' size rule for complex64 (segment limit 4096 nodes)."""
    seg = (n + cl - 1) // cl
    if cl == 1:
        return 2 * K <= seg <= 4096
    return seg >= 4 * K and seg + 8 * K <= 4096


@pytest.mark.parametrize("n", [4096, 4097, 8192])
@pytest.mark.parametrize("cl", [1, 2, 4, 8, 16])
def test_1d_c64_clusters_large_grids(gpu, oracle_lib, n, cl):
    """complex64 radial grids up to 8192 nodes on every cluster size (the batch runs 8192 nodes on
    4-CTA clusters) against the FP32 oracle (3e-5) and the FP64 oracle on |psi|^2 and n (1e-4)."""
    from nls_gb300 import workloads as w
    from nls_gb300.native import nls  # noqa: F401
    import torch
    from nls_gb300 import device
    s, _ = w.plain_1d(n=n, length=n * 0.04, order=5, seed=11)
    iters = 800
    u = torch.tensor(s.u0.astype(np.complex64), device="cuda")
    P = torch.tensor(s.pumping.astype(np.float32), device="cuda")
    if not _feasible_c64(n, cl, 2):
        with pytest.raises(ValueError):
            device.solve_(u, P, order=5, dt=s.dt, dx=s.dx, coeffs=s.coeffs, iters=iters, variant=cl)
        return
    device.solve_(u, P, order=5, dt=s.dt, dx=s.dx, coeffs=s.coeffs, iters=iters, variant=cl)
    got = u.cpu().numpy()
    want32 = oracle_lib.solve(s.dt, s.dx, 5, iters, s.pumping, s.coeffs, s.u0, dtype=np.float32)
    want64 = oracle_lib.solve(s.dt, s.dx, 5, iters, s.pumping, s.coeffs, s.u0, dtype=np.float64)
    assert rel(got, want32) <= 3e-5
    d64 = np.abs(want64) ** 2
    assert rel(np.abs(got) ** 2, d64) <= 1e-4
    c = s.coeffs
    n_got = c[11] * s.pumping / (c[12] + c[13] * np.abs(got) ** 2)
    n_want = c[11] * s.pumping / (c[12] + c[13] * d64)
    assert rel(n_got, n_want) <= 1e-4


@pytest.mark.parametrize("order", [3, 7])
def test_1d_c64_cluster_other_orders(gpu, oracle_lib, order):
    import torch
    from nls_gb300 import device
    from nls_gb300 import workloads as w
    s, _ = w.plain_1d(n=4097, length=4097 * 0.04, order=order, seed=12)
    u = torch.tensor(s.u0.astype(np.complex64), device="cuda")
    P = torch.tensor(s.pumping.astype(np.float32), device="cuda")
    device.solve_(u, P, order=order, dt=s.dt, dx=s.dx, coeffs=s.coeffs, iters=600, variant=4)
    want32 = oracle_lib.solve(s.dt, s.dx, order, 600, s.pumping, s.coeffs, s.u0, dtype=np.float32)
    assert rel(u.cpu().numpy(), want32) <= 3e-5


# ------------------------------------------------------------------ tools/check.py on device reductions

@pytest.mark.parametrize("dim", [1, 2])
def test_checks_fed_by_device_reductions_match_the_host_loop(gpu, dim):
    """check_convergence / check_integral on the GPU-resident state and FP64 device reductions
    against the reference's host loop (tools/check.py:33-37: setInitialSolution, solve(num_iters),
    getChemicalPotential, getDampingIntegral) run through the same API."""
    import copy
    from nls_gb300 import checks
    model = _config0_model(num_iters=400) if dim == 1 else _config1_model(num_nodes=72, num_iters=200)
    sol = model.solve()
    hist = checks.convergence_history(sol, num_steps=6, num_iters=25)
    # the host loop of the reference, through Problem/Model/Solution and nls.native
    m2 = copy.deepcopy(model)
    prof = sol
    eig, ints = [], []
    for _ in range(6):
        m2.setInitialSolution(prof.getSolution())
        prof = m2.solve(25)
        eig.append(m2.getChemicalPotential(prof.getSolution()))
        ints.append(prof.getDampingIntegral())
    eig = np.array(eig, dtype=complex)
    np.testing.assert_allclose(hist["eigenvalues"], eig, rtol=1e-9, atol=0)
    np.testing.assert_allclose(hist["integrals"], ints, rtol=1e-9, atol=1e-12)
    assert checks.check_convergence(sol, num_steps=6, num_iters=25) == (np.std(eig) < checks.TOLERANCE)
    di = checks.damping_integral(sol)
    assert abs(di - sol.getDampingIntegral()) <= 1e-10 * max(1.0, abs(di))
    assert checks.check_integral(sol) == (abs(sol.getDampingIntegral()) <= checks.TOLERANCE)


def test_job_intake_feeds_the_pool(gpu):
    """schedulr-shaped jobs served by a complex128 pool equal Model.solve() of the same jobs
    (the reference worker's path, schedulr/workr.py:45-75) to the drop-in tolerance."""
    import json
    from nls_gb300.intake import JobQueue, job_model, run_jobs
    from nls_gb300.serve import Pool
    q = JobQueue()
    descs = [{"power": 2.0, "num_nodes": 48, "num_iters": 60},
             {"power": 3.5, "num_nodes": 40, "num_iters": 45, "order": 3},
             {"power": 1.5, "model": "1d", "num_nodes": 300, "num_iters": 80}]
    ids = q.post_jobs([json.dumps(d) for d in descs])
    pool = Pool(dtype=np.complex128, budget_bytes=1 << 28, chunk_steps=25)
    sols = run_jobs(q, pool, dtype=np.complex128)
    pool.close()
    assert sorted(sols) == ids and q.pending() == 0
    for jid, d in zip(ids, descs):
        assert q.job(jid).state == "done"
        want = job_model(json.dumps(d)).solve().getSolution()
        got = sols[jid].getSolution()
        assert got.shape == want.shape
        assert rel(got, want) <= 1e-10, (jid, rel(got, want))
