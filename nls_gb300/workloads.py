"""Seeded synthetic workloads with the shapes, sizes and value distributions of the benchmark
configurations (no dataset is involved; every input is generated from a fixed seed).

* plain_1d      -- radial grid of 1000 nodes on [0, 40] (dx = 0.04), Gaussian pump 4 exp(-x^2/8),
                   order 5, dt = 1e-4, 10 000 steps, psi0 = 1e-3 complex Gaussian noise (seed 0).
* plain_2d      -- 256 x 256 on [-20, 20]^2 (dx = 40/256), ring pump 6 exp(-(r-8)^2/2), order 3,
                   dt = 5e-5, 20 000 steps, same noise.
* precision_2d  -- 1024 x 1024 on [-40, 40]^2, ring radius 15, width (variation) 2, amplitude 6,
                   order 5, dt = 1e-5, 50 000 steps, complex64 state.
* batch_mix     -- 256 radial grids with sizes log-uniform over [500, 8192] and 256 square grids
                   with sides from {64, 128, 192, 256, 384, 512}; per-instance seed 1000+i:
                   amplitude U[2, 8], Gaussian or ring pump, gamma U[0.3, 0.8], R U[0.5, 2],
                   g_R U[1, 3]; 1-D dx = 0.04, dt = 1e-4; 2-D dx = 0.15625, dt = 5e-5; 5000 steps.
* serve_stream  -- requests drawn from the batch_mix distribution with steps U[1000, 20000].

Physics coefficients follow the reference's 23-vector (coeffs(k) at index k-1): c3 = R/2,
c4 = gamma/2, c5 = g, c6 = 2 g_R, c12 = 1, c13 = gamma_R, c14 = R, with g = 1, gamma_R = 1.
Pumps are evaluated on the reference's grids (nls/model.py:220-232): linspace(0, n dx, n) in 1-D
and meshgrid(linspace(-n dx/2, n dx/2, n)) in 2-D.
"""

from __future__ import annotations

import numpy as np

from .batch import Spec
from .pumping import GaussianPumping1D, GaussianPumping2D, GaussianRingPumping1D, GaussianRingPumping2D


def coeffs(g=1.0, g_R=2.0, R=1.0, gamma=0.5, gamma_R=1.0) -> np.ndarray:
    c = np.zeros(23)
    c[0] = c[1] = 1.0
    c[2] = R / 2.0
    c[3] = gamma / 2.0
    c[4] = g
    c[5] = 2.0 * g_R
    c[11] = 1.0
    c[12] = gamma_R
    c[13] = R
    return c


def grid_1d(n, dx):
    return np.linspace(0.0, n * dx, n)


def grid_2d(n, dx):
    x = np.linspace(-n * dx / 2, n * dx / 2, n)
    return np.meshgrid(x, x)


def noise(shape, rng, amp=1e-3):
    return amp * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))


def plain_1d(n=1000, length=40.0, order=5, dt=1e-4, steps=10000, seed=0) -> tuple:
    dx = length / n
    P = GaussianPumping1D(power=4.0, variation=2.0)(grid_1d(n, dx))
    u0 = noise(n, np.random.default_rng(seed))
    return Spec(1, n, order, dt, dx, coeffs(), pumping=P, u0=u0), steps


def plain_2d(n=256, length=40.0, order=3, dt=5e-5, steps=20000, seed=0) -> tuple:
    dx = length / n
    P = GaussianRingPumping2D(power=6.0, radius=8.0, variation=1.0)(*grid_2d(n, dx))
    u0 = noise((n, n), np.random.default_rng(seed))
    return Spec(2, n, order, dt, dx, coeffs(), pumping=P, u0=u0), steps


def precision_2d(n=1024, length=80.0, order=5, dt=1e-5, steps=50000, seed=0) -> tuple:
    dx = length / n
    P = GaussianRingPumping2D(power=6.0, radius=15.0, variation=2.0)(*grid_2d(n, dx))
    u0 = noise((n, n), np.random.default_rng(seed))
    return Spec(2, n, order, dt, dx, coeffs(), pumping=P, u0=u0), steps


SIDES_2D = (64, 128, 192, 256, 384, 512)


def mix_instance(i: int, dim: int, with_data: bool = True, variant: int = -1) -> Spec:
    """Instance i of the mixed 1-D/2-D population (seed 1000 + i)."""
    rng = np.random.default_rng(1000 + i)
    amp = rng.uniform(2.0, 8.0)
    ring = bool(rng.integers(0, 2))
    gamma = rng.uniform(0.3, 0.8)
    R = rng.uniform(0.5, 2.0)
    g_R = rng.uniform(1.0, 3.0)
    c = coeffs(g=1.0, g_R=g_R, R=R, gamma=gamma, gamma_R=1.0)
    if dim == 1:
        n = int(round(np.exp(rng.uniform(np.log(500), np.log(8192)))))
        dx, dt, order = 0.04, 1e-4, 5
        spec = Spec(1, n, order, dt, dx, c, variant=variant)
        if with_data:
            x = grid_1d(n, dx)
            pump = (GaussianRingPumping1D(amp, radius=0.25 * n * dx, variation=2.0) if ring
                    else GaussianPumping1D(power=amp, variation=2.0))
            spec.pumping = pump(x)
            spec.u0 = noise(n, rng)
    else:
        n = int(SIDES_2D[int(rng.integers(0, len(SIDES_2D)))])
        dx, dt, order = 0.15625, 5e-5, 3
        spec = Spec(2, n, order, dt, dx, c, variant=variant)
        if with_data:
            X, Y = grid_2d(n, dx)
            L = n * dx
            pump = (GaussianRingPumping2D(amp, radius=0.25 * L, variation=1.0) if ring
                    else GaussianPumping2D(power=amp, variation=0.1 * L))
            spec.pumping = pump(X, Y)
            spec.u0 = noise((n, n), rng)
    return spec


def batch_mix(n1=256, n2=256, with_data=True):
    """The 512-instance mix: first n1 radial instances, then n2 square ones."""
    specs = [mix_instance(i, 1, with_data) for i in range(n1)]
    specs += [mix_instance(n1 + i, 2, with_data) for i in range(n2)]
    return specs


def serve_stream(count=10000, seed=7, with_data=True):
    """Requests (Spec, steps) of the mixed distribution with steps U[1000, 20000]."""
    rng = np.random.default_rng(seed + 1)
    reqs = []
    for i in range(count):
        dim = 1 if rng.random() < 0.5 else 2
        spec = mix_instance(5000 + i, dim, with_data)
        reqs.append((spec, int(rng.integers(1000, 20001))))
    return reqs
