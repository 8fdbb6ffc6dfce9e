"""Solution checks of the reference's tools/check.py, fed by FP64 reductions on the GPU.

``check_convergence`` (tools/check.py:28-61) continues a solved state ``num_steps`` times by
``num_iters`` RK4 steps and asks whether the chemical potential has settled (the standard
deviation of the sequence below ``tolerance``); ``check_integral`` (tools/check.py:63-69) asks
whether the damping integral of Solution.getDampingIntegral (nls/model.py:350-365) vanishes.  The
reference re-sends the state through f2py for every continuation and evaluates both quantities
on the host; here the state stays on the device between continuations (``device.solve_``) and
both quantities come from the library's FP64 device reductions (``nls_chemical_potential_device``,
``nls_damping_integral_device``), so only two scalars per continuation reach the host.  The
reference's plotting and printing are not reproduced; the figures come back in a dict instead.
"""

from __future__ import annotations

import numpy as np

TOLERANCE = 1.0e-1


def _device_state(solution, device: int):
    """The solution's state and its model's pump as device tensors in the library's memory order
    (2-D: the last torch axis is the Fortran first index, as nls.native passes it)."""
    import torch
    model = solution.getModel()
    u = np.asarray(solution.getSolution())
    P = np.asarray(model.getPumping())
    c128 = u.dtype != np.complex64
    ct, rt = (torch.complex128, torch.float64) if c128 else (torch.complex64, torch.float32)
    if u.ndim == 2:
        u, P = u.T, P.T
    dev = torch.device("cuda", device)
    return (torch.tensor(np.ascontiguousarray(u), dtype=ct, device=dev),
            torch.tensor(np.ascontiguousarray(P), dtype=rt, device=dev))


def convergence_history(solution, num_steps: int = 20, num_iters: int = 5, device: int = 0):
    """Chemical potentials and damping integrals after each of num_steps continuations of
    num_iters steps from the solution's state (the loop of tools/check.py:33-37)."""
    from . import device as ndev
    model = solution.getModel()
    u, P = _device_state(solution, device)
    kw = dict(order=model.getApproximationOrder(), dt=model.getTimeStep(), dx=model.getSpatialStep(),
              coeffs=model.getCoefficients())
    eig = np.zeros(num_steps, dtype=complex)
    integrals = np.zeros(num_steps)
    for i in range(num_steps):
        ndev.solve_(u, P, iters=num_iters, **kw)
        mu = ndev.chemical_potential(u, P, dx=kw["dx"], coeffs=kw["coeffs"])
        # the 2-D reference routine returns the real part only (nls/nls.f90:950-971)
        eig[i] = mu if u.dim() == 1 else complex(mu.real, 0.0)
        integrals[i] = ndev.damping_integral(u, P, dx=kw["dx"], coeffs=kw["coeffs"])
    return {"eigenvalues": eig, "integrals": integrals, "mean": float(np.mean(eig.real)),
            "std": float(np.std(eig)), "state": u}


def check_convergence(solution, num_steps: int = 20, num_iters: int = 5, tolerance: float = TOLERANCE,
                      device: int = 0) -> bool:
    """True when the chemical potential has stabilised: std of the num_steps values < tolerance."""
    return convergence_history(solution, num_steps, num_iters, device)["std"] < tolerance


def damping_integral(solution, device: int = 0) -> float:
    """Solution.getDampingIntegral of the solution's state, reduced in FP64 on the GPU."""
    from . import device as ndev
    model = solution.getModel()
    u, P = _device_state(solution, device)
    return ndev.damping_integral(u, P, dx=model.getSpatialStep(), coeffs=model.getCoefficients())


def check_integral(solution, tolerance: float = TOLERANCE, device: int = 0) -> bool:
    """True when |damping integral| <= tolerance."""
    return abs(damping_integral(solution, device)) <= tolerance


__all__ = ["TOLERANCE", "convergence_history", "check_convergence", "damping_integral", "check_integral"]
