"""Precision form: a complex64 solve with FP64 diagnostics, checked against a complex128 run.

Stencil and pointwise work run in complex64 on the fused kernels.  Every ``log_every`` steps the
state's FP64 norm (sum |psi|^2 dx^2) and FP64 chemical potential (the reference's
chemical_potential_1d/2d diagnostic, nls/nls.f90:921-971, evaluated on the device state) are
logged with the simulated time accumulated in FP64 (t = steps * dt).  At the end the same problem
is solved on the plain complex128 path and the relative L2 errors of |psi|^2 and of the reservoir
n = c12 P / (c13 + c14 |psi|^2) are reduced in FP64 on the device.
"""

from __future__ import annotations

import time

import numpy as np
import torch

from . import device as ndev


def _tensors(spec, dtype, dev):
    ct = torch.complex64 if dtype == np.complex64 else torch.complex128
    rt = torch.float32 if dtype == np.complex64 else torch.float64
    # memory with the reference's Fortran first index contiguous (as nls.native passes it)
    u0 = np.asarray(spec.u0).T if spec.dim == 2 else np.asarray(spec.u0)
    P = np.asarray(spec.pumping).T if spec.dim == 2 else np.asarray(spec.pumping)
    u = torch.tensor(np.ascontiguousarray(u0), dtype=ct, device=dev)
    Pt = torch.tensor(np.ascontiguousarray(P), dtype=rt, device=dev)
    return u, Pt


def run(spec, steps: int, log_every: int = 500, reference: bool = True, device: int = 0, variant: int = -1):
    dev = torch.device("cuda", device)
    u, P = _tensors(spec, np.complex64, dev)
    cell = spec.dx ** spec.dim
    kw = dict(order=spec.order, dt=spec.dt, dx=spec.dx, coeffs=spec.coeffs)
    log = []
    solve_s = 0.0
    done = 0
    while done < steps:
        chunk = min(log_every, steps - done)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        ndev.solve_(u, P, iters=chunk, variant=variant, **kw)
        torch.cuda.synchronize(dev)
        solve_s += time.perf_counter() - t0
        done += chunk
        norm = ndev.norm(u) * cell
        mu = ndev.chemical_potential(u, P, dx=spec.dx, coeffs=spec.coeffs)
        log.append({"step": done, "t": done * float(spec.dt), "norm": norm, "mu": mu.real})
    out = {"steps": steps, "log": log, "c64_seconds": solve_s,
           "c64_node_steps_per_s": float(spec.nodes) * steps / solve_s}
    if reference:
        u64, P64 = _tensors(spec, np.complex128, dev)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        ndev.solve_(u64, P64, iters=steps, **kw)
        torch.cuda.synchronize(dev)
        out["c128_seconds"] = time.perf_counter() - t0
        out["c128_node_steps_per_s"] = float(spec.nodes) * steps / out["c128_seconds"]
        d, r = ndev.density_errors(u, u64, P64, spec.coeffs)
        out["rel_l2_density"] = d
        out["rel_l2_reservoir"] = r
    out["state"] = u
    return out
