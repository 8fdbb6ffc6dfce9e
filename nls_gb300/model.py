"""Problem / Model / Solution API (reference: nls/model.py, Python 3, GPU-backed).

The contract kept from the reference (nls/model.py:27-380, 500-532):

* ``Problem().model(**kwargs)`` returns a ``Model1D`` (radial grid, ``solve_nls``) for
  ``model`` in {"1d", "default"} and a ``Model2D`` (square grid, ``solve_nls_2d``) for "2d", or
  restores one from a ``.mat`` file (``filename=``); omitted keywords take the defaults of
  ``MODEL_DEFAULTS`` and the physical parameters of ``DEFAULT_ORIGINALS``;
* ``model.solve(num_iters)`` advances the initial state on the GPU and returns a ``Solution``;
* the dimensionless coefficient vector (23 slots, slot k-1 = the Fortran ``coeffs(k)``) follows
  from the physical parameters by ``dimensionless_coefficients``;
* the pump is evaluated on ``pump_grid``: ``linspace(0, n dx, n)`` in 1-D and the square mesh of
  ``linspace(-n dx/2, n dx/2, n)`` in 2-D, i.e. with spacing n dx/(n-1) while the Laplacian uses dx;
* a ``Solution`` derives the density |psi|^2, the adiabatic reservoir
  n = c12 P / (c13 + c14 |psi|^2) and its damping integral (rectangle rule, radial weight
  2 pi r dx in 1-D);
* ``store``/``restore`` read and write the reference's ``.mat`` keys through scipy.io.

Plotting (``visualize*``, nls/model.py:391-495) is not provided.
"""

from __future__ import annotations

from datetime import datetime
from types import FunctionType

import numpy as np
from scipy.integrate import simpson
from scipy.io import loadmat, savemat

from .pumping import GaussianPumping, GridPumping
from .solver import Solver1D, Solver2D

# Physical parameters of the reference's default problem (R, gamma, g, tilde g, gamma_R).
DEFAULT_ORIGINALS = {
    "R": 0.0242057488654,
    "gamma": 0.0242057488654,
    "g": 0.00162178517398,
    "tilde_g": 0.0169440242057,
    "gamma_R": 0.242057488654,
}

# Keyword defaults of each model kind; "pumping" is made fresh per model.
MODEL_DEFAULTS = {
    "1d": {"dx": 1.0e-1, "dt": 1.0e-3, "t0": 0.0, "u0": 1.0e-1, "order": 5, "num_nodes": 1000,
           "num_iters": 100000},
    "2d": {"dx": 1.0e-1, "dt": 1.0e-3, "t0": 0.0, "u0": 1.0e-1, "order": 3, "num_nodes": 40,
           "num_iters": 1000},
}


def characteristic_scales(originals) -> dict:
    """Field, time, density and length scales of the dimensionless equation."""
    hbar, m_e = 6.61e-34, 9.1e-31
    m_0 = 1.0e-5 * m_e
    phi = np.sqrt(originals["gamma"] / (2.0 * originals["g"]))
    t = phi
    return {"x": np.sqrt(hbar * t / (2 * m_0)), "t": t, "n": 2.0 / (originals["R"] * t), "phi": phi}


def dimensionless_coefficients(originals) -> np.ndarray:
    """The 23-slot coefficient vector: unit coefficients of the time derivative, Laplacian, gain
    and loss and nonlinearity (slots 1-5), the reservoir coupling 4 tilde g / R (slot 6), and the
    reservoir's pump, decay and saturation factors (slots 12-14); the other slots are zero."""
    sc = characteristic_scales(originals)
    c = np.zeros(23)
    c[0:5] = 1.0
    c[5] = 4.0 * originals["tilde_g"] / originals["R"]
    c[11] = 1.0 / (sc["n"] * originals["gamma_R"])
    c[12] = 1.0
    c[13] = originals["R"] * sc["phi"] ** 2 / originals["gamma_R"]
    return c


def pump_grid(num_nodes: int, dx: float, dim: int):
    """Coordinates the pump is evaluated on (see the module docstring)."""
    if dim == 1:
        return np.meshgrid(np.linspace(0.0, num_nodes * dx, num_nodes))
    half = num_nodes * dx / 2
    axis = np.linspace(-half, half, num_nodes)
    return np.meshgrid(axis, axis)


def damping_weights(num_nodes: int, dx: float, dim: int):
    """Quadrature weights of the damping integral: 2 pi r dx on the 1-D pump grid, dx^2 in 2-D."""
    if dim == 1:
        return 2 * np.pi * np.linspace(0, num_nodes * dx, num_nodes) * dx
    return dx ** 2


class Problem:
    """Factory of models."""

    def model(self, *args, **kwargs):
        if "filename" in kwargs:
            return self.modelFromFile(kwargs["filename"])
        kwargs.pop("params", None)
        kind = kwargs.get("model", "default")
        kwargs["model"] = kind
        kwargs["original_params"] = {**DEFAULT_ORIGINALS, **dict(kwargs.get("original_params") or {})}
        if kind in ("1d", "default", str(Model1D)):
            return self.fabricateModel1D(*args, **kwargs)
        if kind in ("2d", str(Model2D)):
            return self.fabricateModel2D(*args, **kwargs)
        raise ValueError("Unknown model passed!")

    def modelFromFile(self, filename):
        kind = str(np.ravel(loadmat(filename)["model"])[0])
        two_d = "Model2D" in kind or kind == "2d"
        return self.model(model="2d" if two_d else "1d").restore(filename)

    @staticmethod
    def _with_defaults(kind: str, kwargs: dict) -> dict:
        for key, value in MODEL_DEFAULTS[kind].items():
            kwargs.setdefault(key, value)
        kwargs.setdefault("pumping", GaussianPumping())
        return kwargs

    def fabricateModel1D(self, *args, **kwargs):
        kw = self._with_defaults("1d", kwargs)
        n, u0 = kw["num_nodes"], kw["u0"]
        if isinstance(u0, (int, float, complex)):
            kw["u0"] = u0 * np.ones(n)                       # a constant initial state
        elif isinstance(u0, FunctionType):
            kw["u0"] = u0(np.linspace(0.0, kw["dx"] * n, n))  # a profile of the radius
        return Model1D(**kw)

    def fabricateModel2D(self, *args, **kwargs):
        kw = self._with_defaults("2d", kwargs)
        n, u0 = kw["num_nodes"], kw["u0"]
        if isinstance(u0, (int, float, complex)):
            kw["u0"] = u0 * np.ones((n, n))
        return Model2D(**kw)


class AbstractModel:
    """State of one problem: steps, grid, pump, initial state and the coefficient vector."""

    def __init__(self, *args, **kwargs):
        self.dt = kwargs["dt"]
        self.dx = kwargs["dx"]
        self.order = kwargs["order"]
        self.num_nodes = kwargs["num_nodes"]
        self.num_iters = kwargs["num_iters"]
        self.pumping = kwargs["pumping"]
        self.init_sol = kwargs["u0"]
        self.originals = kwargs["original_params"]
        self.coeffs = dimensionless_coefficients(self.originals)
        self.verbose = bool(kwargs.get("verbose"))
        self.solver = None

    def __repr__(self):
        from pprint import pformat
        fields = {"dt": self.dt, "dx": self.dx, "order": self.order, "num_nodes": self.num_nodes,
                  "num_iters": self.num_iters, "pumping": self.pumping, "originals": self.originals}
        return f"{type(self).__name__}({pformat(fields)})\ncoefficients: {self.coeffs}"

    @property
    def dim(self) -> int:
        return len(np.shape(self.init_sol))

    # -- accessors of the reference API
    def getApproximationOrder(self):
        return self.order

    def getCharacteristicScale(self, scale):
        return characteristic_scales(self.originals).get(scale)

    def getChemicalPotential(self, solution):
        state = solution.getSolution() if isinstance(solution, Solution) else solution
        self.mu = self.solver.chemicalPotential(state)
        return self.mu

    def getCoefficients(self):
        return self.coeffs

    def getInitialSolution(self):
        return self.init_sol

    def getNumberOfIterations(self):
        return self.num_iters

    def getNumberOfNodes(self):
        return self.num_nodes

    def getParticleNumber(self, method="simps"):
        # Simpson's rule over the last axis of |psi|^2 of ``self.solution`` (as the reference)
        return simpson((np.conj(self.solution) * self.solution).real, dx=self.dx)

    def getPumping(self):
        return self.pumping(*pump_grid(self.num_nodes, self.dx, self.dim))

    def getSpatialStep(self):
        return self.dx

    def getSolver(self):
        return self.solver

    def getTimeStep(self):
        return self.dt

    def setNumberOfIterations(self, num_iters):
        self.num_iters = num_iters

    def setPumping(self, pumping):
        self.pumping = pumping

    def setInitialSolution(self, solution):
        self.init_sol = solution

    def solve(self, num_iters=None):
        return self.solver(num_iters)

    # -- the reference's .mat record
    def _mat_record(self, date: str) -> dict:
        return {"model": str(type(self)), "date": date, "dim": self.dim, "dimlesses": self.coeffs,
                "init_solution": self.init_sol, "num_iters": self.num_iters, "num_nodes": self.num_nodes,
                "order": self.order, "originals": self.originals, "pumping": self.getPumping(),
                "spatial_step": self.dx, "time_step": self.dt}

    def store(self, filename=None, label=None, desc=None, date=None):
        date = date if date else datetime.now()
        date = date.replace(microsecond=0).isoformat() if isinstance(date, datetime) else str(date)
        record = self._mat_record(date)
        if desc:
            record["desc"] = desc
        if label:
            record["label"] = label
        savemat(filename if filename else date + ".mat", record)

    def restore(self, filename):
        mat = loadmat(filename)
        scalar = lambda key, kind: kind(np.ravel(mat[key])[0])  # noqa: E731
        one_d = scalar("dim", int) == 1
        self.coeffs = mat["dimlesses"][0, :]
        self.init_sol = mat["init_solution"][0, :] if one_d else mat["init_solution"]
        self.pumping = GridPumping(mat["pumping"][0, :] if one_d else mat["pumping"])
        self.num_nodes = scalar("num_nodes", int)
        self.num_iters = scalar("num_iters", int)
        self.dx = scalar("spatial_step", float)
        self.dt = scalar("time_step", float)
        self.order = scalar("order", int)
        originals = mat["originals"][0, 0]
        self.originals = {name: float(np.ravel(originals[name])[0]) for name in originals.dtype.names}
        if "desc" in mat:
            self.desc = str(mat["desc"][0])
        if "label" in mat:
            self.label = str(mat["label"][0])
        return self


class Model1D(AbstractModel):
    """Radially symmetric model (solve_nls)."""

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.solver = Solver1D(self)


class Model2D(AbstractModel):
    """Square-grid model (solve_nls_2d)."""

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.solver = Solver2D(self)


class Solution:
    """A solved state with the model that produced it."""

    def __init__(self, model, solution=None, verbose=False):
        self.elapsed_time = 0.0
        self.model = model
        self.solution = solution
        self.verbose = verbose

    def getDampingIntegral(self):
        """Rectangle-rule integral of (n - 1) |psi|^2 with the weights of ``damping_weights``."""
        m = self.model
        weights = damping_weights(m.getNumberOfNodes(), m.getSpatialStep(), np.ndim(self.solution))
        return np.sum((self.getReservoir() - 1.0) * self.getDensity() * weights)

    def getDensity(self):
        return (np.conj(self.solution) * self.solution).real

    def getElapsedTime(self):
        return self.elapsed_time

    def getModel(self):
        return self.model

    def getReservoir(self):
        c = self.model.coeffs
        return c[11] * self.model.getPumping() / (c[12] + c[13] * self.getDensity())

    def getSolution(self):
        return self.solution

    def setElapsedTime(self, seconds):
        self.elapsed_time = seconds

    def setSolution(self, solution):
        self.solution = solution

    def store(self, filename=None, label=None, desc=None, date=None):
        from .native import nls
        date = datetime.now() if date is None else date
        filename = filename if filename else date.replace(microsecond=0).isoformat() + ".mat"
        self.model.store(filename, label, desc, date)
        record = {k: v for k, v in loadmat(filename).items() if not k.startswith("__")}
        record.update({"elapsed_time": self.elapsed_time, "solution": self.solution,
                       "version": np.array(nls.version())})
        savemat(filename, record)

    def restore(self, filename):
        mat = loadmat(filename)
        one_d = int(np.ravel(mat["dim"])[0]) == 1
        self.solution = mat["solution"][0, :] if one_d else mat["solution"]
        self.elapsed_time = float(mat["elapsed_time"][0, 0])
        return self

    def report(self):
        m = self.model
        print(f"Elapsed in {self.elapsed_time} seconds with {m.getNumberOfIterations()} iteration "
              f"on {m.getNumberOfNodes()} grid nodes.")


__all__ = ["Problem", "AbstractModel", "Model1D", "Model2D", "Solution", "DEFAULT_ORIGINALS", "MODEL_DEFAULTS",
           "characteristic_scales", "dimensionless_coefficients", "pump_grid", "damping_weights"]
