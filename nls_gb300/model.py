"""Problem / Model / Solution API (reference: nls/model.py, Python 3, GPU-backed).

``Problem().model(**kwargs)`` builds a ``Model1D`` (radial, solve_nls) or ``Model2D``
(Cartesian, solve_nls_2d) with the reference's defaults (nls/model.py:32-117), coefficient
vector (:125-160) and pump-grid convention (:220-232); ``model.solve(num_iters)`` returns a
``Solution`` (:252-255, 337-536).  Conventions kept on purpose:

* the pump is evaluated on ``linspace(0, n*dx, n)`` in 1-D and on
  ``meshgrid(linspace(-n*dx/2, n*dx/2, n))`` in 2-D, i.e. with spacing n*dx/(n-1), while the
  Laplacian uses dx;
* ``coeffs`` is the 23-slot vector with 0-based index = Fortran index - 1;
* ``Solution.getReservoir`` recomputes n = c12 P / (c13 + c14 |psi|^2) from the final state.

Plotting (``visualize*``, nls/model.py:391-495) is not provided.  ``store``/``restore`` write and
read the reference's .mat layout (nls/model.py:257-314, 500-532) through scipy.io.
"""

from __future__ import annotations

from datetime import datetime
from types import FunctionType

import numpy as np
from scipy.integrate import simpson
from scipy.io import loadmat, savemat

from .pumping import GaussianPumping, GridPumping
from .solver import Solver1D, Solver2D

_DEFAULT_ORIGINALS = {
    "R": 0.0242057488654,
    "gamma": 0.0242057488654,
    "g": 0.00162178517398,
    "tilde_g": 0.0169440242057,
    "gamma_R": 0.242057488654,
}


class Problem:
    """Factory of models (nls/model.py:27-117)."""

    def model(self, *args, **kwargs):
        if "filename" in kwargs:
            return self.modelFromFile(kwargs["filename"])
        kwargs.pop("params", None)
        kwargs["model"] = kwargs.get("model", "default")
        originals = dict(kwargs.get("original_params") or {})
        for k, v in _DEFAULT_ORIGINALS.items():
            originals.setdefault(k, v)
        kwargs["original_params"] = originals
        if kwargs["model"] in ("1d", "default", str(Model1D)):
            return self.fabricateModel1D(*args, **kwargs)
        if kwargs["model"] in ("2d", str(Model2D)):
            return self.fabricateModel2D(*args, **kwargs)
        raise ValueError("Unknown model passed!")

    def modelFromFile(self, filename):
        mat = loadmat(filename)
        kind = str(np.ravel(mat["model"])[0])
        model = self.model(model="2d" if "Model2D" in kind or kind == "2d" else "1d")
        return model.restore(filename)

    def fabricateModel1D(self, *args, **kwargs):
        kwargs.setdefault("dx", 1.0e-1)
        kwargs.setdefault("dt", 1.0e-3)
        kwargs.setdefault("t0", 0.0)
        kwargs.setdefault("u0", 1.0e-1)
        kwargs.setdefault("order", 5)
        kwargs.setdefault("pumping", GaussianPumping())
        kwargs.setdefault("num_nodes", 1000)
        kwargs.setdefault("num_iters", 100000)
        if isinstance(kwargs["u0"], (int, float, complex)):
            kwargs["u0"] = kwargs["u0"] * np.ones(kwargs["num_nodes"])
        elif isinstance(kwargs["u0"], FunctionType):
            grid = np.linspace(0.0, kwargs["dx"] * kwargs["num_nodes"], kwargs["num_nodes"])
            kwargs["u0"] = kwargs["u0"](grid)
        return Model1D(**kwargs)

    def fabricateModel2D(self, *args, **kwargs):
        kwargs.setdefault("dx", 1.0e-1)
        kwargs.setdefault("dt", 1.0e-3)
        kwargs.setdefault("t0", 0.0)
        kwargs.setdefault("u0", 1.0e-1)
        kwargs.setdefault("order", 3)
        kwargs.setdefault("pumping", GaussianPumping())
        kwargs.setdefault("num_nodes", 40)
        kwargs.setdefault("num_iters", 1000)
        if isinstance(kwargs["u0"], (int, float, complex)):
            kwargs["u0"] = kwargs["u0"] * np.ones((kwargs["num_nodes"], kwargs["num_nodes"]))
        return Model2D(**kwargs)


class AbstractModel:
    """Shared model state: steps, grid, pump, initial state and the coefficient vector."""

    def __init__(self, *args, **kwargs):
        self.dt = kwargs["dt"]
        self.dx = kwargs["dx"]
        self.order = kwargs["order"]
        self.num_nodes = kwargs["num_nodes"]
        self.num_iters = kwargs["num_iters"]
        self.pumping = kwargs["pumping"]
        self.init_sol = kwargs["u0"]
        self.originals = kwargs["original_params"]
        self.coeffs = np.zeros(23)
        self.verbose = bool(kwargs.get("verbose"))
        self.solver = None
        o = self.originals
        phi0 = np.sqrt(o["gamma"] / (2.0 * o["g"]))
        t0 = phi0
        n0 = 2.0 / (o["R"] * t0)
        # equation coefficients (nls/model.py:147-160); slot k-1 holds Fortran coeffs(k)
        self.coeffs[0] = 1.0
        self.coeffs[1] = 1.0
        self.coeffs[2] = 1.0
        self.coeffs[3] = 1.0
        self.coeffs[4] = 1.0
        self.coeffs[5] = 4.0 * o["tilde_g"] / o["R"]
        self.coeffs[10] = 0.0
        self.coeffs[11] = 1.0 / (n0 * o["gamma_R"])
        self.coeffs[12] = 1.0
        self.coeffs[13] = o["R"] * phi0 ** 2 / o["gamma_R"]
        self.coeffs[14] = 0.0

    def __repr__(self):
        from pprint import pformat
        return pformat({"dt": self.dt, "dx": self.dx, "order": self.order, "num_nodes": self.num_nodes,
                        "num_iters": self.num_iters, "pumping": self.pumping,
                        "originals": self.originals}) + "\n" + str(self.coeffs)

    def getApproximationOrder(self):
        return self.order

    def getCharacteristicScale(self, scale):
        hbar, m_e = 6.61e-34, 9.1e-31
        m_0 = 1.0e-5 * m_e
        o = self.originals
        phi0 = np.sqrt(o["gamma"] / (2.0 * o["g"]))
        t0 = phi0
        x0 = np.sqrt(hbar * t0 / (2 * m_0))
        n0 = 2.0 / (o["R"] * t0)
        return {"x": x0, "t": t0, "n": n0, "phi": phi0}.get(scale)

    def getChemicalPotential(self, solution):
        if isinstance(solution, Solution):
            solution = solution.getSolution()
        self.mu = self.solver.chemicalPotential(solution)
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
        return simpson((self.solution.conj() * self.solution).real, dx=self.dx)

    def getPumping(self):
        if len(np.shape(self.init_sol)) == 1:
            x = np.linspace(0.0, self.num_nodes * self.dx, self.num_nodes)
            return self.pumping(*np.meshgrid(x))
        right = self.num_nodes * self.dx / 2
        x = np.linspace(-right, right, self.num_nodes)
        return self.pumping(*np.meshgrid(x, x))

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

    def store(self, filename=None, label=None, desc=None, date=None):
        date = date if date else datetime.now()
        date = date.replace(microsecond=0).isoformat() if isinstance(date, datetime) else str(date)
        filename = filename if filename else date + ".mat"
        mat = {
            "model": str(type(self)),
            "date": date,
            "dim": len(np.shape(self.init_sol)),
            "dimlesses": self.coeffs,
            "init_solution": self.init_sol,
            "num_iters": self.num_iters,
            "num_nodes": self.num_nodes,
            "order": self.order,
            "originals": self.originals,
            "pumping": self.getPumping(),
            "spatial_step": self.dx,
            "time_step": self.dt,
        }
        if desc:
            mat["desc"] = desc
        if label:
            mat["label"] = label
        savemat(filename, mat)

    def restore(self, filename):
        mat = loadmat(filename)
        originals = mat["originals"][0, 0]
        if int(np.ravel(mat["dim"])[0]) == 1:
            mat["init_solution"] = mat["init_solution"][0, :]
            mat["pumping"] = mat["pumping"][0, :]
        self.coeffs = mat["dimlesses"][0, :]
        self.init_sol = mat["init_solution"]
        self.num_nodes = int(mat["num_nodes"][0, 0])
        self.num_iters = int(mat["num_iters"][0, 0])
        self.pumping = GridPumping(mat["pumping"])
        self.dx = float(mat["spatial_step"][0, 0])
        self.dt = float(mat["time_step"][0, 0])
        self.order = int(mat["order"][0, 0])
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
    """A solved state plus the model that produced it (nls/model.py:337-536)."""

    def __init__(self, model, solution=None, verbose=False):
        self.elapsed_time = 0.0
        self.model = model
        self.solution = solution
        self.verbose = verbose

    def getDampingIntegral(self):
        """Rectangle-rule integral of (n - 1) |psi|^2 (nls/model.py:350-365)."""
        reservoir = self.getReservoir()
        density = self.getDensity()
        length = self.model.getSpatialStep()
        if self.solution.ndim == 1:
            nodes = self.model.getNumberOfNodes()
            radius = np.linspace(0, nodes * length, nodes)
            return 2 * np.pi * np.sum((reservoir - 1.0) * density * radius * length)
        return np.sum((reservoir - 1.0) * density * length ** 2)

    def getDensity(self):
        return (self.solution.conj() * self.solution).real

    def getElapsedTime(self):
        return self.elapsed_time

    def getModel(self):
        return self.model

    def getReservoir(self):
        p = self.model.getPumping()
        u = self.getDensity()
        c = self.model.coeffs
        return c[11] * p / (c[12] + c[13] * u)

    def getSolution(self):
        return self.solution

    def setElapsedTime(self, seconds):
        self.elapsed_time = seconds

    def setSolution(self, solution):
        self.solution = solution

    def store(self, filename=None, label=None, desc=None, date=None):
        date = datetime.now() if date is None else date
        filename = filename if filename else date.replace(microsecond=0).isoformat() + ".mat"
        from .native import nls
        self.model.store(filename, label, desc, date)
        content = loadmat(filename)
        content = {k: v for k, v in content.items() if not k.startswith("__")}
        content.update({"elapsed_time": self.elapsed_time, "solution": self.solution,
                        "version": np.array(nls.version())})
        savemat(filename, content)

    def restore(self, filename):
        mat = loadmat(filename)
        sol = mat["solution"]
        if int(np.ravel(mat["dim"])[0]) == 1:
            sol = sol[0, :]
        self.elapsed_time = float(mat["elapsed_time"][0, 0])
        self.solution = sol
        return self

    def report(self):
        msg = "Elapsed in {0} seconds with {1} iteration on {2} grid nodes."
        print(msg.format(self.elapsed_time, self.model.getNumberOfIterations(), self.model.getNumberOfNodes()))


__all__ = ["Problem", "AbstractModel", "Model1D", "Model2D", "Solution"]
