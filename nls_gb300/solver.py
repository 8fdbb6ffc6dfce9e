"""Solver facade over the GPU module object (reference: nls/solver.py:13-83).

``AbstractSolver.__call__(num_iters)`` times the native call on the wall clock and wraps the
result in a ``Solution``; ``Solver1D`` calls ``nls.solve_nls`` and ``Solver2D`` calls
``nls.solve_nls_2d``, with the reference's argument order
``(dt, dx, order, iters, pumping, coeffs, u0)``.
"""

from __future__ import annotations

from time import time

from .native import nls


class AbstractSolver:
    def __init__(self, model):
        self.model = model
        self.elapsed_time = 0.0

    def __call__(self, num_iters=None):
        from .model import Solution

        if num_iters:
            self.model.setNumberOfIterations(num_iters)
        self.elapsed_time = -time()
        self.solution = Solution(self.model)
        self.solution.setSolution(self.solve(
            self.model.getTimeStep(),
            self.model.getSpatialStep(),
            self.model.getApproximationOrder(),
            self.model.getNumberOfIterations(),
            self.model.getPumping(),
            self.model.getCoefficients(),
            self.model.getInitialSolution()))
        self.elapsed_time += time()
        self.solution.setElapsedTime(self.elapsed_time)
        return self.solution

    def solve(self, *args, **kwargs):
        raise NotImplementedError("AbstractSolver: native solver routine is not passed!")

    def chemicalPotential(self, solution, *args, **kwargs):
        return self.chemicalPotentialRoutine(
            self.model.getSpatialStep(),
            self.model.getPumping(),
            self.model.getCoefficients(),
            solution)

    def chemicalPotentialRoutine(self, *args, **kwargs):
        raise NotImplementedError("AbstractSolver: native solver routine is not passed!")


class Solver1D(AbstractSolver):
    def solve(self, *args, **kwargs):
        return nls.solve_nls(*args, **kwargs)

    def chemicalPotentialRoutine(self, *args, **kwargs):
        return nls.chemical_potential_1d(*args, **kwargs)


class Solver2D(AbstractSolver):
    def solve(self, *args, **kwargs):
        return nls.solve_nls_2d(*args, **kwargs)

    def chemicalPotentialRoutine(self, *args, **kwargs):
        return nls.chemical_potential_2d(*args, **kwargs)


__all__ = ["AbstractSolver", "Solver1D", "Solver2D"]
