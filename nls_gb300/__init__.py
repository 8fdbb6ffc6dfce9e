"""nls_gb300 -- GB300 (sm_103a) solver for the time-stepping path of daskol/nls.

Public surface, mirroring the reference package `nls`:
    from nls_gb300.native import nls          # the f2py module object (solve_nls, solve_nls_2d, ...)
    from nls_gb300 import Problem             # Problem().model(...).solve()
plus the batched form (nls_gb300.batch) and the serving loop (nls_gb300.serve).
"""

from .model import AbstractModel, Model1D, Model2D, Problem, Solution
from .pumping import *  # noqa: F401,F403
from .pumping import __all__ as _pumping_all

__version__ = "0.2.0"


def version():
    """(major, minor, patch) of the reference interface this build mirrors (nls/version.py)."""
    return (0, 2, 0)


__all__ = ["Problem", "AbstractModel", "Model1D", "Model2D", "Solution", "version"] + list(_pumping_all)
