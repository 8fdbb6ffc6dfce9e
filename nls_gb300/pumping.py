"""Pump profiles P(x[, y]) -- host-side producers of the pump array the kernels read.

Same classes, constructor arguments and values as the reference's nls/pumping.py:
    AbstractPumping (:11-40), OpSumPumping (:43-57), OpSubPumping (:60-74), OpMulPumping (:77-92),
    GridPumping (:95-110), GaussianPumping (:113-130), GaussianPumping1D (:133-141),
    GaussianPumping2D (:144-149), GaussianRingPumping1D (:152-159), GaussianRingPumping2D
    (:162-178), GaussianElipticPumping2D (:181-202), RectangularPumping1D (:205-221),
    RectangularRingPumping1D (:224-228).
Reference conventions kept on purpose: ``AbstractPumping.__init__`` ignores its ``power``
argument (so composite pumps multiply by 1.0), and GaussianElipticPumping2D divides by
``2 * variation`` rather than ``2 * variation**2``.
"""

from __future__ import annotations

import numpy as np


class AbstractPumping:
    def __init__(self, power=1.0):
        self.power = 1.0          # the argument is ignored, as in the reference

    def setPower(self, power):
        self.power = power

    def __call__(self, *args, **kwargs):
        raise NotImplementedError("an abstract pumping has no profile")

    def __add__(self, other):
        return OpSumPumping(self, other)

    def __sub__(self, other):
        return OpSubPumping(self, other)

    def __str__(self):
        return repr(self)

    def __repr__(self):
        return "AbstractPumping"


class OpSumPumping(AbstractPumping):
    def __init__(self, lhs, rhs):
        super().__init__()
        self.lhs, self.rhs = lhs, rhs

    def __call__(self, *args, **kwargs):
        return self.power * (self.lhs(*args, **kwargs) + self.rhs(*args, **kwargs))

    def __repr__(self):
        return f"{self.lhs!r} + {self.rhs!r}"


class OpSubPumping(AbstractPumping):
    def __init__(self, lhs, rhs):
        super().__init__()
        self.lhs, self.rhs = lhs, rhs

    def __call__(self, *args, **kwargs):
        return self.power * (self.lhs(*args, **kwargs) - self.rhs(*args, **kwargs))

    def __repr__(self):
        return f"{self.lhs!r} - {self.rhs!r}"


class OpMulPumping(AbstractPumping):
    def __init__(self, lhs, rhs):
        super().__init__()
        self.lhs, self.rhs = lhs, rhs

    def __call__(self, *args, **kwargs):
        raise NotImplementedError("Not supported yet!")

    def __repr__(self):
        return f"{self.lhs!r} x {self.rhs!r}"


class GridPumping(AbstractPumping):
    """A pump given directly on the grid (also what a restored .mat file yields)."""

    def __init__(self, pumping, desciption=None):
        super().__init__()
        self.pumping = pumping
        self.desciption = desciption or "<class GridPumping>"

    def __call__(self, *args, **kwargs):
        return self.pumping

    def __repr__(self):
        return self.desciption


class GaussianPumping(AbstractPumping):
    """power * exp(-((x - x0)^2 + (y - y0)^2) / (2 variation^2))."""

    def __init__(self, power=1.0, x0=0.0, y0=0.0, variation=5.0):
        super().__init__()
        self.power, self.x0, self.y0, self.variation = power, x0, y0, variation

    def __call__(self, x, y, t=None):
        r2 = (x - self.x0) ** 2 + (y - self.y0) ** 2
        return self.power * np.exp(-r2 / (2.0 * self.variation ** 2))

    def __repr__(self):
        return (f"{type(self).__name__}(power={self.power!r}, x0={self.x0!r}, y0={self.y0!r}, "
                f"variation={self.variation!r})")


class GaussianPumping1D(GaussianPumping):
    def __call__(self, x, t=None):
        return GaussianPumping.__call__(self, x, 0.0, t)


class GaussianPumping2D(GaussianPumping):
    pass


class GaussianRingPumping1D(OpSumPumping):
    """Two Gaussians at +radius and -radius (a ring when evaluated on r)."""

    def __init__(self, power=1.0, radius=0.0, variation=5.0):
        super().__init__(GaussianPumping1D(power, +radius, 0.0, variation),
                         GaussianPumping1D(power, -radius, 0.0, variation))


class GaussianRingPumping2D(AbstractPumping):
    def __init__(self, power=1.0, x0=0.0, y0=0.0, variation=5.0, radius=1.0):
        super().__init__()
        self.x0, self.y0 = x0, y0
        self.pumping = GaussianRingPumping1D(power, radius, variation)

    def __call__(self, x, y, t=None):
        r = np.sqrt((x - self.x0) ** 2 + (y - self.y0) ** 2)
        return self.pumping(r, t)

    def __repr__(self):
        g = self.pumping.lhs
        return (f"GaussianRingPumping2D(power={g.power!r}, x0={self.x0!r}, y0={self.y0!r}, "
                f"variation={g.variation!r}, radius={g.x0!r})")


class GaussianElipticPumping2D(AbstractPumping):
    def __init__(self, power=1.0, x0=0.0, y0=0.0, variation=5.0, a=1.0, b=1.0):
        super().__init__(power)
        self.x0, self.y0, self.var, self.a, self.b = x0, y0, variation, a, b

    def __call__(self, x, y, t=None):
        th = np.arctan2(x - self.x0, y - self.y0)
        re = np.sqrt((self.a * np.cos(th)) ** 2 + (self.b * np.sin(th)) ** 2)
        rp = np.sqrt(x ** 2 + y ** 2)
        return self.power * (np.exp(-(re - rp) ** 2 / (2 * self.var)) + np.exp(-(re + rp) ** 2 / (2 * self.var)))

    def __repr__(self):
        return (f"GaussianElipticPumping2D(power={self.power!r}, x0={self.x0!r}, y0={self.y0!r}, "
                f"variation={self.var!r}, a={self.a!r}, b={self.b!r})")


class RectangularPumping1D(AbstractPumping):
    def __init__(self, power=10.0, x0=0.0, width=1.0):
        super().__init__(power)
        self.x0, self.width, self.power = x0, width, power

    def __call__(self, x, t=None):
        x = np.asarray(x)
        out = np.zeros(x.shape)
        out[(x >= self.x0 - self.width / 2.0) & (x <= self.x0 + self.width / 2.0)] = self.power
        return out

    def __repr__(self):
        return f"RectangularPumping1D(power={self.power!r}, x0={self.x0!r}, width={self.width!r})"


class RectangularRingPumping1D(OpSumPumping):
    def __init__(self, power=10.0, radius=10.0, width=2.0):
        super().__init__(RectangularPumping1D(power, +radius, width), RectangularPumping1D(power, -radius, width))


__all__ = [
    "AbstractPumping", "OpSumPumping", "OpSubPumping", "OpMulPumping", "GridPumping",
    "GaussianPumping", "GaussianPumping1D", "GaussianPumping2D", "GaussianRingPumping1D",
    "GaussianRingPumping2D", "GaussianElipticPumping2D", "RectangularPumping1D",
    "RectangularRingPumping1D",
]
