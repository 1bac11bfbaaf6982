"""Physical domain and boundary conditions (mirror of pysit.core.domain).

Same public names and argument meaning as the reference:
``RectangularDomain(*axis_configs)`` with one ``(lbound, rbound, lbc, rbc[, unit])``
tuple per axis (pysit/core/domain.py:36-134), and the boundary conditions
``Dirichlet()`` and ``PML(length, amplitude, ftype='quadratic', boundary='dirichlet',
compact=False)`` (pysit/core/domain.py:154-254).  Axes are ordered (x, [y,] z)
with z last, 1D is z only.
"""
from __future__ import annotations

import numpy as np

__all__ = ["RectangularDomain", "DomainBC", "Dirichlet", "PML", "Bunch"]

_AXES = {1: ["z"], 2: ["x", "z"], 3: ["x", "y", "z"]}


class Bunch(dict):
    """dict with attribute access."""

    def __init__(self, **kw):
        super().__init__(**kw)
        self.__dict__ = self


class DomainBC:
    type = None


class Dirichlet(DomainBC):
    """Homogeneous Dirichlet boundary."""
    type = "dirichlet"


class PML(DomainBC):
    """Perfectly matched layer of physical width ``length`` and profile scale
    ``amplitude``; profile ``amplitude * f(x)`` on [0, 1] with f(x) = x**2
    ('quadratic') or a cubic b-spline ('b-spline') (pysit/core/domain.py:203-254)."""
    type = "pml"

    def __init__(self, length, amplitude, ftype="quadratic", boundary="dirichlet", compact=False):
        self.length = length
        self.amplitude = amplitude
        self.compact = compact
        self.ftype = ftype
        if ftype == "quadratic":
            self.pml_func = self._quadratic
        elif ftype == "b-spline":
            self.pml_func = self._bspline
        else:
            raise NotImplementedError(f"{ftype} is not a currently defined PML function.")
        if boundary not in ("neumann", "dirichlet"):
            raise ValueError(f"'{boundary}' is not 'neumann' or 'dirichlet'.")
        self.boundary_type = boundary

    @staticmethod
    def _quadratic(x):
        return x ** 2

    @staticmethod
    def _bspline(x):
        x = np.atleast_1d(np.asarray(x, dtype=float)).copy()
        out = np.zeros_like(x)
        lo = x < 0.5
        out[lo] = 1.5 * (8.0 / 6.0) * x[lo] ** 3
        hi = ~lo
        out[hi] = 1.5 * (-4.0 * x[hi] ** 3 + 8.0 * x[hi] ** 2 - 4.0 * x[hi] + 2.0 / 3.0)
        return out

    def evaluate(self, n, orientation="right"):
        """Profile on ``n`` equispaced points of [0, 1], reversed for the left side."""
        val = self.amplitude * self.pml_func(np.linspace(0.0, 1.0, n))
        if orientation == "left":
            val = val[::-1]
        return val


class RectangularDomain:
    """Rectangular domain; ``axis_configs`` = one (lbound, rbound, lbc, rbc[, unit]) per axis."""
    type = "rectangular"

    def __init__(self, *axis_configs):
        if not 1 <= len(axis_configs) <= 3:
            raise ValueError("Domain construction must be between one and three dimensions.")
        self.dim = len(axis_configs)
        self.parameters = {}
        for i, key in enumerate(_AXES[self.dim]):
            cfg = axis_configs[i]
            if len(cfg) == 4:
                L, R, lbc, rbc = cfg
                unit = None
            elif len(cfg) == 5:
                L, R, lbc, rbc, unit = cfg
            else:
                raise ValueError("each axis config is (lbound, rbound, lbc, rbc[, unit])")
            p = Bunch(lbound=float(L), rbound=float(R), lbc=lbc, rbc=rbc, unit=unit)
            p.length = float(R) - float(L)
            self.parameters[i] = p
            self.parameters[key] = p
            setattr(self, key, p)

    def collect(self, prop):
        return tuple(self.parameters[i][prop] for i in range(self.dim))

    def get_lengths(self):
        return self.collect("length")
