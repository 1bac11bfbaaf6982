"""Optimizers over the GPU objective (mirror of pysit.optimization): LBFGS,
GradientDescent and GaussNewton with the reference's histories and line searches."""
from .optimization import OptimizationBase  # noqa: F401
from .lbfgs import LBFGS  # noqa: F401
from .gradient_descent import GradientDescent  # noqa: F401
from .gauss_newton import GaussNewton  # noqa: F401
from . import krylov  # noqa: F401

__all__ = ["OptimizationBase", "LBFGS", "GradientDescent", "GaussNewton", "krylov"]
