"""Gauss-Newton with PySIT's interface (pysit/optimization/gauss_newton.py:15-85).

The direction d solves the Gauss-Newton system H d = -g approximately with GMRES
(``krylov.gmres``: one cycle of at most ``krylov_maxiter`` iterations), where H v is
``objective.apply_hessian(shots, m0, v)`` - on the GPU the batched Hessian of all shots,
one plan call per Krylov iteration.  The line search starts from the full Newton step
(length 1).  ``krylov_residuals`` holds |H d - (-g)| per Krylov iteration of the last
iteration.

Difference from the reference: its Hessian product passes the raw Krylov vector to
apply_hessian, whose Born modelling needs a model perturbation (:57-60); here the vector
is wrapped as one.
"""
from __future__ import annotations

import numpy as np

from .krylov import gmres
from .optimization import OptimizationBase

__all__ = ["GaussNewton"]


class GaussNewton(OptimizationBase):

    def __init__(self, objective, krylov_maxiter=50, *args, **kwargs):
        super().__init__(objective, *args, **kwargs)
        self.krylov_maxiter = krylov_maxiter
        self.krylov_residuals = []

    def search_direction(self, shots, gradient, iteration, objective_arguments):
        m0 = self.base_model

        def hessian_times(v):
            h = self.objective_function.apply_hessian(shots, m0, m0.perturbation(data=np.reshape(v, (-1, 1))),
                                                      **objective_arguments)
            return np.asarray(h.data, dtype=float).reshape(-1)

        rhs = -np.asarray(gradient.asarray(), dtype=float).reshape(-1)
        residuals = []
        d, info = gmres(hessian_times, rhs, maxiter=self.krylov_maxiter, residuals=residuals)
        self.krylov_residuals = residuals
        outcome = "converged" if info == 0 else ("broke down" if info < 0 else f"stopped after {info} iterations")
        self._log(f"  Krylov solve {outcome}, residual {residuals[-1] if residuals else None}")
        return m0.perturbation(data=d.reshape(-1, 1))

    def trial_length(self, value, gradient, iteration):
        return 1.0
