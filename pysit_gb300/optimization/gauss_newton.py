"""Gauss-Newton with a Krylov inner solve (mirror of pysit.optimization.GaussNewton,
pysit/optimization/gauss_newton.py:15-85).

Each iteration solves H d = -g with GMRES (``krylov.gmres``, pyamg's convention, one
cycle of up to ``krylov_maxiter`` iterations) where H v is
``objective.apply_hessian(shots, m0, v, **objective_arguments)`` - on the GPU the batched
Gauss-Newton Hessian of all shots in one plan call per Krylov iteration - then takes a
line-search step along d with alpha0 = 1.

Deviation: the reference's matvec builds ``m0.perturbation(data=x)`` but passes the raw
array to apply_hessian (:57-60), whose Born modelling then calls ``with_padding`` on it;
here the perturbation is passed.
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

    def _select_step(self, shots, current_objective_value, gradient, iteration, objective_arguments, **kwargs):
        m0 = self.base_model
        rhs = -1 * np.asarray(gradient.asarray(), dtype=float).reshape(-1)

        def matvec(x):
            m1 = m0.perturbation(data=np.asarray(x, dtype=float).reshape(-1, 1))
            h = self.objective_function.apply_hessian(shots, self.base_model, m1, **objective_arguments)
            return np.asarray(h.data, dtype=float).reshape(-1)

        resid = []
        d, info = gmres(matvec, rhs, maxiter=self.krylov_maxiter, residuals=resid)
        self.krylov_residuals = list(resid)  # ||H d - (-g)|| per Krylov iteration, last outer iteration
        direction = m0.perturbation(data=d.reshape(-1, 1))
        if info < 0:
            self._print("CG Failure")
        if info == 0:
            self._print("CG Converge")
        if info > 0:
            self._print("CG ran {0} iterations".format(info))

        alpha = self.select_alpha(shots, gradient, direction, objective_arguments,
                                  current_objective_value=current_objective_value,
                                  alpha0_kwargs={"reset": iteration == 0}, **kwargs)
        self._print("  alpha {0}".format(alpha))
        self.store_history("alpha", iteration, alpha)
        return alpha * direction

    def _compute_alpha0(self, phi0, grad0, reset=False, upscale_factor=None, **kwargs):
        return 1.0
