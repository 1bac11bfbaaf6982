"""Steepest descent with a line search (mirror of pysit.optimization.GradientDescent,
pysit/optimization/gradient_descent.py:13-57): direction -g; the backtracking line
search starts from f / (|g| * prod(deltas))**2 on the first iteration and from the
previous step length / 0.7 afterwards."""
from __future__ import annotations

import numpy as np

from .optimization import OptimizationBase

__all__ = ["GradientDescent"]


class GradientDescent(OptimizationBase):

    def __init__(self, objective, *args, **kwargs):
        super().__init__(objective, *args, **kwargs)
        self.prev_alpha = None

    def _select_step(self, shots, current_objective_value, gradient, iteration, objective_arguments, **kwargs):
        direction = -1 * gradient
        alpha = self.select_alpha(shots, gradient, direction, objective_arguments,
                                  current_objective_value=current_objective_value,
                                  alpha0_kwargs={"reset": iteration == 0}, **kwargs)
        self._print("  alpha {0}".format(alpha))
        self.store_history("alpha", iteration, alpha)
        return alpha * direction

    def _compute_alpha0(self, phi0, grad0, reset=False, upscale_factor=None, **kwargs):
        if reset or self.prev_alpha is None:
            return phi0 / (grad0.norm() * np.prod(self.solver.mesh.deltas)) ** 2
        return self.prev_alpha / upscale_factor
