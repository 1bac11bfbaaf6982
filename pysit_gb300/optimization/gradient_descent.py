"""Steepest descent with PySIT's interface (pysit/optimization/gradient_descent.py:13-57):
the direction is -g; the line search starts from f / (|g| prod(deltas))^2 at iteration 0
and from the previous accepted length / 0.7 afterwards (a little longer than the last
step, so that the step can grow again)."""
from __future__ import annotations

from .line_search import Backtracking
from .optimization import OptimizationBase

__all__ = ["GradientDescent"]


class GradientDescent(OptimizationBase):

    def search_direction(self, shots, gradient, iteration, objective_arguments):
        return -1 * gradient

    def trial_length(self, value, gradient, iteration):
        if iteration == 0 or self.prev_alpha is None:
            return self._scaled_first_length(value, gradient)
        return self.prev_alpha / Backtracking.trial_growth
