"""Limited-memory BFGS with PySIT's interface (pysit/optimization/lbfgs.py:13-124).

The direction is -H_k g_k with H_k the L-BFGS inverse-Hessian approximation applied by the
two-loop recursion of Nocedal & Wright (Numerical Optimization, 2nd ed., Algorithm 7.4):
over the m newest curvature pairs (s_i, y_i), rho_i = 1 / <y_i, s_i>, with the initial
matrix gamma_k I, gamma_k = <s, y> / <y, y> of the newest pair (1 while there is none).
A pair is known one iteration after its step:
  s_k = m_{k+1} - m_k  (the models the iterations actually used, in PySIT's linear form
        m = C**-2),
  y_k = g_{k+1} - g_k,
with the model-space inner product (cell-volume weighted).  The line search starts from
f / (|g| prod(deltas))^2 on the first step after the memory is cleared (at every call of
``inner_loop`` unless ``reset_on_new_inner_loop_call`` is False) and from 1 afterwards.
"""
from __future__ import annotations

import copy
from collections import deque
from dataclasses import dataclass

from .optimization import OptimizationBase

__all__ = ["LBFGS", "two_loop"]


@dataclass
class CurvaturePair:
    s: object     # model difference (ModelPerturbation)
    y: object     # gradient difference (ModelPerturbation)
    rho: float    # 1 / <y, s>


def two_loop(gradient, pairs, gamma):
    """H g for the L-BFGS matrix of `pairs` (oldest first) with H0 = gamma I."""
    q = copy.deepcopy(gradient)
    coeffs = []
    for p in reversed(pairs):            # newest to oldest
        a = p.rho * p.s.inner_product(q)
        q -= a * p.y
        coeffs.append(a)
    r = gamma * q
    for p, a in zip(pairs, reversed(coeffs)):  # oldest to newest
        b = p.rho * p.y.inner_product(r)
        r += (a - b) * p.s
    return r


class LBFGS(OptimizationBase):

    def __init__(self, objective, memory_length=None, reset_on_new_inner_loop_call=True, *args, **kwargs):
        super().__init__(objective, *args, **kwargs)
        self.memory_length = memory_length  # None: every pair is kept
        self.reset_on_new_inner_loop_call = reset_on_new_inner_loop_call
        self.clear_memory()

    def clear_memory(self):
        self.memory = deque(maxlen=self.memory_length)  # CurvaturePair, oldest first
        self._last = None     # (model, gradient) of the previous iteration: half of the next pair
        self._fresh = True    # the next line search starts from the scaled first length

    def inner_loop(self, *args, **kwargs):
        if self.reset_on_new_inner_loop_call:
            self.clear_memory()
        super().inner_loop(*args, **kwargs)

    def search_direction(self, shots, gradient, iteration, objective_arguments):
        model = copy.deepcopy(self.base_model)
        if self._last is not None:
            m_prev, g_prev = self._last
            s = model - m_prev
            y = gradient - g_prev
            self.memory.append(CurvaturePair(s=s, y=y, rho=1.0 / y.inner_product(s)))
        gamma = 1.0
        if self.memory:
            p = self.memory[-1]
            gamma = p.s.inner_product(p.y) / p.y.inner_product(p.y)
        self._last = (model, copy.deepcopy(gradient))
        return -1.0 * two_loop(gradient, list(self.memory), gamma)

    def trial_length(self, value, gradient, iteration):
        return self._scaled_first_length(value, gradient) if self._fresh else 1.0

    def step_taken(self, length, direction):
        self._fresh = False
