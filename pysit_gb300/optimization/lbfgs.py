"""Limited-memory BFGS (mirror of pysit.optimization.LBFGS, pysit/optimization/lbfgs.py:13-124).

The search direction is the two-loop recursion of Nocedal & Wright (Algorithm
7.4) over the stored pairs (s, y, rho), with the initial scaling
gamma = <s, y> / <y, y> of the newest pair (1 before any pair exists).  As in
the reference, a pair is completed one iteration late, when the next gradient
is known:
  s_k = m_{k+1} - m_k  (the difference of the models actually used, after any
        post-processing of ``base_model += step``, in the linear form m = C**-2),
  y_k = g_{k+1} - g_k,  rho_k = 1 / <y_k, s_k>,
with the model-space inner product (cell volume weighted).  The step length
comes from the line search; the backtracking line search starts from
alpha_0 = f / (|g| * prod(deltas))**2 on the first step after a memory reset,
and from 1 afterwards.
"""
from __future__ import annotations

import copy
from collections import deque

import numpy as np

from .optimization import OptimizationBase

__all__ = ["LBFGS"]


class LBFGS(OptimizationBase):

    def __init__(self, objective, memory_length=None, reset_on_new_inner_loop_call=True, *args, **kwargs):
        super().__init__(objective, *args, **kwargs)
        self.prev_alpha = None
        self.prev_model = None
        self.memory_length = memory_length  # None: unbounded
        self.reset_on_new_inner_loop_call = reset_on_new_inner_loop_call
        self._reset_memory()

    def _reset_memory(self):
        # entries [rho, s, y]; the newest holds [None, None, -g_k] until g_{k+1} is known
        self.memory = deque([], maxlen=self.memory_length)
        self._reset_line_search = True
        self.prev_model = None

    def inner_loop(self, *args, **kwargs):
        if self.reset_on_new_inner_loop_call:
            self._reset_memory()
        super().inner_loop(*args, **kwargs)

    def _select_step(self, shots, current_objective_value, gradient, iteration, objective_arguments, **kwargs):
        mem = self.memory
        q = copy.deepcopy(gradient)
        x_k = copy.deepcopy(self.base_model)

        gamma = 1.0
        if len(mem) > 0:
            newest = mem[-1]
            newest[2] += gradient                       # y = g_k - g_{k-1}
            newest[1] = x_k - self.prev_model            # s = m_k - m_{k-1}
            newest[0] = 1.0 / newest[2].inner_product(newest[1])
            gamma = newest[1].inner_product(newest[2]) / newest[2].inner_product(newest[2])

        # first loop, newest to oldest
        alphas = []
        for rho, s, y in reversed(mem):
            a = rho * s.inner_product(q)
            q -= a * y
            alphas.append(a)
        alphas.reverse()
        # second loop, oldest to newest
        r = gamma * q
        for a, (rho, s, y) in zip(alphas, mem):
            b = rho * y.inner_product(r)
            r += (a - b) * s
        direction = -1.0 * r

        a0kw = {"reset": self._reset_line_search}
        self._reset_line_search = False
        alpha = self.select_alpha(shots, gradient, direction, objective_arguments,
                                  current_objective_value=current_objective_value, alpha0_kwargs=a0kw, **kwargs)
        self._print("  alpha {0}".format(alpha))
        self.store_history("alpha", iteration, alpha)

        self.prev_model = x_k
        mem.append([None, None, copy.deepcopy(-1 * gradient)])
        return alpha * direction

    def _compute_alpha0(self, phi0, grad0, reset=False, *args, **kwargs):
        if reset:
            return phi0 / (grad0.norm() * np.prod(self.solver.mesh.deltas)) ** 2
        return 1.0
