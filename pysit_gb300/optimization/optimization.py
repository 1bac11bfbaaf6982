"""The descent driver shared by the optimizers, with PySIT's calling convention and
histories (pysit/optimization/optimization.py).

One iteration of a line-search method (Nocedal & Wright, Numerical Optimization, 2nd
ed., chapter 3): the objective and its gradient at the iterate, a search direction from
the method (``search_direction``), a step length from the rule chosen by ``line_search``
(``line_search.py``) starting at the method's trial length (``trial_length``), and the
move ``base_model += length * direction``.

The public surface is PySIT's: ``opt(shots, initial_value, iteration_parameters,
line_search='backtrack', verbose=False, append=False, status_configuration={})`` with
``iteration_parameters`` an int, or an iterable of ints and (steps, objective arguments)
pairs run one after the other; ``retrieve_history(name)`` -> (iterations, values) for
the histories switched on by ``status_configuration`` ('<name>_frequency': keep every
n-th iteration; alpha is kept every iteration by default).

With a GPU objective (TemporalLeastSquares of a cuda solver) every gradient and every
line-search evaluation is one batched device call over all shots.
"""
from __future__ import annotations

import copy
import sys
import time

import numpy as np

from .line_search import Backtracking, StepProblem, make_rule

__all__ = ["OptimizationBase"]

HISTORY_NAMES = ("value", "gradient", "gradient_length", "step", "step_length", "residual_length", "objective",
                 "run_time", "alpha")


class _History:
    """Values of one quantity at the iterations that are multiples of `every` (0: none)."""

    def __init__(self, every):
        self.every = every
        self.values = {}

    def keep(self, iteration, value, force=False):
        if self.every and (force or iteration % self.every == 0):
            self.values[iteration] = copy.deepcopy(value)

    def items(self):
        if not self.every:
            return None, None
        return list(zip(*sorted(self.values.items())))


def _phases(iteration_parameters):
    """(steps, objective arguments) of each phase of a run."""
    if isinstance(iteration_parameters, (int, np.integer)):
        return [(int(iteration_parameters), {})]
    if not np.iterable(iteration_parameters):
        raise ValueError(f"iteration parameters must be an int or an iterable, not {type(iteration_parameters)}")
    phases = []
    for entry in iteration_parameters:
        if isinstance(entry, (int, np.integer)):
            phases.append((int(entry), {}))
        elif isinstance(entry, (tuple, list)) and len(entry) == 2:
            phases.append((int(entry[0]), entry[1]))
        else:
            raise ValueError(f"iteration parameter {entry!r} is neither a step count nor a (steps, arguments) pair")
    return phases


class OptimizationBase:
    """Line-search descent over a PySIT-style objective (evaluate / compute_gradient)."""

    def __init__(self, objective):
        self.objective_function = objective
        self.solver = objective.solver
        self.use_parallel = objective.use_parallel()
        self.verbose = False
        self.logfile = sys.stdout
        self.max_linesearch_iterations = 10
        self.iteration = 0
        self.prev_alpha = None
        self._histories = {name: _History(0) for name in HISTORY_NAMES}

    # ---- methods supply these --------------------------------------------------------------
    def search_direction(self, shots, gradient, iteration, objective_arguments):
        raise NotImplementedError

    def trial_length(self, value, gradient, iteration):
        raise NotImplementedError

    def step_taken(self, length, direction):
        """Called once per iteration after the step length is chosen."""

    # ---- histories ---------------------------------------------------------------------------
    def _start_histories(self, config):
        every = {name: 0 for name in HISTORY_NAMES}
        every["alpha"] = 1
        for key, value in config.items():
            name = key[:-len("_frequency")] if key.endswith("_frequency") else key
            if name in every:
                every[name] = value
        self._histories = {name: _History(every[name]) for name in HISTORY_NAMES}

    def _on_root(self):
        return not (self.use_parallel and self.objective_function.parallel_wrap_shot.rank != 0)

    def store_history(self, name, iteration, value, force=False):
        if self._on_root():
            self._histories[name].keep(iteration, value, force)

    def retrieve_history(self, name):
        return self._histories[name].items()

    def _log(self, message):
        if self.verbose and self._on_root():
            print(message, file=self.logfile)

    # ---- the run -------------------------------------------------------------------------------
    def __call__(self, shots, initial_value, iteration_parameters, line_search="backtrack", verbose=False,
                 append=False, status_configuration={}, **kwargs):
        phases = _phases(iteration_parameters)
        if not (append and hasattr(self, "base_model")):
            self.iteration = 0
            self._start_histories(status_configuration)
        self.verbose = verbose
        self.line_search = line_search
        self._rule = make_rule(line_search, self.max_linesearch_iterations)
        self.base_model = copy.deepcopy(initial_value)
        self.solver.model_parameters = self.base_model
        for steps, arguments in phases:
            self.inner_loop(shots, steps, objective_arguments=arguments, **kwargs)
        return self.base_model

    def inner_loop(self, shots, steps, objective_arguments={}, **kwargs):
        arguments = dict(objective_arguments, **kwargs)
        for _ in range(steps):
            self._iterate(shots, arguments)

    def _iterate(self, shots, arguments):
        started = time.time()
        k = self.iteration
        self._log(f"iteration {k}")
        self.store_history("value", k, self.base_model)
        self.solver.model_parameters = self.base_model
        aux = {"objective_value": (True, None), "residual_norm": (True, None)}
        gradient = self.objective_function.compute_gradient(shots, self.base_model, aux_info=aux, **arguments)
        value, rnorm = aux["objective_value"][1], aux["residual_norm"][1]
        gnorm = gradient.norm()
        self.store_history("gradient", k, gradient)
        self.store_history("gradient_length", k, gnorm)
        if value is not None:
            self.store_history("objective", k, value)
        if rnorm is not None:
            self.store_history("residual_length", k, rnorm)
        self._log(f"  objective {value}, residual norm {rnorm}, gradient norm {gnorm}")

        direction = self.search_direction(shots, gradient, k, arguments)
        length = self._step_length(shots, value, gradient, direction, k, arguments)
        self.store_history("alpha", k, length)
        self._log(f"  step length {length}")
        self.step_taken(length, direction)
        step = length * direction
        self.store_history("step_length", k, step.norm())
        self.store_history("step", k, step)
        self.base_model += step

        self.store_history("run_time", k, time.time() - started)
        self.iteration += 1

    def _step_length(self, shots, value, gradient, direction, iteration, arguments):
        def evaluate(model):
            self.solver.model_parameters = model
            return self.objective_function.evaluate(shots, model, **arguments)

        problem = StepProblem(base_model=self.base_model, value=value, gradient=gradient, direction=direction,
                              trial_length=lambda: self.trial_length(value, gradient, iteration), evaluate=evaluate,
                              log=self._log)
        length = self._rule(problem)
        if isinstance(self._rule, Backtracking):
            self.prev_alpha = length
        return length

    # ---- shared trial lengths ------------------------------------------------------------------
    def _scaled_first_length(self, value, gradient):
        """f / (|g| prod(deltas))^2: a first step whose size suits the model's units."""
        return value / (gradient.norm() * np.prod(self.solver.mesh.deltas)) ** 2
