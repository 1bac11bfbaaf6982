"""Descent loop shared by the optimizers (mirror of pysit.optimization.OptimizationBase).

Behaviour followed (pysit/optimization/optimization.py):
  * ``__call__(shots, initial_value, iteration_parameters, line_search='backtrack',
    verbose=False, append=False, status_configuration={}, **kwargs)`` runs the inner
    loop for an int, or once per entry of an iterable of ints / (steps, arguments)
    pairs (:197-273; plain ints in an iterable, which the reference's docstring
    promises but its type check rejects, are accepted here);
  * every iteration: one ``compute_gradient`` with ``aux_info`` asking for the
    objective value and residual norm, histories, ``_select_step``, then
    ``base_model += step`` (:275-341);
  * histories are dicts {iteration: deep copy} kept when the iteration is a
    multiple of the frequency (:100-214); ``retrieve_history`` returns
    ``(iterations, values)``;
  * line search: ``'constant'`` (the first element of a tuple config) or
    ``'backtrack'`` (Armijo condition with c = 1e-3, the trial step scaled by
    0.8 per pass, alpha halved until the trial model validates, at most
    ``max_linesearch_iterations`` + 1 passes, acceptance also when the two
    sides agree to 1e-6 relative) (:343-502).

With a GPU objective (TemporalLeastSquares of a cuda solver) every gradient and
every line-search evaluation is one batched device call over all shots.
"""
from __future__ import annotations

import copy
import sys
import time

import numpy as np

__all__ = ["OptimizationBase"]

# backtracking line search constants (optimization.py:454-458)
_SHRINK = 0.8        # trial step factor after a rejected pass
_UPSCALE = 0.7       # passed to _compute_alpha0 as upscale_factor
_ARMIJO_C = 1e-3     # sufficient-decrease constant
_FP_REL = 1e-6       # accept when |f_new - bound| / |f_new| is below this

_HISTORIES = ("value", "gradient", "gradient_length", "step", "step_length", "residual_length",
              "objective", "run_time", "alpha")


class OptimizationBase:
    """Stateful descent algorithm over a PySIT-style objective."""

    def __init__(self, objective):
        self.objective_function = objective
        self.solver = objective.solver
        self.verbose = False
        self.use_parallel = objective.use_parallel()
        self.max_linesearch_iterations = 10
        self.logfile = sys.stdout

    # ---- histories ---------------------------------------------------------------------
    def reset(self, append_mode, value_frequency=0, gradient_frequency=0, gradient_length_frequency=0,
              step_frequency=0, step_length_frequency=0, residual_length_frequency=0, objective_frequency=0,
              run_time_frequency=0, alpha_frequency=1, *args, **kwargs):
        if append_mode and hasattr(self, "iteration"):
            return
        self.base_model = self.solver.ModelParameters(self.solver.mesh)
        self.iteration = 0
        freqs = dict(value=value_frequency, gradient=gradient_frequency,
                     gradient_length=gradient_length_frequency, step=step_frequency,
                     step_length=step_length_frequency, residual_length=residual_length_frequency,
                     objective=objective_frequency, run_time=run_time_frequency, alpha=alpha_frequency)
        for name in _HISTORIES:
            self.init_history(name, freqs[name])

    def init_history(self, arg, freq):
        setattr(self, arg + "_history", {})
        setattr(self, arg + "_frequency", freq)

    def query_store_history(self, arg, i):
        f = getattr(self, arg + "_frequency")
        return bool(f) and i % f == 0

    def _is_root(self):
        return not (self.use_parallel and self.objective_function.parallel_wrap_shot.rank != 0)

    def store_history(self, arg, i, val, force=False):
        if not self._is_root():
            return
        f = getattr(self, arg + "_frequency")
        if f and (force or i % f == 0):
            getattr(self, arg + "_history")[i] = copy.deepcopy(val)

    def retrieve_history(self, arg):
        if not getattr(self, arg + "_frequency"):
            return None, None
        return list(zip(*sorted(getattr(self, arg + "_history").items())))

    def _print(self, *args):
        if self._is_root() and self.verbose:
            print(*args, file=self.logfile)

    # ---- the loop -------------------------------------------------------------------------
    def initialize(self, initial_value, **kwargs):
        self.base_model = copy.deepcopy(initial_value)
        self.solver.model_parameters = self.base_model

    def __call__(self, shots, initial_value, iteration_parameters, line_search="backtrack", verbose=False,
                 append=False, status_configuration={}, **kwargs):
        self.reset(append, **status_configuration)
        self.verbose = verbose
        self.line_search = line_search
        if isinstance(line_search, str):
            self.ls_method, self.ls_config = line_search, None
        else:  # ('method', config...)
            self.ls_method, self.ls_config = line_search[0], line_search[1:]
        self.initialize(initial_value, **kwargs)

        if isinstance(iteration_parameters, int):
            self.inner_loop(shots, iteration_parameters, **kwargs)
        elif np.iterable(iteration_parameters):
            for ip in iteration_parameters:
                if isinstance(ip, (tuple, list)):
                    steps, arguments = ip
                elif isinstance(ip, (int, np.integer)):
                    # documented at optimization.py:233; the reference's check (:239) tests the
                    # whole iterable instead of the entry and raises for plain ints
                    steps, arguments = int(ip), {}
                else:
                    raise ValueError("Invalid iteration parameter {0} detected.".format(ip))
                self.inner_loop(shots, steps, objective_arguments=arguments, **kwargs)
        else:
            raise ValueError("Singular iteration parameters of type {0} are not permitted at this time."
                             .format(type(iteration_parameters)))
        return self.base_model

    def inner_loop(self, shots, steps, objective_arguments={}, **kwargs):
        for _ in range(steps):
            t0 = time.time()
            i = self.iteration
            self.store_history("value", i, self.base_model)
            self._print("Iteration {0}".format(i))
            self.solver.model_parameters = self.base_model
            aux_info = {"objective_value": (True, None), "residual_norm": (True, None)}
            objective_arguments.update(kwargs)

            gradient = self.objective_function.compute_gradient(shots, self.base_model, aux_info=aux_info,
                                                                 **objective_arguments)
            objective_value = aux_info["objective_value"][1]
            self.store_history("gradient", i, gradient)
            gnorm = gradient.norm()
            self._print("  gradnorm {0}".format(gnorm))
            self.store_history("gradient_length", i, gnorm)
            if objective_value is not None:
                self.store_history("objective", i, objective_value)
                self._print("  objective {0}".format(objective_value))
            if aux_info["residual_norm"][1] is not None:
                self.store_history("residual_length", i, aux_info["residual_norm"][1])
                self._print("  residual {0}".format(aux_info["residual_norm"][1]))

            step = self._select_step(shots, objective_value, gradient, i, objective_arguments, **kwargs)
            self.store_history("step_length", i, step.norm())
            self.store_history("step", i, step)
            self.base_model += step

            elapsed = time.time() - t0
            self.store_history("run_time", i, elapsed)
            self.iteration += 1
            self._print("  run time {0}s".format(elapsed))

    def _select_step(self, shots, current_objective_value, gradient, iteration, objective_arguments, **kwargs):
        raise NotImplementedError("_select_step must be implemented by a subclass.")

    # ---- step length -----------------------------------------------------------------------
    def select_alpha(self, shots, gradient, direction, objective_arguments, **kwargs):
        if self.ls_method == "constant":
            return self.ls_config[0]
        if self.ls_method == "linear":
            raise NotImplementedError("Linear selection of alpha is an objective function dependent operation.")
        if self.ls_method == "backtrack":
            return self._backtrack_line_search(shots, gradient, direction, objective_arguments, **kwargs)
        raise ValueError("Alpha selection method {0} invalid".format(self.ls_method))

    def _backtrack_line_search(self, shots, gradient, direction, objective_arguments, current_objective_value=None,
                               alpha0_kwargs={}, **kwargs):
        if current_objective_value is None:
            fk = self.objective_function.evaluate(shots, self.base_model, **objective_arguments)
        else:
            fk = current_objective_value
        a0kw = dict(alpha0_kwargs)
        a0kw["upscale_factor"] = _UPSCALE
        alpha = self._compute_alpha0(current_objective_value, gradient, **a0kw)
        self._print("  Starting: ", alpha, fk)

        npass = 1
        while True:
            # the largest alpha (halving from the proposal) whose model is valid
            alpha *= 2
            while True:
                alpha /= 2
                trial_step = alpha * direction
                model = self.base_model + trial_step
                if model.validate():
                    break
            self.solver.model_parameters = model
            fnew = self.objective_function.evaluate(shots, model, **objective_arguments)
            bound = fk + alpha * _ARMIJO_C * gradient.inner_product(trial_step)
            self._print("  Pass {0}: a:{1}; {2} ?<= {3}".format(npass, alpha, fnew, bound))
            if fnew <= bound or abs(fnew - bound) / abs(fnew) <= _FP_REL:
                break
            if npass > self.max_linesearch_iterations:
                self._print("Too many passes ({0}), attempting to use current alpha ({1}).".format(npass, alpha))
                break
            npass += 1
            alpha *= _SHRINK
        self.prev_alpha = alpha
        return alpha

    def _compute_alpha0(self, phi0, grad0, **kwargs):
        raise NotImplementedError("_compute_alpha0 must be implemented by a subclass.")
