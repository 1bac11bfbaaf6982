"""Step-length rules of the descent methods (Nocedal & Wright, Numerical Optimization,
2nd ed., section 3.1), with the constants and tests PySIT's optimizers use
(pysit/optimization/optimization.py:343-502), so that a run takes PySIT's steps:

``FixedStep``      every step has the same length (PySIT's ``('constant', alpha)``);
``Backtracking``   Algorithm 3.1 of Nocedal & Wright: start from a trial length and
                   contract it until a sufficient-decrease test holds (PySIT's
                   ``'backtrack'``).

A rule is called with a ``StepProblem``: the objective at the base model, the gradient,
the search direction and the trial length, plus a way to evaluate the objective at a
trial model.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable

__all__ = ["StepProblem", "FixedStep", "Backtracking", "make_rule"]


@dataclass
class StepProblem:
    """What a step-length rule needs from the optimizer for one step."""
    base_model: object                 # ModelParameters at the current iterate
    value: float                       # objective at base_model
    gradient: object                   # ModelPerturbation
    direction: object                  # ModelPerturbation (a descent direction)
    trial_length: Callable[[], float]  # the first length to try (asked for only by rules that use it)
    evaluate: Callable[[object], float]  # objective at a trial model
    log: Callable[[str], None]


class FixedStep:
    """The same length for every step."""

    def __init__(self, length):
        self.length = float(length)

    def __call__(self, problem: StepProblem) -> float:
        return self.length


class Backtracking:
    """Backtracking until sufficient decrease.

    From the trial length a, each pass first halves a until the trial model
    m + a p is a valid model (``validate()``), then evaluates f(m + a p) and accepts a
    when f(m + a p) <= f(m) + c a <g, a p> (PySIT's test carries the length twice), or
    when both sides agree to 1e-6 relative, or when `max_passes` + 1 passes have run.
    Otherwise a is contracted by 0.8 and the next pass begins.  c = 1e-3."""

    contraction = 0.8
    sufficient_decrease = 1e-3
    agreement = 1e-6
    trial_growth = 0.7  # optimizers that start from the last accepted length divide it by this

    def __init__(self, max_passes=10):
        self.max_passes = max_passes

    def __call__(self, problem: StepProblem) -> float:
        a = problem.trial_length()
        problem.log(f"  line search from length {a} at objective {problem.value}")
        passes = 0
        while True:
            passes += 1
            a = self._largest_valid(problem, a)
            step = a * problem.direction
            trial = problem.base_model + step
            f = problem.evaluate(trial)
            bound = problem.value + a * self.sufficient_decrease * problem.gradient.inner_product(step)
            problem.log(f"  pass {passes}: length {a}, objective {f}, bound {bound}")
            if f <= bound or abs(f - bound) / abs(f) <= self.agreement:
                return a
            if passes > self.max_passes:
                problem.log(f"  no sufficient decrease after {passes} passes; keeping length {a}")
                return a
            a *= self.contraction

    @staticmethod
    def _largest_valid(problem, a):
        """a, halved until the trial model is valid (a itself when it already is)."""
        while not (problem.base_model + a * problem.direction).validate():
            a /= 2
        return a


def make_rule(line_search, max_passes):
    """The rule for PySIT's ``line_search`` argument: 'backtrack', or a tuple
    ('constant', length)."""
    if isinstance(line_search, str):
        name, args = line_search, ()
    else:
        name, args = line_search[0], tuple(line_search[1:])
    if name == "backtrack":
        return Backtracking(max_passes)
    if name == "constant":
        return FixedStep(args[0])
    if name == "linear":
        raise NotImplementedError("a linear step-length rule depends on the objective and is not provided")
    raise ValueError(f"unknown line search {line_search!r}")
