"""Solver factory (mirror of pysit.solvers.wave_factory / util.basic_registration_factory).

``ConstantDensityAcousticWave(mesh, spatial_accuracy_order=..., kernel_implementation='cuda', ...)``
resolves the registered class whose ``supports`` dictionary matches every
keyword given (a "complete" match, pysit/solvers/solver_base.py:75-102 and
pysit/util/basic_registration_factory.py:167-208): keywords absent from the call
make the match "incomplete"; the first incomplete match is used when no
complete one exists; no match raises NoMatchError; several complete matches
raise MultipleMatchError.
"""
from __future__ import annotations

from .cda_time import (ConstantDensityAcousticTimeScalar_1D_cuda, ConstantDensityAcousticTimeScalar_2D_cuda,
                       ConstantDensityAcousticTimeScalar_3D_cuda)
from .model_parameter import ConstantDensityAcousticParameters

__all__ = ["ConstantDensityAcousticWave", "SolverFactory", "NoMatchError", "MultipleMatchError",
           "ConstantDensityAcousticParameters", "ConstantDensityAcousticTimeScalar_1D_cuda",
           "ConstantDensityAcousticTimeScalar_2D_cuda", "ConstantDensityAcousticTimeScalar_3D_cuda"]

DoesNotMatch, IncompleteMatch, CompleteMatch = 0, 1, 2


class NoMatchError(Exception):
    """No registered solver matches the arguments."""


class MultipleMatchError(Exception):
    """Several registered solvers match the arguments."""


def _supports(needle, haystack):
    if isinstance(haystack, (list, tuple, set)):
        return needle in haystack
    return needle == haystack


class SolverFactory:
    """Ternary-matching registry of solver classes."""

    supports = {"equation_physics": None, "equation_dynamics": None}

    def __init__(self, supports=None):
        if supports is not None:
            self.supports = dict(supports)
        self.registry = []

    def register(self, cls, is_default=False):
        for key in ("equation_physics", "equation_dynamics"):
            if self.supports.get(key) != cls.supports.get(key):
                raise ValueError(f"Factory accepts '{self.supports.get(key)}' {key} while solver "
                                 f"{cls.__name__} supports '{cls.supports.get(key)}'.")
        self.registry.append(cls)

    @staticmethod
    def _match(cls, mesh, kwargs):
        complete = True
        for key, values in cls.supports.items():
            if key in kwargs:
                if not _supports(kwargs[key], values):
                    return DoesNotMatch
            elif key == "boundary_conditions":
                for i in range(mesh.dim):
                    p = mesh.parameters[i]
                    if not (_supports(p.lbc.type, values) and _supports(p.rbc.type, values)):
                        return DoesNotMatch
            elif key == "spatial_dimension":
                if not _supports(mesh.dim, values):
                    return DoesNotMatch
            else:
                complete = False
        return CompleteMatch if complete else IncompleteMatch

    def resolve(self, mesh, **kwargs):
        kw = dict(self.supports)
        kw.update(kwargs)
        complete, incomplete = [], []
        for cls in self.registry:
            m = self._match(cls, mesh, kw)
            (complete if m == CompleteMatch else incomplete if m == IncompleteMatch else []).append(cls)
        if len(complete) == 1:
            return complete[0]
        if len(complete) > 1:
            raise MultipleMatchError(f"Too many candidate types match ({len(complete)}).")
        if incomplete:
            return incomplete[0]
        raise NoMatchError("No types match specified arguments and no default is set.")

    def __call__(self, mesh, *args, **kwargs):
        cls = self.resolve(mesh, **kwargs)
        return cls(mesh, *args, **kwargs)


ConstantDensityAcousticWave = SolverFactory({"equation_physics": "constant-density-acoustic",
                                             "equation_dynamics": "time"})
ConstantDensityAcousticWave.register(ConstantDensityAcousticTimeScalar_1D_cuda)
ConstantDensityAcousticWave.register(ConstantDensityAcousticTimeScalar_2D_cuda)
ConstantDensityAcousticWave.register(ConstantDensityAcousticTimeScalar_3D_cuda)
