"""Objective functions (mirror of pysit.objective_functions for the time-domain path)."""
from .temporal_least_squares import ObjectiveFunctionBase, TemporalLeastSquares  # noqa: F401
