"""Geometry and acquisition (mirror of pysit.core for the time-domain CDA path)."""
from .domain import PML, Dirichlet, DomainBC, RectangularDomain  # noqa: F401
from .mesh import CartesianMesh, StructuredDirichlet, StructuredPML  # noqa: F401
from .acquisition import (DerivativeGaussianPulse, GaussianPulse, PointReceiver, PointSource,  # noqa: F401
                          ReceiverSet, RickerWavelet, Shot, SourceEncodedSupershot, SourceSet,
                          equispaced_acquisition,
                          linear_interpolate)
