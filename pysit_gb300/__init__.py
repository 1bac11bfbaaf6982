"""pysit_gb300: GB300-native engine for PySIT's time-domain constant-density
acoustic solver with PML and its adjoint-state FWI gradient.

``from pysit_gb300 import *`` exposes the same names a PySIT script uses on
this path (RectangularDomain, PML, CartesianMesh, PointSource, ReceiverSet,
RickerWavelet, equispaced_acquisition, ConstantDensityAcousticWave,
generate_seismic_data, TemporalModeling, TemporalLeastSquares, LBFGS,
GradientDescent, GaussNewton), with
``kernel_implementation='cuda'``.  ``pysit_gb300.plugin.register()`` adds the
same solvers to an installed PySIT's own factory instead.
"""
from .core import *  # noqa: F401,F403
from .solvers import (ConstantDensityAcousticWave, ConstantDensityAcousticParameters,  # noqa: F401
                      ConstantDensityAcousticTimeScalar_1D_cuda, ConstantDensityAcousticTimeScalar_2D_cuda,
                      ConstantDensityAcousticTimeScalar_3D_cuda, NoMatchError, MultipleMatchError)
from .modeling import (TemporalModeling, generate_seismic_data, generate_seismic_data_from_file,  # noqa: F401
                       generate_shot_data_time)
from .objective_functions import TemporalLeastSquares  # noqa: F401
from .optimization import LBFGS, GradientDescent, GaussNewton  # noqa: F401

__version__ = "0.1.0"
