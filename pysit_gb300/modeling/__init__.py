"""Modelling (mirror of pysit.modeling for the time-domain CDA path)."""
from .temporal_modeling import TemporalModeling  # noqa: F401
from .data_modeling import (generate_seismic_data, generate_seismic_data_from_file,  # noqa: F401
                            generate_shot_data_time)
