"""skewtcloudsim_gb300: GB300-native per-timestep 3D atmosphere solver of skewTCloudSim.

The compute path is libskewt_gb300.so (hand-written CUDA for sm_103a behind the C ABI in
include/skewt.h). This package holds the host-side mirror of the reference's environmentGPU
(``Environment``), the synthetic sounding generator, the radiosonde readers (``radiosonde``)
and the build recipe.
"""
from .environment import (Environment, Ensemble, SolverConfig, step_ensemble, Parameter, Direction, Ground, Column, Status,
                          SktError, FIELDS, GROUND_FIELDS, COLUMNS, DIAG_BUOYANCY, RATE_NAMES)
from . import sounding
from . import radiosonde

__all__ = ["radiosonde", "step_ensemble", "Ensemble", "Environment", "SolverConfig", "Parameter", "Direction", "Ground", "Column", "Status", "SktError",
           "FIELDS", "GROUND_FIELDS", "COLUMNS", "DIAG_BUOYANCY", "RATE_NAMES", "sounding"]
