"""GB300-native periodic-box pair counting for intrinsic-alignment measurements.

Drop-in for MeasureIA's ``MeasureIABox`` (w_gg, w_g+, multipoles, jackknife
covariance); the pair counts run in hand-written sm_103a CUDA kernels behind
the C ABI of ``include/measure_ia_gb300.h``.
"""

from .lightcone import MeasureIALightcone
from .measure_ia import MeasureIABox
from .output import open_output, read_output
from .read_data import ReadData
from .sim_info import SimInfo

__all__ = ["MeasureIABox", "MeasureIALightcone", "ReadData", "SimInfo", "open_output", "read_output"]
