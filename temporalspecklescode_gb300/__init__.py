"""GB300-native next-event-estimation speckle path tracer.

Drop-in for the rendering path of chabner/temporalSpecklesCode's
``sstmc2D``/``sstmc3D`` MEX functions: the same config semantics, a C-ABI
(include/sstmc.h) over hand-written sm_103a CUDA kernels, and a Python mirror
of the MATLAB call.
"""
from .config import ConfigError, prepare  # noqa: F401
from .api import Scene, SstmcError, load_library, sstmc2D, sstmc3D  # noqa: F401
