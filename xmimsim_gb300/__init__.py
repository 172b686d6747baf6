"""GB300-native XRF photon-transport Monte Carlo engine with XMI-MSIM's
library surface.  The compute lives in libxmimsim_gb300.so (CUDA, sm_103a);
this package holds the build recipe, the ctypes mirror of the C-ABI and the
Python host mirror of the reference's call chain."""
from . import abi
from .simulation import (ContinuousPoint, DiscreteLine, InputSpec, Layer, Simulation, XmiError, gpu_options,
                         last_timing, make_options)

__all__ = ["abi", "ContinuousPoint", "DiscreteLine", "InputSpec", "Layer", "Simulation", "XmiError",
           "gpu_options", "last_timing", "make_options"]
