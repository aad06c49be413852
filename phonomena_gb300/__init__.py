"""phonomena_gb300: GB300-native (sm_103a) time-stepping solver for phonomena.

The hot path is one fused CUDA kernel per FDTD step (csrc/fdtd_step.cu)
behind the C ABI of include/phono.h; ``solver_gb300.Solver`` is the drop-in
plugin for phonomena's solver registry.
"""
from .model import Grid, Material, solver_inputs  # noqa: F401

__version__ = "0.1.0"
