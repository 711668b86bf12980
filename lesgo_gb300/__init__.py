"""GB300-native implementation of LESGO's per-timestep LES hot path.

The compute lives in the CUDA library ``liblesgo_gpu.so`` (sources in
``csrc/``, C ABI in ``include/lesgo_gpu.h``); ``LesgoGPU`` is the host-side
mirror of the reference's subroutine interface.
"""
from .build import build, LIB  # noqa: F401


def __getattr__(name):
    if name in ("LesgoGPU", "LesgoError"):
        from . import solver
        return getattr(solver, name)
    raise AttributeError(name)
