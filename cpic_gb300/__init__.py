"""cpic_gb300: cpic's 2D electrostatic PIC time step on one GB300.

The compute path is libcpic_gb300.so (CUDA, sm_103a), reached through the
C ABI declared in include/cpic_gpu.h.  This package holds the build recipe
(`build`), the ctypes binding (`_lib`) and the host-side mirror of the
reference's simulation interface (`sim`).
"""
from . import build  # noqa: F401
from ._lib import (FP64, MIXED, Context, CpicError, load, init_two_stream,  # noqa: F401
                   init_maxwellian, uniform)
