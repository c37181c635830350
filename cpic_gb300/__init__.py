"""cpic_gb300: cpic's 2D electrostatic PIC time step on one GB300.

The compute path is libcpic_gb300.so (CUDA, sm_103a), reached through the
C ABI declared in include/cpic_gpu.h.  This package holds the build recipe
(`build`), the ctypes binding (`_lib`, used by the tests and the benchmark),
the test-only torch.autograd binding of the adjoint (`autograd`) and the C
drop-in for the reference's host program (`dropin/sim_gpu.c`, which exports
its sim_init / sim_step / sim_run).
"""
from . import build  # noqa: F401
from ._lib import (FP64, MIXED, Context, CpicError, load, init_two_stream,  # noqa: F401
                   init_maxwellian, uniform)
