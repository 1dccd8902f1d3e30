"""nuto_gb300 — GB300-native (sm_103a) element-assembly hot path of the NuTo finite-element library.

The product is the CUDA library nuto_gb300/lib/libnuto_gb300.so behind the C ABI in include/nuto_gpu.h;
this package binds it for Python callers, builds the structured meshes with NuTo's DOF numbering and provides
the configurations used by the tests and the benchmark.
"""

from . import _lib, adaptive, mesh, configs  # noqa: F401
from ._lib import (FP32, FP64, FP64X, GRADIENT_DAMAGE, HEX8, HEX20, MB_LINEAR_ELASTIC, MB_LOCAL_DAMAGE,  # noqa: F401
                   MIXED, PRECOND_AMG, PRECOND_JACOBI, QUAD4, SOLVER_AUTO, SOLVER_BICGSTAB, SOLVER_GMRES, SOLVER_PCG,
                   NoConvergence, NutoGpuError, load)
from .assembly import GpuCellGroup  # noqa: F401
