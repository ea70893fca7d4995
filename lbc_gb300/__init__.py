"""lbc_gb300: a GB300-native (sm_103a) D2Q9 lattice Boltzmann engine behind lbc's C API.

The product is lbc_gb300/_build/liblbm_gpu.so (CUDA kernels + C ABI). This
package holds its build recipe, Python bindings and case-setup recipes.
"""
from .cases import BC, Case, State  # noqa: F401
from .runtime import (F16_SHIFTED, F32_SHIFTED, F64, F64_FMA, STORAGE, GpuBatch, GpuServer, GpuSolver,  # noqa: F401
                      PinnedArray,
                      dropin, last_error, load_library)
