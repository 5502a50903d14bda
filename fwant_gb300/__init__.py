"""fwant_gb300: GB300-native forward solver of FWANT (seis3d_wave) behind a C ABI.

The compute path is the native library ``lib/libfwant_gb300.so`` (CUDA kernels for
sm_103a plus the C++ host driver); this package only binds it (``_lib``) and builds
the reference's input arrays (``inputs``).
"""
from ._lib import (COMPONENTS, STF_RICKER, STORAGE_BF16, STORAGE_FP16, STORAGE_FP32, STORAGE_FP64, FwantError,
                   Assm, Batch, KerInfo, Lsqr, Media, SgtKernel, Solver, load_library, metric, reference_steps,
                   source_time_function)

__all__ = ["Solver", "Batch", "Assm", "KerInfo", "SgtKernel", "Lsqr", "Media", "FwantError", "load_library", "metric", "reference_steps", "source_time_function", "COMPONENTS", "STF_RICKER",
           "STORAGE_FP32", "STORAGE_BF16", "STORAGE_FP16", "STORAGE_FP64"]
