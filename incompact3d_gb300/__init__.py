"""incompact3d_gb300: GB300-native (sm_103a) per-timestep hot path of Xcompact3d.

The compute lives in libx3dgpu.so (CUDA, C ABI in include/x3d_gpu.h); this
package builds it in-tree and mirrors the reference's operator interfaces on
the host.  There is no CPU fallback: without the built library every call
raises.
"""
from .build import build  # noqa: F401
from ._lib import (OP_DER1, OP_DER2, OP_DPV, OP_DVP, OP_FIL, OP_IPV, OP_IVP,  # noqa: F401
                   PREC_FP64, PREC_MIXED, X3DError, load)
from .operators import Context, Solver  # noqa: F401
