"""omni3d: GB300 (sm_103a) omni-directional 3D pressure reconstruction.

The compute path is libomni3d_gb300.so (CUDA kernels behind the C ABI of
include/omni3d.h); this package is its Python binding.  It has no CPU fallback: every
compute call goes through the library and fails when it is not built.
"""
from ._lib import Omni3DError, lib  # noqa: F401
from .build import build  # noqa: F401
from .solver import (Batch, Omni3D, SolveResult, bernoulli_face, icosphere, read_directions, read_params,  # noqa: F401
                     read_tecplot, write_curl, write_pressure)

__all__ = ["Batch", "Omni3D", "SolveResult", "Omni3DError", "build", "lib", "icosphere", "read_directions", "read_params",
           "read_tecplot", "write_pressure", "write_curl", "bernoulli_face"]
