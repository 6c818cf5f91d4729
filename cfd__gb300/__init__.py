"""cfd__gb300 — GB300-native (sm_103a) solver hot path of the CFD_ browser wind tunnel.

The D3Q19 TRT/LES stream-collide step, the momentum-exchange force and the
triangle-mesh voxelizer run as hand-written CUDA kernels behind the C ABI in
include/lbm.h and include/vox.h.  ``SolverCUDA`` mirrors the reference's
solver class API (src/backend/webgpu/solver.js) on top of that ABI; the
modules beside it restate the reference's host-side helpers (tunnel assembly,
units, coefficients, validation correlations).
"""
from . import lattice  # noqa: F401  (runs the velocity-set self check)
from ._native import LbmError, NativeUnavailable  # noqa: F401
from .solver import SolverCUDA  # noqa: F401

__all__ = ["SolverCUDA", "LbmError", "NativeUnavailable", "lattice"]
