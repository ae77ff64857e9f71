"""GB300 (sm_103a) treecode convolution path of Treecode-Accelerated Green Iteration.

Reference-facing modules (same names and call signatures as
3D-GreenIteration/src/utilities):
  BaryTreeInterface          callTreedriver + enums
  orthogonalization_wrapper  callOrthogonalization
  interpolation_wrapper      callInterpolator
Device API over torch CUDA tensors: device (TreecodePlan, Systems, Graph,
treecode, treecode_batched, direct, mgs, interp).  Launch-shape tuning:
autotune.  Synthetic seeded workloads: synthetic.  Build: build.

TAGI imports these modules by name after putting the utilities directory on
sys.path; putting this directory on sys.path does the same here.
"""
from . import BaryTreeInterface, interpolation_wrapper, orthogonalization_wrapper, synthetic  # noqa: F401
from . import _native  # noqa: F401

__all__ = ["BaryTreeInterface", "orthogonalization_wrapper", "interpolation_wrapper", "synthetic",
           "device", "autotune", "build"]
