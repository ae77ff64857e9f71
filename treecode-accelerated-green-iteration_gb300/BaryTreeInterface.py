"""Drop-in for 3D-GreenIteration/src/utilities/BaryTreeInterface.py.

Same enums (values from BaryTreeInterface.py:20-46), same ``callTreedriver``
signature and return value (a new float64 array of length numTargets,
BaryTreeInterface.py:88-158), but the call lands in libtagi_gb300.so, the
GB300 treecode, instead of BaryTree.  ``GPUpresent`` keeps its reference
meaning for argument checking only: there is one implementation, on the GPU,
and no CPU fallback.

Two optional keyword arguments are added at the end and default to the
reference behaviour:
  precision  "fp64" (default; the library default, see tagi_set_precision)
             or "mixed" (FP32 pair sums with compensated accumulation).
"""
import ctypes
from enum import IntEnum

import numpy as np

try:
    from . import _native
except ImportError:  # imported as a top-level module, the way TAGI imports it
    import _native


class CEnum(IntEnum):
    @classmethod
    def from_param(cls, self):
        if not isinstance(self, cls):
            raise TypeError
        return int(self)


class Kernel(CEnum):
    NO_KERNEL = 0
    COULOMB = 1
    YUKAWA = 2
    REGULARIZED_COULOMB = 3
    REGULARIZED_YUKAWA = 4
    ATAN = 5
    TCF = 6
    DCF = 7
    SIN_OVER_R = 8
    MQ = 9


class Singularity(CEnum):
    NO_SINGULARITY = 0
    SKIPPING = 1
    SUBTRACTION = 2


class Approximation(CEnum):
    NO_APPROXIMATION = 0
    LAGRANGE = 1
    HERMITE = 2


class ComputeType(CEnum):
    NO_COMPUTE_TYPE = 0
    PARTICLE_CLUSTER = 1
    CLUSTER_PARTICLE = 2
    CLUSTER_CLUSTER = 3


_PRECISION = {"mixed": _native.PREC_MIXED, "fp64": _native.PREC_FP64}


def _as_c_double(a, name):
    a = np.asarray(a)
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous float64 array")
    return a


def callTreedriver(numTargets, numSources,
                   targetX, targetY, targetZ, targetValue,
                   sourceX, sourceY, sourceZ, sourceValue, sourceWeight,
                   kernelName, numberOfKernelParameters, kernelParameters, singularityHandling,
                   approximationName, computeType, GPUpresent, verbosity,
                   beta=None, theta=None, degree=None, sourceLeafSize=None, targetLeafSize=None,
                   sizeCheck=None, precision=None):
    """Treecode convolution; returns a new float64 array of length numTargets.

    Argument handling follows BaryTreeInterface.py:98-137: either ``beta``
    (truthy) or all of theta, degree, sourceLeafSize and targetLeafSize must
    be given; sizeCheck defaults to 1.0 for LAGRANGE (4.0 for HERMITE).
    """
    if beta:
        theta = -1.0
        degree = -1
        sourceLeafSize = 1
        targetLeafSize = 1
    else:
        assert theta is not None, "If beta isn't provided, theta must be."
        assert degree is not None, "If beta isn't provided, degree must be."
        assert sourceLeafSize is not None, "If beta isn't provided, sourceLeafSize must be."
        assert targetLeafSize is not None, "If beta isn't provided, targetLeafSize must be."
        beta = -1

    if not sizeCheck:
        if approximationName == Approximation.LAGRANGE:
            sizeCheck = 1.0
        if approximationName == Approximation.HERMITE:
            sizeCheck = 4.0

    if GPUpresent is not True and GPUpresent is not False:
        print("What should GPUpresent be set to in the wrapper?")
        exit(-1)

    arrays = [_as_c_double(a, n) for a, n in (
        (targetX, "targetX"), (targetY, "targetY"), (targetZ, "targetZ"),
        (targetValue, "targetValue"), (sourceX, "sourceX"), (sourceY, "sourceY"),
        (sourceZ, "sourceZ"), (sourceValue, "sourceValue"), (sourceWeight, "sourceWeight"))]
    kp = _as_c_double(np.atleast_1d(np.asarray(kernelParameters, dtype=np.float64)),
                      "kernelParameters")
    resultArray = np.zeros(numTargets)

    L = _native.lib()
    if precision is None:
        prec = int(L.tagi_get_precision())
    else:
        prec = _PRECISION[precision]
    L.tagi_clear_error()
    rc = L.tagi_BaryTreeInterface_ex(
        ctypes.c_int(numTargets), ctypes.c_int(numSources),
        *[_native.dptr(a) for a in arrays], _native.dptr(resultArray),
        ctypes.c_int(int(kernelName)), ctypes.c_int(numberOfKernelParameters), _native.dptr(kp),
        ctypes.c_int(int(singularityHandling)), ctypes.c_int(int(approximationName)),
        ctypes.c_int(int(computeType)), ctypes.c_double(theta), ctypes.c_int(degree),
        ctypes.c_int(sourceLeafSize), ctypes.c_int(targetLeafSize), ctypes.c_double(sizeCheck),
        ctypes.c_double(beta), ctypes.c_int(verbosity), ctypes.c_int(prec))
    _native.check(rc)
    return resultArray
