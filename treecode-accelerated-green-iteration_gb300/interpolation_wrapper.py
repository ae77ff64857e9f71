"""Drop-in for 3D-GreenIteration/src/utilities/interpolation_wrapper.py.

``callInterpolator`` keeps the reference's signature and return value
(interpolation_wrapper.py:46-93 -> TwoMeshInterpolation.c:163-234): a new
float64 array of fine-mesh values interpolated cell by cell from the coarse
mesh.  The work runs in libtagi_gb300.so on the GPU; ``gpuPresent`` is
accepted for compatibility.
"""
import numpy as np

try:
    from . import _native
except ImportError:
    import _native


def callInterpolator(coarseX, coarseY, coarseZ, coarseF, pointsPerCoarseCell,
                     fineX, fineY, fineZ, pointsPerFineCell, numberOfCells, order, gpuPresent):
    pointsPerCoarseCell = np.ascontiguousarray(pointsPerCoarseCell, dtype=np.int32)
    pointsPerFineCell = np.ascontiguousarray(pointsPerFineCell, dtype=np.int32)
    arrs = []
    for a, n in ((coarseX, "coarseX"), (coarseY, "coarseY"), (coarseZ, "coarseZ"),
                 (coarseF, "coarseF"), (fineX, "fineX"), (fineY, "fineY"), (fineZ, "fineZ")):
        a = np.asarray(a)
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise TypeError(f"{n} must be a C-contiguous float64 array")
        arrs.append(a)
    cX, cY, cZ, cF, fX, fY, fZ = arrs
    fineF = np.zeros(len(fX))
    L = _native.lib()
    L.tagi_clear_error()
    L.InterpolateBetweenTwoMeshes(_native.dptr(cX), _native.dptr(cY), _native.dptr(cZ),
                                  _native.dptr(cF), _native.iptr(pointsPerCoarseCell), len(cX),
                                  _native.dptr(fX), _native.dptr(fY), _native.dptr(fZ),
                                  _native.dptr(fineF), _native.iptr(pointsPerFineCell), len(fX),
                                  int(numberOfCells), int(order))
    _native.check_void_call()
    return fineF
