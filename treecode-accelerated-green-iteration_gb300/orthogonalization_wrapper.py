"""Drop-in for 3D-GreenIteration/src/utilities/orthogonalization_wrapper.py.

``callOrthogonalization(wavefunctions, target, W, targetWavefunction,
gpuPresent)`` keeps the reference's signature and in-place semantics
(orthogonalization_wrapper.py:43-74 -> Orthogonalization.c:14-119): ``target``
is orthogonalized against rows 0..targetWavefunction-1 of ``wavefunctions``
in the W-weighted inner product, normalized, and written to ``target`` and to
row targetWavefunction.  The work runs in libtagi_gb300.so on the GPU
(host arrays are copied in and out); ``gpuPresent`` is accepted for
compatibility.  For device-resident orbitals use ``device.mgs``.
"""
import numpy as np

try:
    from . import _native
except ImportError:
    import _native


def callOrthogonalization(wavefunctions, target, W, targetWavefunction, gpuPresent):
    numWavefunctions, numPoints = np.shape(wavefunctions)
    for a, n in ((wavefunctions, "wavefunctions"), (target, "target"), (W, "W")):
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise TypeError(f"{n} must be a C-contiguous float64 array")
    L = _native.lib()
    L.tagi_clear_error()
    L.modifiedGramSchmidt_singleWavefunction(_native.dptr(wavefunctions), _native.dptr(target),
                                             _native.dptr(W), int(targetWavefunction),
                                             int(numPoints), int(numWavefunctions))
    _native.check_void_call()
    return
