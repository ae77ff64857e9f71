"""ctypes binding of libtagi_gb300.so (the C ABI declared in include/tagi_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present, calls fail with an exception naming the problem.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtagi_gb300.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double

TAGI_OK, TAGI_ERR_ARG, TAGI_ERR_CUDA, TAGI_ERR_UNSUPPORTED, TAGI_ERR_DEVICE, TAGI_ERR_STATE = range(6)
PREC_MIXED, PREC_FP64 = 0, 1

_treecode_params = [_i, _i, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _i, _i, _dp, _i, _i, _i,
                    _d, _i, _i, _i, _d, _d, _i]

SIGNATURES = {
    "BaryTreeInterface": (None, _treecode_params),
    "tagi_BaryTreeInterface_ex": (_i, _treecode_params + [_i]),
    "modifiedGramSchmidt_singleWavefunction": (None, [_dp, _dp, _dp, _i, _i, _i]),
    "InterpolateBetweenTwoMeshes": (None, [_dp, _dp, _dp, _dp, _ip, _i, _dp, _dp, _dp, _dp, _ip, _i,
                                           _i, _i]),
    "tagi_treecode_dev": (_i, [_i, _i] + [_vp] * 10 + [_i, _i, _dp, _i, _i, _i, _d, _i, _i, _i, _d,
                                                       _d, _i, _i, _vp]),
    "tagi_plan_create": (_i, [ctypes.POINTER(_vp), _i, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _d, _i,
                              _i, _i, _d, _vp]),
    "tagi_plan_destroy": (_i, [_vp]),
    "tagi_plan_convolve": (_i, [_vp, _i, _vp, _vp, _vp, _i, _i, _dp, _i, _i, _vp]),
    "tagi_plan_convolve_ex": (_i, [_vp, _i, _vp, _vp, _vp, _i, _i, _vp, _i, _i, _i, _i, _i, _vp]),
    "tagi_plan_check_parameters": (_i, [_vp, _ip, _vp]),
    "tagi_systems_create": (_i, [ctypes.POINTER(_vp), _i, ctypes.POINTER(_vp), _ip, _i, _i, _i, _i, _vp]),
    "tagi_systems_convolve": (_i, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp), _i,
                                   ctypes.POINTER(_vp), _i, _i, _vp]),
    "tagi_systems_info": (_i, [_vp, _ip]),
    "tagi_systems_destroy": (_i, [_vp]),
    "tagi_treecode_batched": (_i, [_i, _ip, _ip, _vp, _vp, _vp, _vp, _vp, _vp, _i, _dp, _i, _d, _i, _i, _i,
                                   _d, _i, _vp]),
    "tagi_graph_begin": (_i, [_vp]),
    "tagi_graph_end": (_i, [_vp, ctypes.POINTER(_vp)]),
    "tagi_graph_launch": (_i, [_vp, _vp]),
    "tagi_graph_nodes": (_i, [_vp, _ip]),
    "tagi_graph_destroy": (_i, [_vp]),
    "tagi_gi_workspace_doubles": (ctypes.c_longlong, [ctypes.c_longlong, _i]),
    "tagi_gi_source": (_i, [_vp, _vp, ctypes.c_longlong, _i, _vp, _vp]),
    "tagi_gi_update": (_i, [_vp, _vp, _vp, _vp, ctypes.c_longlong, _i, _d, _vp, _vp, _vp, _d, _vp, _vp, _vp,
                            ctypes.c_longlong, _vp]),
    "tagi_gi_residual": (_i, [_vp, _vp, _vp, ctypes.c_longlong, _i, _vp, _vp, _vp, _vp, _vp, ctypes.c_longlong,
                              _vp]),
    "tagi_wdot_rows": (_i, [_vp, ctypes.c_longlong, _vp, ctypes.c_longlong, _vp, ctypes.c_longlong, _i, _vp, _vp,
                            ctypes.c_longlong, _vp]),
    "tagi_scf_density": (_i, [_vp, _vp, _i, ctypes.c_longlong, _vp, _d, _vp, _vp, ctypes.c_longlong, _vp]),
    "tagi_lda_exchange": (_i, [_vp, ctypes.c_longlong, _vp, _vp, _vp]),
    "tagi_veff": (_i, [_vp, _vp, _vp, _d, ctypes.c_longlong, _vp, _vp]),
    "tagi_anderson_combine": (_i, [_vp, _vp, _i, _i, _vp, _vp, _d, ctypes.c_longlong, _vp, _vp]),
    "tagi_mlp_gemm": (_i, [_vp, ctypes.c_longlong, ctypes.c_longlong, _vp, ctypes.c_longlong, ctypes.c_longlong,
                           _i, _i, _i, _i, _vp, _vp, ctypes.c_longlong, _vp, _vp, _vp]),
    "tagi_mlp_gemm_splitk": (_i, [_vp, ctypes.c_longlong, ctypes.c_longlong, _vp, ctypes.c_longlong,
                                  ctypes.c_longlong, _i, _i, _i, _i, _vp, _vp, _vp]),
    "tagi_mlp_patch_features": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, ctypes.c_longlong, _i, _vp, _vp, _vp, _vp]),
    "tagi_mlp_patch_target": (_i, [_vp, _vp, _i, _i, _i, ctypes.c_longlong, _vp, _vp]),
    "tagi_mlp_mse_grad": (_i, [_vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "tagi_mlp_colsum_workspace": (ctypes.c_longlong, [ctypes.c_longlong, _i]),
    "tagi_mlp_colsum": (_i, [_vp, _i, ctypes.c_longlong, _i, _vp, _vp, ctypes.c_longlong, _vp]),
    "tagi_mlp_adam": (_i, [_vp, _vp, _vp, _vp, ctypes.c_longlong, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                           ctypes.c_float, _i, _vp, _vp]),
    "tagi_mlp_patch_apply": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _i, ctypes.c_longlong, _vp, _vp, _vp]),
    "tagi_mlp_to_bf16": (_i, [_vp, ctypes.c_longlong, _vp, _vp]),
    "tagi_gi_anderson_workspace_doubles": (ctypes.c_longlong, [ctypes.c_longlong, _i, _i]),
    "tagi_gi_anderson_gram": (_i, [_vp, _i, _i, ctypes.c_longlong, _vp, _vp, _vp, ctypes.c_longlong, _vp]),
    "tagi_gi_anderson_mix": (_i, [_vp, _vp, _i, _i, _vp, _vp, _d, _i, ctypes.c_longlong, _vp, _vp]),
    "tagi_plan_info": (_i, [_vp, _dp]),
    "tagi_plan_get_tree": (_i, [_vp, _i, _u64p, _ip, _ip, _ip, _ip, _ip, _ip, _dp, _dp, _dp]),
    "tagi_plan_get_lists": (_i, [_vp, _ip, _ip, _ip, _ip, _ip, _ip]),
    "tagi_plan_get_charges": (_i, [_vp, _i, _i, _dp]),
    "tagi_direct_dev": (_i, [_i, _vp, _vp, _vp, _vp, _i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i,
                             _dp, _i, _vp]),
    "tagi_mgs_dev": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp]),
    "tagi_mgs_dev_noalloc": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp]),
    "tagi_interp_dev": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp]),
    "tagi_mesh_refine": (_i, [_vp, _i, _vp, _i, _i, _d, _d, _d, _d, _i, _i] + [_vp] * 8 +
                         [_i, _ip, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), _vp]),
    "tagi_mesh_points": (_i, [_vp] * 7 + [_i, _i, _dp, _dp] + [_vp] * 4 + [ctypes.c_longlong] + [_vp] * 4 +
                         [ctypes.c_longlong, _vp]),
    "tagi_set_precision": (_i, [_i]),
    "tagi_get_precision": (_i, []),
    "tagi_beta_parameters": (_i, [_d, _dp, _ip, _ip, _ip]),
    "tagi_orbitals_per_item": (_i, [_i, _i, _i, _i, _i, _ip]),
    "tagi_launch_count": (ctypes.c_longlong, []),
    "tagi_pair_peak": (_i, [_i, _i, _i, _d, _dp, _vp]),
    "tagi_pipe_rates": (_i, [_dp, _vp]),
    "tagi_profile": (_i, [_i]),
    "tagi_profile_read": (_i, [_dp, ctypes.POINTER(ctypes.c_longlong), _i]),
    "tagi_last_error": (_i, []),
    "tagi_last_error_message": (ctypes.c_char_p, []),
    "tagi_clear_error": (None, []),
    "tagi_version": (_i, []),
}

_LIB = None


class TagiError(RuntimeError):
    """A libtagi_gb300 entry point returned a nonzero status."""

    def __init__(self, code, message):
        super().__init__(f"libtagi_gb300 error {code}: {message}")
        self.code = code


def lib():
    """Load the library (once).  Raises if it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; "
                "g.build()' or python build.py in the package directory); there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def last_error():
    L = lib()
    return int(L.tagi_last_error()), (L.tagi_last_error_message() or b"").decode(errors="replace")


def check(rc):
    """Raise TagiError for a nonzero status."""
    if rc:
        code, msg = last_error()
        raise TagiError(rc, msg or f"status {rc}")
    return rc


def check_void_call():
    """For the void drop-ins: raise if the call recorded an error."""
    code, msg = last_error()
    if code:
        raise TagiError(code, msg)


def dptr(a):
    """numpy float64 array -> POINTER(c_double) (array must be C-contiguous)."""
    return a.ctypes.data_as(_dp)


def iptr(a):
    return a.ctypes.data_as(_ip)
