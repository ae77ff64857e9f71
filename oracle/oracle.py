"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the cpu_baseline leg of bench.py
import this module, and only as the checker or the timed CPU baseline.

* ``liboracle.so`` (built from ``tagi_oracle.c``): FP64 direct sum, the
  project-defined FP64 treecode (same tree/list rules as the device), and
  restatements of the reference's MGS (Orthogonalization.c:14-119) and
  two-mesh interpolation (TwoMeshInterpolation.c:12-234).
* ``_ref/libref_orth.so`` / ``_ref/libref_interp.so``: the reference's own
  C sources compiled here (``make -C oracle ref``) when the reference tree is
  present.  They are absent on machines without the reference; callers skip.

Treecode parity against BaryTree itself is unpinned (BaryTree is not part of
the reference); MGS and interpolation are pinned by the compiled reference C
and by the golden vectors in tests/golden/.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = {}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def build(ref=False):
    """Compile liboracle.so (and, when asked and present, the reference C)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.oracle_direct.restype = None
        L.oracle_plan_create.restype = ctypes.c_void_p
        L.oracle_plan_create.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _dp, _dp, _dp,
                                         _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_double]
        L.oracle_plan_destroy.argtypes = [ctypes.c_void_p]
        L.oracle_plan_info.argtypes = [ctypes.c_void_p, _ip]
        L.oracle_plan_get_tree.argtypes = [ctypes.c_void_p, ctypes.c_int, _u64p, _ip, _ip, _ip, _ip,
                                           _ip, _ip, _dp, _dp, _dp]
        L.oracle_plan_get_lists.argtypes = [ctypes.c_void_p, _ip, _ip, _ip, _ip, _ip, _ip]
        L.oracle_plan_modified_charges.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.oracle_plan_weight_charges.argtypes = [ctypes.c_void_p, _dp]
        L.oracle_plan_convolve.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int, _dp,
                                           ctypes.c_int, _dp, ctypes.c_int]
        L.oracle_plan_convolve_batches.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int, _dp,
                                                   ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int,
                                                   _ip, _dp, _dp]
        L.oracle_plan_convolve_batches_timed.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int, _dp,
                                                         ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int,
                                                         _ip, _dp, _dp, _dp]
        L.oracle_mgs.argtypes = [_dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_interp.argtypes = [_dp, _dp, _dp, _dp, _ip, ctypes.c_int, _dp, _dp, _dp, _dp,
                                    _ip, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _LIB = L
    return _LIB


def _c(a, dt=np.float64):
    return np.ascontiguousarray(a, dtype=dt)


def direct(tx, ty, tz, tv, sx, sy, sz, sv, sw, kernel, kparams, singularity, subset=None,
           nthreads=0):
    """FP64 direct sum; returns values at ``subset`` (all targets if None)."""
    tx, ty, tz, tv = map(_c, (tx, ty, tz, tv))
    sx, sy, sz, sv, sw = map(_c, (sx, sy, sz, sv, sw))
    kp = _c(np.atleast_1d(kparams))
    if subset is None:
        sub = None
        nsub = len(tx)
    else:
        sub = _c(subset, np.int32)
        nsub = len(sub)
    out = np.zeros(nsub)
    lib().oracle_direct(ctypes.c_int(len(tx)), _p(tx), _p(ty), _p(tz), _p(tv), ctypes.c_int(len(sx)),
                        _p(sx), _p(sy), _p(sz), _p(sv), _p(sw), ctypes.c_int(int(kernel)), _p(kp),
                        ctypes.c_int(int(singularity)), ctypes.c_int(nsub),
                        _p(sub, _ip) if sub is not None else None, _p(out), ctypes.c_int(nthreads))
    return out


class Plan:
    """The project-defined FP64 treecode on the CPU (same rules as the device)."""

    def __init__(self, tx, ty, tz, sx, sy, sz, sw, theta, degree, source_leaf, target_leaf,
                 size_check=1.0):
        self._keep = [_c(a) for a in (tx, ty, tz, sx, sy, sz, sw)]
        tx, ty, tz, sx, sy, sz, sw = self._keep
        self.nt, self.ns = len(tx), len(sx)
        self.h = lib().oracle_plan_create(len(tx), _p(tx), _p(ty), _p(tz), len(sx), _p(sx), _p(sy),
                                          _p(sz), _p(sw), theta, degree, source_leaf, target_leaf,
                                          size_check)
        if not self.h:
            raise ValueError("oracle plan rejected its arguments")
        info = np.zeros(9, np.int32)
        lib().oracle_plan_info(self.h, _p(info, _ip))
        (self.n_src_nodes, self.n_tgt_nodes, self.n_batches, self.n_near, self.n_far,
         self.n_slots, self.src_levels, self.tgt_levels, self.P) = [int(v) for v in info]

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_plan_destroy(self.h)
            self.h = None

    def tree(self, which):
        n = self.ns if which == 0 else self.nt
        nn = self.n_src_nodes if which == 0 else self.n_tgt_nodes
        out = dict(codes=np.zeros(n, np.uint64), perm=np.zeros(n, np.int32),
                   begin=np.zeros(nn, np.int32), end=np.zeros(nn, np.int32),
                   parent=np.zeros(nn, np.int32), first_child=np.zeros(nn, np.int32),
                   nchild=np.zeros(nn, np.int32), center=np.zeros(3 * nn),
                   half=np.zeros(3 * nn), radius=np.zeros(nn))
        lib().oracle_plan_get_tree(self.h, which, _p(out["codes"], _u64p), _p(out["perm"], _ip),
                                   _p(out["begin"], _ip), _p(out["end"], _ip),
                                   _p(out["parent"], _ip), _p(out["first_child"], _ip),
                                   _p(out["nchild"], _ip), _p(out["center"]), _p(out["half"]),
                                   _p(out["radius"]))
        return out

    def lists(self):
        nb = self.n_batches
        out = dict(batch_node=np.zeros(nb, np.int32), near_off=np.zeros(nb + 1, np.int32),
                   near_list=np.zeros(max(self.n_near, 1), np.int32),
                   far_off=np.zeros(nb + 1, np.int32),
                   far_list=np.zeros(max(self.n_far, 1), np.int32),
                   slot_node=np.zeros(max(self.n_slots, 1), np.int32))
        lib().oracle_plan_get_lists(self.h, _p(out["batch_node"], _ip), _p(out["near_off"], _ip),
                                    _p(out["near_list"], _ip), _p(out["far_off"], _ip),
                                    _p(out["far_list"], _ip), _p(out["slot_node"], _ip))
        out["near_list"] = out["near_list"][: self.n_near]
        out["far_list"] = out["far_list"][: self.n_far]
        out["slot_node"] = out["slot_node"][: self.n_slots]
        return out

    def modified_charges(self, sv, sw):
        sv, sw = _c(sv), _c(sw)
        q = np.zeros(max(self.n_slots, 1) * self.P)
        lib().oracle_plan_modified_charges(self.h, _p(sv), _p(sw), _p(q))
        return q[: self.n_slots * self.P].reshape(self.n_slots, self.P)

    def weight_charges(self):
        q = np.zeros(max(self.n_slots, 1) * self.P)
        lib().oracle_plan_weight_charges(self.h, _p(q))
        return q[: self.n_slots * self.P].reshape(self.n_slots, self.P)

    def convolve(self, tv, sv, sw, kernel, kparams, singularity, nthreads=0):
        tv, sv, sw = _c(tv), _c(sv), _c(sw)
        kp = _c(np.atleast_1d(kparams))
        out = np.zeros(self.nt)
        lib().oracle_plan_convolve(self.h, _p(tv), _p(sv), _p(sw), int(kernel), _p(kp),
                                   int(singularity), _p(out), nthreads)
        return out


def convolve_batches(plan, tv, sv, sw, kernel, kparams, singularity, batches, nthreads=0, per_batch=False):
    """Convolve only the listed batches; returns (out, (t_upward, t_fields, thread_seconds_fields),
    (near, far pairs)): wall seconds of the upward pass and of the fields, and the fields' time
    summed over the batches (per-thread busy time, independent of load imbalance).  With
    per_batch, a fourth item: each listed batch's own seconds."""
    tv, sv, sw = _c(tv), _c(sv), _c(sw)
    kp = _c(np.atleast_1d(kparams))
    sel = _c(batches, np.int32)
    out = np.zeros(plan.nt)
    times = np.zeros(3)
    pairs = np.zeros(2)
    bs = np.zeros(max(len(sel), 1))
    lib().oracle_plan_convolve_batches_timed(plan.h, _p(tv), _p(sv), _p(sw), int(kernel), _p(kp),
                                             int(singularity), _p(out), nthreads, len(sel), _p(sel, _ip),
                                             _p(times), _p(pairs), _p(bs))
    if per_batch:
        return out, tuple(times), tuple(pairs), bs[: len(sel)]
    return out, tuple(times), tuple(pairs)


def mgs(V, U, W, target):
    """In place on V (row ``target``) and U, like Orthogonalization.c:14."""
    assert V.flags.c_contiguous and V.dtype == np.float64
    nw, n = V.shape
    lib().oracle_mgs(_p(V), _p(U), _p(_c(W)), target, n, nw)


def interp(cX, cY, cZ, cF, ppc_c, fX, fY, fZ, ppc_f, ncells, order, fineF=None):
    ppc_c, ppc_f = _c(ppc_c, np.int32), _c(ppc_f, np.int32)
    cX, cY, cZ, cF, fX, fY, fZ = map(_c, (cX, cY, cZ, cF, fX, fY, fZ))
    fF = np.zeros(len(fX)) if fineF is None else _c(fineF).copy()
    lib().oracle_interp(_p(cX), _p(cY), _p(cZ), _p(cF), _p(ppc_c, _ip), len(cX), _p(fX), _p(fY),
                        _p(fZ), _p(fF), _p(ppc_f, _ip), len(fX), ncells, order)
    return fF


# ---------------------------------------------------------------------------
# The reference's own C, compiled from its sources (present only where the
# reference tree was available at build time).
# ---------------------------------------------------------------------------
def ref_available():
    return all(os.path.exists(os.path.join(HERE, "_ref", f))
               for f in ("libref_orth.so", "libref_interp.so"))


def _ref(name):
    if name not in _REF:
        _REF[name] = ctypes.CDLL(os.path.join(HERE, "_ref", name))
    return _REF[name]


def ref_mgs(V, U, W, target):
    """modifiedGramSchmidt_singleWavefunction from Orthogonalization.c (compiled)."""
    nw, n = V.shape
    f = _ref("libref_orth.so").modifiedGramSchmidt_singleWavefunction
    f.argtypes = [_dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    f(_p(V), _p(U), _p(_c(W)), target, n, nw)


def ref_interp(cX, cY, cZ, cF, ppc_c, fX, fY, fZ, ppc_f, ncells, order, fineF=None):
    """InterpolateBetweenTwoMeshes from TwoMeshInterpolation.c (compiled)."""
    ppc_c, ppc_f = _c(ppc_c, np.int32), _c(ppc_f, np.int32)
    cX, cY, cZ, cF, fX, fY, fZ = map(_c, (cX, cY, cZ, cF, fX, fY, fZ))
    fF = np.zeros(len(fX)) if fineF is None else _c(fineF).copy()
    f = _ref("libref_interp.so").InterpolateBetweenTwoMeshes
    f.argtypes = [_dp, _dp, _dp, _dp, _ip, ctypes.c_int, _dp, _dp, _dp, _dp, _ip, ctypes.c_int,
                  ctypes.c_int, ctypes.c_int]
    f(_p(cX), _p(cY), _p(cZ), _p(cF), _p(ppc_c, _ip), len(cX), _p(fX), _p(fY), _p(fZ), _p(fF),
      _p(ppc_f, _ip), len(fX), ncells, order)
    return fF
