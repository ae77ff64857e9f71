"""Device-resident API over torch CUDA tensors (torch supplies memory and the
stream; all arithmetic is in libtagi_gb300.so).

``TreecodePlan`` holds the part of a callTreedriver call that depends only on
the mesh (trees, lists, proxy grids, weight charges), so a Green-iteration
sweep re-uses it for every orbital and every iteration; ``convolve`` takes one
or many charge vectors (batched orbitals, one k_i each) in one launch
sequence.
"""
import ctypes

import numpy as np
import torch

try:
    from . import _native
    from .BaryTreeInterface import Kernel, Singularity
except ImportError:
    import _native
    from BaryTreeInterface import Kernel, Singularity

PRECISION = {"mixed": _native.PREC_MIXED, "fp64": _native.PREC_FP64}


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _dev(t, name, dtype=torch.float64):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}")
    if not t.is_contiguous():
        raise TypeError(f"{name} must be contiguous")
    return ctypes.c_void_p(t.data_ptr())


def _kp_array(params, norb):
    kp = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(norb, -1))
    return kp, kp.shape[1]


class TreecodePlan:
    """Trees + interaction lists + proxy data for fixed targets/sources/weights."""

    def __init__(self, tx, ty, tz, sx, sy, sz, sw, theta=0.7, degree=7, source_leaf=500,
                 target_leaf=500, size_check=1.0, stream=None):
        self.nt, self.ns = int(tx.numel()), int(sx.numel())
        self.device = tx.device
        h = ctypes.c_void_p()
        L = _native.lib()
        _native.check(L.tagi_plan_create(
            ctypes.byref(h), self.nt, _dev(tx, "tx"), _dev(ty, "ty"), _dev(tz, "tz"), self.ns,
            _dev(sx, "sx"), _dev(sy, "sy"), _dev(sz, "sz"), _dev(sw, "sw"), float(theta),
            int(degree), int(source_leaf), int(target_leaf), float(size_check), _stream(stream)))
        self._h = h
        self.theta, self.degree = theta, degree
        self.source_leaf, self.target_leaf, self.size_check = source_leaf, target_leaf, size_check

    @classmethod
    def for_mesh(cls, x, y, z, w, **kw):
        """Targets = sources = mesh points (the Green-iteration case)."""
        return cls(x, y, z, x, y, z, w, **kw)

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().tagi_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def convolve(self, target_values, source_values, kernel=Kernel.YUKAWA, kernel_params=(1.0,),
                 singularity=Singularity.SUBTRACTION, precision="mixed", out=None, stream=None,
                 orbitals_per_item=0, targets_per_thread=0):
        """target_values [norb, nt] (or [nt]), source_values [norb, ns] -> [norb, nt].

        kernel_params: one row per orbital (k_i for Yukawa, alpha for Coulomb
        subtraction); a single row is broadcast.  A float64 CUDA tensor of
        norb values is read on the device when the call runs (the form for
        graph capture; see check_parameters)."""
        squeeze = target_values.dim() == 1
        tv = target_values.reshape(-1, self.nt)
        sv = source_values.reshape(-1, self.ns)
        norb = tv.shape[0]
        if sv.shape[0] != norb:
            raise ValueError("target_values and source_values hold different orbital counts")
        if out is None:
            out = torch.empty((norb, self.nt), dtype=torch.float64, device=self.device)
        if isinstance(kernel_params, torch.Tensor) and kernel_params.is_cuda:
            if kernel_params.numel() != norb:
                raise ValueError("device kernel_params needs one value per orbital")
            kptr, nkp, on_dev, keep = _dev(kernel_params, "kernel_params"), 1, 1, None
        else:
            kp = np.asarray(kernel_params, dtype=np.float64)
            if kp.ndim == 0:
                kp = np.full((norb, 1), float(kp))
            elif kp.ndim == 1:
                # one value per orbital, or one parameter row shared by all orbitals
                kp = kp[:, None] if (norb > 1 and kp.size == norb) else np.broadcast_to(kp, (norb, kp.size))
            elif kp.shape[0] != norb:
                raise ValueError("kernel_params needs one row per orbital")
            keep, nkp = _kp_array(kp, norb)
            kptr, on_dev = ctypes.c_void_p(keep.ctypes.data), 0
        _native.check(_native.lib().tagi_plan_convolve_ex(
            self._h, norb, _dev(tv, "target_values"), _dev(sv, "source_values"), _dev(out, "out"),
            int(kernel), nkp, kptr, on_dev, int(singularity), PRECISION[precision],
            int(orbitals_per_item), int(targets_per_thread), _stream(stream)))
        del keep
        return out[0] if squeeze else out

    def check_parameters(self, stream=None):
        """True if a call since the last check met an unusable device kernel parameter."""
        f = ctypes.c_int(0)
        _native.check(_native.lib().tagi_plan_check_parameters(self._h, ctypes.byref(f), _stream(stream)))
        return bool(f.value)

    def info(self):
        v = np.zeros(13)
        _native.check(_native.lib().tagi_plan_info(self._h, _native.dptr(v)))
        keys = ("src_nodes", "tgt_nodes", "batches", "near_entries", "far_entries", "slots", "P",
                "upward_items", "near_ranges", "max_batch", "near_pairs", "far_pairs",
                "near_close_pairs")
        return {k: (float(x) if k.endswith("pairs") else int(x)) for k, x in zip(keys, v)}

    def tree(self, which):
        inf = self.info()
        n = self.ns if which == 0 else self.nt
        nn = inf["src_nodes"] if which == 0 else inf["tgt_nodes"]
        out = dict(codes=np.zeros(n, np.uint64), perm=np.zeros(n, np.int32),
                   begin=np.zeros(nn, np.int32), end=np.zeros(nn, np.int32),
                   parent=np.zeros(nn, np.int32), first_child=np.zeros(nn, np.int32),
                   nchild=np.zeros(nn, np.int32), center=np.zeros(3 * nn), half=np.zeros(3 * nn),
                   radius=np.zeros(nn))
        _native.check(_native.lib().tagi_plan_get_tree(
            self._h, which, out["codes"].ctypes.data_as(_native._u64p), _native.iptr(out["perm"]),
            _native.iptr(out["begin"]), _native.iptr(out["end"]), _native.iptr(out["parent"]),
            _native.iptr(out["first_child"]), _native.iptr(out["nchild"]),
            _native.dptr(out["center"]), _native.dptr(out["half"]), _native.dptr(out["radius"])))
        return out

    def lists(self):
        inf = self.info()
        nb = inf["batches"]
        out = dict(batch_node=np.zeros(nb, np.int32), near_off=np.zeros(nb + 1, np.int32),
                   near_list=np.zeros(max(inf["near_entries"], 1), np.int32),
                   far_off=np.zeros(nb + 1, np.int32),
                   far_list=np.zeros(max(inf["far_entries"], 1), np.int32),
                   slot_node=np.zeros(max(inf["slots"], 1), np.int32))
        _native.check(_native.lib().tagi_plan_get_lists(
            self._h, *[_native.iptr(out[k]) for k in ("batch_node", "near_off", "near_list",
                                                      "far_off", "far_list", "slot_node")]))
        out["near_list"] = out["near_list"][: inf["near_entries"]]
        out["far_list"] = out["far_list"][: inf["far_entries"]]
        out["slot_node"] = out["slot_node"][: inf["slots"]]
        return out

    def charges(self, which, norb=1):
        """which 0: weight charges; 1: last FP64 call's charges; 2: last mixed call's."""
        inf = self.info()
        n = inf["slots"] * inf["P"] * (1 if which == 0 else norb)
        out = np.zeros(max(n, 1))
        _native.check(_native.lib().tagi_plan_get_charges(self._h, which, norb, _native.dptr(out)))
        shape = (inf["slots"], inf["P"]) if which == 0 else (norb, inf["slots"], inf["P"])
        return out[:n].reshape(shape)


def treecode(tx, ty, tz, tv, sx, sy, sz, sv, sw, kernel, kernel_params, singularity, theta,
             degree, source_leaf, target_leaf, size_check=1.0, precision="mixed", beta=-1.0,
             verbosity=0, out=None, stream=None):
    """One-shot treecode on device tensors (tagi_treecode_dev)."""
    nt, ns = int(tx.numel()), int(sx.numel())
    kp = np.ascontiguousarray(np.atleast_1d(np.asarray(kernel_params, dtype=np.float64)))
    if out is None:
        out = torch.empty(nt, dtype=torch.float64, device=tx.device)
    _native.check(_native.lib().tagi_treecode_dev(
        nt, ns, _dev(tx, "tx"), _dev(ty, "ty"), _dev(tz, "tz"), _dev(tv, "tv"), _dev(sx, "sx"),
        _dev(sy, "sy"), _dev(sz, "sz"), _dev(sv, "sv"), _dev(sw, "sw"), _dev(out, "out"),
        int(kernel), len(kp), _native.dptr(kp), int(singularity), 1, 1, float(theta), int(degree),
        int(source_leaf), int(target_leaf), float(size_check), float(beta), int(verbosity),
        PRECISION[precision], _stream(stream)))
    return out


def direct(tx, ty, tz, tv, sx, sy, sz, sv, sw, kernel, kernel_params, singularity, subset=None,
           stream=None):
    """Exact FP64 direct sum at the targets in ``subset`` (int32 CUDA tensor) or all."""
    nt, ns = int(tx.numel()), int(sx.numel())
    kp = np.ascontiguousarray(np.atleast_1d(np.asarray(kernel_params, dtype=np.float64)))
    nsub = nt if subset is None else int(subset.numel())
    out = torch.empty(nsub, dtype=torch.float64, device=tx.device)
    sub = ctypes.c_void_p(0) if subset is None else _dev(subset, "subset", torch.int32)
    _native.check(_native.lib().tagi_direct_dev(
        nt, _dev(tx, "tx"), _dev(ty, "ty"), _dev(tz, "tz"), _dev(tv, "tv"), nsub, sub, ns,
        _dev(sx, "sx"), _dev(sy, "sy"), _dev(sz, "sz"), _dev(sv, "sv"), _dev(sw, "sw"),
        _dev(out, "out"), int(kernel), _native.dptr(kp), int(singularity), _stream(stream)))
    return out


def mgs(V, U, W, target, stream=None):
    """In-place weighted Gram-Schmidt of U against rows < target of V; U -> V[target]."""
    nw, n = V.shape
    _native.check(_native.lib().tagi_mgs_dev(_dev(V, "V"), _dev(U, "U"), _dev(W, "W"), int(target),
                                             int(n), int(nw), _stream(stream)))
    return U


def interp(cX, cY, cZ, cF, ppc_c, fX, fY, fZ, ppc_f, ncells, order, fineF=None, stream=None):
    """Device form of InterpolateBetweenTwoMeshes; returns fineF (accumulated into)."""
    if fineF is None:
        fineF = torch.zeros(fX.numel(), dtype=torch.float64, device=fX.device)
    _native.check(_native.lib().tagi_interp_dev(
        _dev(cX, "cX"), _dev(cY, "cY"), _dev(cZ, "cZ"), _dev(cF, "cF"),
        _dev(ppc_c, "ppc_c", torch.int32), int(cX.numel()), _dev(fX, "fX"), _dev(fY, "fY"),
        _dev(fZ, "fZ"), _dev(fineF, "fineF"), _dev(ppc_f, "ppc_f", torch.int32), int(fX.numel()),
        int(ncells), int(order), _stream(stream)))
    return fineF


class Systems:
    """Several plans (meshes), each with its own orbital count, convolved in
    one persistent launch per field pass (tagi_systems_*).  Plans are borrowed:
    keep them alive while this object is used."""

    def __init__(self, plans, num_orbitals, kernel=Kernel.YUKAWA, precision="mixed",
                 orbitals_per_item=0, targets_per_thread=0, stream=None):
        self.plans = list(plans)
        self.norb = [int(n) for n in num_orbitals]
        if len(self.plans) != len(self.norb):
            raise ValueError("one orbital count per plan")
        self.kernel, self.precision = int(kernel), precision
        n = len(self.plans)
        hp = (ctypes.c_void_p * n)(*[p._h.value for p in self.plans])
        no = (ctypes.c_int * n)(*self.norb)
        h = ctypes.c_void_p()
        _native.check(_native.lib().tagi_systems_create(
            ctypes.byref(h), n, hp, no, self.kernel, PRECISION[precision], int(orbitals_per_item),
            int(targets_per_thread), _stream(stream)))
        self._h = h

    def info(self):
        v = (ctypes.c_int * 5)()
        _native.check(_native.lib().tagi_systems_info(self._h, v))
        return dict(systems=v[0], orbitals_per_item=v[1], near_items=v[2], close_items=v[3],
                    far_items=v[4])

    def convolve(self, target_values, source_values, kernel_params, singularity=Singularity.SUBTRACTION,
                 outs=None, stream=None):
        """Lists (one entry per system) of [norb_s, n_s] device tensors; kernel_params:
        per system a sequence of norb_s host values, or a float64 CUDA tensor of them."""
        n = len(self.plans)
        if outs is None:
            outs = [torch.empty((self.norb[i], self.plans[i].nt), dtype=torch.float64,
                                device=self.plans[i].device) for i in range(n)]
        on_dev = all(isinstance(k, torch.Tensor) and k.is_cuda for k in kernel_params)
        keep = []
        kps = []
        for i, k in enumerate(kernel_params):
            if on_dev:
                if k.numel() != self.norb[i]:
                    raise ValueError(f"system {i}: one kernel parameter per orbital")
                kps.append(_dev(k, "kernel_params").value)
            else:
                a = np.ascontiguousarray(np.asarray(k, dtype=np.float64).reshape(-1))
                if a.size != self.norb[i]:
                    raise ValueError(f"system {i}: one kernel parameter per orbital")
                keep.append(a)
                kps.append(a.ctypes.data)
        VP = ctypes.c_void_p * n
        tv = VP(*[_dev(t.reshape(self.norb[i], -1), "target_values").value
                  for i, t in enumerate(target_values)])
        sv = VP(*[_dev(t.reshape(self.norb[i], -1), "source_values").value
                  for i, t in enumerate(source_values)])
        ov = VP(*[_dev(o, "out").value for o in outs])
        _native.check(_native.lib().tagi_systems_convolve(
            self._h, tv, sv, ov, 1, VP(*kps), 1 if on_dev else 0, int(singularity), _stream(stream)))
        del keep
        return outs

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().tagi_systems_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def treecode_batched(point_offsets, num_orbitals, x, y, z, w, values, kernel, kernel_params, singularity,
                     theta=0.7, degree=7, source_leaf=500, target_leaf=500, size_check=1.0,
                     precision="mixed", out=None, stream=None):
    """One-shot tagi_treecode_batched over concatenated meshes (targets = sources)."""
    ns = len(num_orbitals)
    off = np.ascontiguousarray(point_offsets, dtype=np.int32)
    no = np.ascontiguousarray(num_orbitals, dtype=np.int32)
    kp = np.ascontiguousarray(kernel_params, dtype=np.float64)
    if out is None:
        out = torch.empty_like(values)
    _native.check(_native.lib().tagi_treecode_batched(
        ns, _native.iptr(off), _native.iptr(no), _dev(x, "x"), _dev(y, "y"), _dev(z, "z"), _dev(w, "w"),
        _dev(values, "values"), _dev(out, "out"), int(kernel), _native.dptr(kp), int(singularity),
        float(theta), int(degree), int(source_leaf), int(target_leaf), float(size_check),
        PRECISION[precision], _stream(stream)))
    return out


class Graph:
    """CUDA graph of a captured call sequence (tagi_graph_*).

        with Graph.capture(stream) as g:
            plan.convolve(..., kernel_params=k_dev, stream=stream)
        g.replay(stream)

    Every call inside must have been made once before, uncaptured, with the
    same orbital counts and precision; kernel parameters must be CUDA tensors."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def capture(cls, stream):
        return _Capture(stream)

    def replay(self, stream):
        _native.check(_native.lib().tagi_graph_launch(self._h, _stream(stream)))

    def nodes(self):
        n = ctypes.c_int(0)
        _native.check(_native.lib().tagi_graph_nodes(self._h, ctypes.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "_h", None):
            _native.lib().tagi_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Capture:
    def __init__(self, stream):
        if stream is None:
            raise ValueError("graph capture needs a created stream (torch.cuda.Stream())")
        self.stream = stream
        self.graph = None

    def __enter__(self):
        _native.check(_native.lib().tagi_graph_begin(_stream(self.stream)))
        self.graph = Graph(None)
        return self.graph

    def __exit__(self, et, ev, tb):
        h = ctypes.c_void_p()
        rc = _native.lib().tagi_graph_end(_stream(self.stream), ctypes.byref(h))
        if et is None:
            _native.check(rc)
            self.graph._h = h
        elif rc == 0:
            _native.lib().tagi_graph_destroy(h)
        return False
