"""Green iteration on the device: all orbitals of one mesh per sweep.

One sweep (greenIterationFixedPoint.py:155-484, every orbital at once):

    f_m      = -2 psi_m V_eff
    c_m      = G_{k_m} * f_m          one batched Yukawa convolution, k_m = sqrt(-2 eps_m)
    psi_m'   = c_m / (4 pi)
    eps_m   += -<psi_m V_eff (psi_m - psi_m')>_W / <psi_m'^2>_W
    psi_m    = psi_m', then Gram-Schmidt in orbital order (Orthogonalization.c:14)
    residual = |(psi, eps) - (psi, eps)_before|  with weights (W, 1)

The reference iterates one orbital at a time to its tolerance (with Anderson
mixing on (psi, eps), scfFixedPoint.py:381-597); here every orbital advances
in the same sweep, so the sweep's convolutions share one launch per field
pass and the whole sweep is one CUDA graph.  Every buffer is allocated once;
the sweep's launches never allocate, so ``capture`` records it for replay.
"""
import ctypes
import math

import numpy as np
import torch

try:
    from . import _native
    from . import device as dev
    from .BaryTreeInterface import Kernel, Singularity
except ImportError:
    import _native
    import device as dev
    from BaryTreeInterface import Kernel, Singularity


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


# Largest orbital count whose in-order Gram-Schmidt fits the library's
# allocation-free scratch (tagi_mgs_dev_noalloc handles targetWavefunction
# <= 128, i.e. orbitals 0..128).
NOALLOC_MAX_ORBITALS = 129

# The allocation-free Gram-Schmidt keeps its scratch in ONE fixed device array
# per GPU, shared by every caller in the process.  Every GreenIteration, SCF
# and LearnedExtrapolator in this package takes its turn on that array through
# `mgs_turn`: the stream waits for the last recorded use (an event) before its
# Gram-Schmidt launches (or a graph replay that holds them) and records its own
# use after them, so objects stepping on different streams never overlap on
# the array.  Nothing is waited for or recorded while a stream is being
# captured; the replay of the captured graph takes its turn instead.
_MGS_LAST = {}


class mgs_turn:
    """Context manager: order `stream`'s Gram-Schmidt work after every earlier
    use of the shared scratch in this process, and record this use."""

    def __init__(self, stream):
        self.stream = stream
        self.live = False

    def __enter__(self):
        self.live = not _capturing(self.stream)
        if self.live:
            ev = _MGS_LAST.get(self.stream.device)
            if ev is not None:
                self.stream.wait_event(ev)
        return self

    def __exit__(self, et, ev, tb):
        if self.live and et is None:
            done = torch.cuda.Event()
            done.record(self.stream)
            _MGS_LAST[self.stream.device] = done
        return False


def _capturing(stream):
    with torch.cuda.stream(stream):
        return torch.cuda.is_current_stream_capturing()


def orthonormalize(psi, weights, stream, first=0):
    """Weighted Gram-Schmidt of psi's rows first.. in orbital order
    (Orthogonalization.c:14-119 per row) on `stream`.  Up to 129 orbitals the
    allocation-free entry point runs, in the package-wide turn on its shared
    scratch; above that the allocating tagi_mgs_dev does (not capturable)."""
    L = _native.lib()
    m, n = int(psi.shape[0]), int(psi.shape[1])
    s = ctypes.c_void_p(stream.cuda_stream)
    if m <= NOALLOC_MAX_ORBITALS:
        with mgs_turn(stream):
            for j in range(first, m):
                _native.check(L.tagi_mgs_dev_noalloc(_p(psi), _p(psi[j]), _p(weights), j, n, m, s))
    else:
        if _capturing(stream):
            raise RuntimeError(f"{m} orbitals: Gram-Schmidt above {NOALLOC_MAX_ORBITALS} orbitals allocates and "
                               "cannot be captured")
        for j in range(first, m):
            _native.check(L.tagi_mgs_dev(_p(psi), _p(psi[j]), _p(weights), j, n, m, s))


class GreenIteration:
    """Device state and launch sequence of simultaneous Green iteration.

    plan: TreecodePlan over the mesh (targets = sources); weights: [n]
    quadrature weights; psi: [norb, n] orbitals (updated in place); eps:
    [norb] eigenvalues; veff: [n] effective potential (the caller may refill
    it between sweeps, also between graph replays)."""

    def __init__(self, plan, weights, psi, eps, veff, gauge_shift=-0.5, precision="mixed", stream=None):
        self.plan = plan
        self.n = int(weights.numel())
        self.norb = int(psi.shape[0])
        if psi.shape != (self.norb, self.n):
            raise ValueError("psi must be [norb, n]")
        # a created stream of its own by default: graph capture cannot use the default stream
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self.stream.wait_stream(torch.cuda.current_stream())
        self.precision = precision
        self.gauge = float(gauge_shift)
        d = psi.device
        f64 = dict(dtype=torch.float64, device=d)
        self.w = weights.contiguous()
        self.psi = psi
        self.veff = veff
        self.eps = torch.as_tensor(eps, **f64).contiguous().clone()
        self.eps_prev = self.eps.clone()
        self.k = torch.sqrt(-2.0 * self.eps.clamp(max=-1e-12))
        self.psi_prev = torch.empty_like(psi)
        self.f = torch.empty_like(psi)
        self.conv = torch.empty_like(psi)
        self.dE = torch.zeros(self.norb, **f64)
        self.flags = torch.zeros(self.norb, dtype=torch.int32, device=d)
        self.res = torch.zeros(self.norb, **f64)
        self.psi_res = torch.zeros(self.norb, **f64)
        L = _native.lib()
        nw = int(L.tagi_gi_workspace_doubles(self.n, self.norb))
        self.work = torch.empty(nw, **f64)
        self._graph = None
        self._eager_sweeps = 0
        self.anderson = None

    def set_eigenvalues(self, eps):
        self.eps.copy_(torch.as_tensor(eps, dtype=torch.float64))
        self.k.copy_(torch.sqrt(-2.0 * self.eps.clamp(max=-1e-12)))

    def _launches(self):
        L = _native.lib()
        s = ctypes.c_void_p(self.stream.cuda_stream)
        n, m = self.n, self.norb
        self.psi_prev.copy_(self.psi)
        _native.check(L.tagi_gi_source(_p(self.psi), _p(self.veff), n, m, _p(self.f), s))
        self.plan.convolve(self.f, self.f, Kernel.YUKAWA, self.k, Singularity.SUBTRACTION,
                           precision=self.precision, out=self.conv, stream=self.stream)
        _native.check(L.tagi_gi_update(_p(self.psi), _p(self.conv), _p(self.veff), _p(self.w), n, m,
                                       1.0 / (4.0 * math.pi), _p(self.eps), _p(self.eps_prev), _p(self.k),
                                       self.gauge, _p(self.dE), _p(self.flags), _p(self.work),
                                       self.work.numel(), s))
        orthonormalize(self.psi, self.w, self.stream)
        _native.check(L.tagi_gi_residual(_p(self.psi), _p(self.psi_prev), _p(self.w), n, m, _p(self.eps),
                                         _p(self.eps_prev), _p(self.res), _p(self.psi_res), _p(self.work),
                                         self.work.numel(), s))

    def sweep(self):
        """One sweep, launched eagerly on the stream."""
        with torch.cuda.stream(self.stream):
            self._launches()
        self._eager_sweeps += 1

    def capture(self):
        """Record one sweep as a CUDA graph.  A captured sweep must not allocate
        or look anything up: the plan's scratch and work list, and the
        Gram-Schmidt scratch address, come from an earlier eager sweep, so one
        runs here first if none has.  Above 129 orbitals the sweep's
        Gram-Schmidt allocates and capture is refused."""
        if self.norb > NOALLOC_MAX_ORBITALS:
            raise RuntimeError(f"{self.norb} orbitals: sweeps above {NOALLOC_MAX_ORBITALS} orbitals are not "
                               "capturable (their Gram-Schmidt allocates); use sweep()")
        if self._eager_sweeps == 0:
            self.sweep()
        if self._graph is not None:
            self._graph.close()
        with torch.cuda.stream(self.stream):
            with dev.Graph.capture(self.stream) as g:
                self._launches()
        self._graph = g
        return g

    def replay(self):
        if self._graph is None:
            raise RuntimeError("capture() first")
        with mgs_turn(self.stream):   # the graph holds Gram-Schmidt launches
            self._graph.replay(self.stream)

    def step(self):
        """One sweep: graph replay when captured, else eager."""
        if self._graph is not None:
            self.replay()
        else:
            self.sweep()

    # -- Anderson mixing of (psi, eps) per orbital (scfFixedPoint.py:483-597) ----------
    def enable_anderson(self, history=5, mixing=0.5, activate=3e-2):
        """After every sweep once the largest residual is below `activate`, mix
        each orbital's (psi, eps) over its last `history` sweeps (weights (W, 1)),
        then Gram-Schmidt: the mixed orbitals are the next sweep's input."""
        H = int(history)
        if not 2 <= H <= 8:
            raise ValueError("history must be in [2, 8]")
        f64 = dict(dtype=torch.float64, device=self.psi.device)
        L = _native.lib()
        self.anderson = dict(H=H, beta=float(mixing), activate=float(activate), count=0,
                             X=torch.zeros(H, self.norb, self.n, **f64),
                             F=torch.zeros(H, self.norb, self.n, **f64),
                             ex=np.zeros((H, self.norb)), ef=np.zeros((H, self.norb)),
                             gram=torch.zeros(self.norb * H * (H + 1) // 2, **f64),
                             work=torch.empty(int(L.tagi_gi_anderson_workspace_doubles(self.n, H, self.norb)),
                                              **f64),
                             mixed=0)

    def reset_anderson(self):
        if self.anderson is not None:
            self.anderson["count"] = 0

    def anderson_checkpoint(self):
        """The part of the mixing history the next anderson_step may change
        (its count and the ring row it writes), copied; None without mixing."""
        a = self.anderson
        if a is None:
            return None
        row = a["count"] % a["H"]
        with torch.cuda.stream(self.stream):
            return dict(count=a["count"], mixed=a["mixed"], row=row, X=a["X"][row].clone(), F=a["F"][row].clone(),
                        ex=a["ex"][row].copy(), ef=a["ef"][row].copy())

    def anderson_restore(self, ck):
        """Undo the mixing-history changes made since anderson_checkpoint: the
        history is again exactly the plain method's."""
        a = self.anderson
        if a is None or ck is None:
            return
        r = ck["row"]
        with torch.cuda.stream(self.stream):
            a["X"][r].copy_(ck["X"])
            a["F"][r].copy_(ck["F"])
        a["ex"][r], a["ef"][r] = ck["ex"], ck["ef"]
        a["count"], a["mixed"] = ck["count"], ck["mixed"]

    def anderson_step(self, residual):
        """Mix after a sweep (the stream must be idle); returns True if it mixed."""
        a = self.anderson
        if a is None or (a["count"] == 0 and residual > a["activate"]):
            return False
        H, m, n = a["H"], self.norb, self.n
        row = a["count"] % H
        with torch.cuda.stream(self.stream):
            a["X"][row].copy_(self.psi_prev)
            torch.sub(self.psi, self.psi_prev, out=a["F"][row])
            e_in, e_out = self.eps_prev.cpu().numpy(), self.eps.cpu().numpy()
            a["ex"][row], a["ef"][row] = e_in, e_out - e_in
            a["count"] += 1
            nh = min(a["count"], H)
            if nh < 2:
                return False
            L = _native.lib()
            s = ctypes.c_void_p(self.stream.cuda_stream)
            _native.check(L.tagi_gi_anderson_gram(_p(a["F"]), nh, m, n, _p(self.w), _p(a["gram"]), _p(a["work"]),
                                                  a["work"].numel(), s))
            np_ = nh * (nh + 1) // 2
            G = a["gram"][: m * np_].cpu().numpy().reshape(m, np_)

            def idx(i, j):
                i, j = min(i, j), max(i, j)
                return i * nh - i * (i - 1) // 2 + (j - i)

            older = [(row - 1 - k) % H for k in range(nh - 1)]
            c = np.zeros((m, nh - 1))
            eps_new = np.empty(m)
            for o in range(m):
                g = lambda i, j: G[o, idx(i, j)] + a["ef"][i, o] * a["ef"][j, o]
                A = np.array([[g(row, row) - g(row, ki) - g(row, kj) + g(ki, kj) for kj in older] for ki in older])
                rhs = np.array([g(row, row) - g(row, ki) for ki in older])
                try:
                    c[o] = np.linalg.solve(A, rhs)
                except np.linalg.LinAlgError:
                    c[o] = np.linalg.lstsq(A, rhs, rcond=None)[0]
                xm = a["ex"][row, o] + sum(c[o, k] * (a["ex"][ki, o] - a["ex"][row, o]) for k, ki in enumerate(older))
                fm = a["ef"][row, o] + sum(c[o, k] * (a["ef"][ki, o] - a["ef"][row, o]) for k, ki in enumerate(older))
                e = xm + a["beta"] * fm
                eps_new[o] = e if e < 0.0 else self.gauge - 1.5
            rows_t = torch.as_tensor(np.asarray(older, dtype=np.int32), device=self.psi.device)
            c_t = torch.as_tensor(c, dtype=torch.float64, device=self.psi.device).contiguous()
            _native.check(L.tagi_gi_anderson_mix(_p(a["X"]), _p(a["F"]), nh, row, _p(rows_t), _p(c_t), a["beta"], m,
                                                 n, _p(self.psi), s))
            orthonormalize(self.psi, self.w, self.stream)  # the mixed orbitals are no longer orthonormal
            self.set_eigenvalues(eps_new)
            self.stream.synchronize()
        a["mixed"] += 1
        return True

    def close(self):
        if self._graph is not None:
            self._graph.close()
            self._graph = None
