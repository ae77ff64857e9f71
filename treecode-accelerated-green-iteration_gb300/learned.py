"""Learned extrapolation for Green iteration (the learned part of the SCF).

A 3-layer MLP (hidden width 256, BF16 weights, FP32 accumulation; kernels in
csrc/mlp.cu) reads per-cell patches of an orbital iterate psi_t, its latest
Green-iteration update d_t = psi_t - psi_{t-1} and the eigenvalue, and
predicts the next update d_{t+1} of the patch (in units of the patch's RMS
update, with a learned skip term alpha d_t).  It is trained online, on the
device, on the run's own consecutive plain iterates.  A proposal rolls the
prediction out for a few steps and jumps there; the sweep that follows is the
check: if its Green-iteration residual does not fall below the last plain
residual, the jump is undone and the plain iterate continues, so plain Green
iteration stays both fallback and check.

No counterpart in the reference; the closest is its Anderson mixing of
(psi, eps) histories (scfFixedPoint.py:491-597).
"""
import ctypes
import math

import numpy as np
import torch

try:
    from . import _native
    from .gi import orthonormalize
except ImportError:
    import _native
    from gi import orthonormalize


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class MLP:
    """Parameters (FP32 masters + BF16 copies), Adam state and the kernels'
    forward / backward passes for rows of ``ldx`` BF16 features."""

    def __init__(self, P, hidden=256, lr=1e-3, seed=0, stream=None):
        self.P, self.H = int(P), int(hidden)
        self.din = 2 * self.P + 1
        self.ldx = ((self.din + 31) // 32) * 32
        self.lr = float(lr)
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        g = torch.Generator().manual_seed(seed)
        f32 = dict(dtype=torch.float32)

        def init(o, i, scale=1.0):
            b = scale * math.sqrt(6.0 / i)  # He-uniform
            return ((torch.rand(o, i, generator=g, **f32) * 2 - 1) * b).cuda()

        W1 = init(self.H, self.ldx)
        W1[:, self.din:] = 0.0
        self.params = dict(W1=W1, b1=torch.zeros(self.H, device="cuda"),
                           W2=init(self.H, self.H), b2=torch.zeros(self.H, device="cuda"),
                           W3=init(self.P, self.H, 0.01), b3=torch.zeros(self.P, device="cuda"),
                           alpha=torch.full((1,), 0.5, device="cuda"))
        self.half = {k: self.params[k].to(torch.bfloat16).contiguous() for k in ("W1", "W2", "W3")}
        self.grads = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.m1 = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.m2 = {k: torch.zeros_like(v) for k, v in self.params.items()}
        self.t = 0
        self.rows = 0
        self._lossbuf = torch.zeros(2, device="cuda")

    def _ensure(self, rows):
        if rows <= self.rows:
            return
        d = "cuda"
        self.H1 = torch.empty(rows, self.H, dtype=torch.bfloat16, device=d)
        self.H2 = torch.empty(rows, self.H, dtype=torch.bfloat16, device=d)
        self.Y = torch.empty(rows, self.P, dtype=torch.float32, device=d)
        self.dY = torch.empty(rows, self.P, dtype=torch.float32, device=d)
        self.dY16 = torch.empty(rows, self.P, dtype=torch.bfloat16, device=d)
        self.dH2 = torch.empty(rows, self.H, dtype=torch.bfloat16, device=d)
        self.dH1 = torch.empty(rows, self.H, dtype=torch.bfloat16, device=d)
        self.part = torch.empty(2 * rows, dtype=torch.float32, device=d)
        self.splits = max(1, min(64, (rows + 2047) // 2048))
        self.kpart = torch.empty(self.splits * self.H * max(self.ldx, self.P), dtype=torch.float32, device=d)
        L = _native.lib()
        self.cwork = torch.empty(int(L.tagi_mlp_colsum_workspace(rows, max(self.H, self.P))), dtype=torch.float32,
                                 device=d)
        self.rows = rows

    def _s(self):
        return ctypes.c_void_p(self.stream.cuda_stream)

    def forward(self, X, rows):
        """X: [rows, ldx] BF16 -> self.Y[:rows] (f32)."""
        self._ensure(rows)
        L, s, P, H, ldx = _native.lib(), self._s(), self.P, self.H, self.ldx
        h, pr = self.half, self.params
        _native.check(L.tagi_mlp_gemm(_p(X), ldx, 1, _p(h["W1"]), 1, ldx, rows, H, ldx, 1, None, _p(self.H1), H,
                                      _p(pr["b1"]), None, s))
        _native.check(L.tagi_mlp_gemm(_p(self.H1), H, 1, _p(h["W2"]), 1, H, rows, H, H, 1, None, _p(self.H2), H,
                                      _p(pr["b2"]), None, s))
        _native.check(L.tagi_mlp_gemm(_p(self.H2), H, 1, _p(h["W3"]), 1, H, rows, P, H, 3, _p(self.Y), None, P,
                                      _p(pr["b3"]), None, s))
        return self.Y[:rows]

    def loss_and_grads(self, X, dn, T, rows):
        """Forward, MSE against T (targets in units of s_d), backward into self.grads; returns the loss."""
        self.forward(X, rows)
        L, s, P, H, ldx = _native.lib(), self._s(), self.P, self.H, self.ldx
        h, g = self.half, self.grads
        _native.check(L.tagi_mlp_mse_grad(_p(self.Y), _p(dn), _p(T), _p(self.params["alpha"]), rows, P, _p(self.dY),
                                          _p(self.dY16), _p(self.part), _p(self._lossbuf), s))
        g["alpha"].copy_(self._lossbuf[1:2])
        cw = self.cwork.numel()
        # layer 3
        _native.check(L.tagi_mlp_gemm_splitk(_p(self.dY16), 1, P, _p(self.H2), H, 1, P, H, rows, self.splits,
                                             _p(self.kpart), _p(g["W3"]), s))
        _native.check(L.tagi_mlp_colsum(_p(self.dY), 0, rows, P, _p(g["b3"]), _p(self.cwork), cw, s))
        _native.check(L.tagi_mlp_gemm(_p(self.dY16), P, 1, _p(h["W3"]), H, 1, rows, H, P, 2, None, _p(self.dH2), H,
                                      None, _p(self.H2), s))
        # layer 2
        _native.check(L.tagi_mlp_gemm_splitk(_p(self.dH2), 1, H, _p(self.H1), H, 1, H, H, rows, self.splits,
                                             _p(self.kpart), _p(g["W2"]), s))
        _native.check(L.tagi_mlp_colsum(_p(self.dH2), 1, rows, H, _p(g["b2"]), _p(self.cwork), cw, s))
        _native.check(L.tagi_mlp_gemm(_p(self.dH2), H, 1, _p(h["W2"]), H, 1, rows, H, H, 2, None, _p(self.dH1), H,
                                      None, _p(self.H1), s))
        # layer 1
        _native.check(L.tagi_mlp_gemm_splitk(_p(self.dH1), 1, H, _p(X), ldx, 1, H, ldx, rows, self.splits,
                                             _p(self.kpart), _p(g["W1"]), s))
        _native.check(L.tagi_mlp_colsum(_p(self.dH1), 1, rows, H, _p(g["b1"]), _p(self.cwork), cw, s))
        return self._lossbuf[0]

    def adam_step(self, beta1=0.9, beta2=0.999, eps=1e-8):
        self.t += 1
        L, s = _native.lib(), self._s()
        for k, w in self.params.items():
            _native.check(L.tagi_mlp_adam(_p(w), _p(self.grads[k]), _p(self.m1[k]), _p(self.m2[k]), w.numel(),
                                          self.lr, beta1, beta2, eps, self.t, _p(self.half.get(k)), s))


class LearnedExtrapolator:
    """Online-trained extrapolation of Green-iteration sweeps (see module doc).

    P: points per cell (the mesh stores cells contiguously); rollout: the
    largest number of predicted steps per proposal (the length adapts: it
    starts at `rollout`, halves after a rejected jump down to 1 and doubles
    after a kept one back up to `rollout`); train_steps: Adam steps per new
    training pair; warmup:
    training pairs seen before the first proposal; cooldown: sweeps without
    proposals after a rejected one (doubling on repeated rejections).

    Each new training pair is first a validation pair: the network's loss on
    it is compared with the loss of its skip term alone (alpha d), and the
    network's correction enters proposals only while it at least halves that
    loss (running average); otherwise proposals use the learned skip term.
    Eigenvalues are extrapolated by the geometric sum of their last two
    updates over the same rollout."""

    def __init__(self, P, hidden=256, rollout=6, train_steps=4, warmup=2, cooldown=2, lr=1e-3, floor=1e-3,
                 seed=0, correction=1.0, min_residual=0.0):
        self.P, self.rollout, self.train_steps = int(P), int(rollout), int(train_steps)
        self.steps = self.rollout   # current rollout length
        # weight of the network's correction to the learned skip term, and the residual below
        # which no more proposals are made (plain sweeps finish the convergence)
        self.correction, self.min_residual = float(correction), float(min_residual)
        self.warmup, self.cooldown_len, self.floor = int(warmup), int(cooldown), float(floor)
        self.hidden, self.lr, self.seed = hidden, lr, seed
        self.net = None
        self.disabled = False  # set for the rest of the run when too few jumps are kept
        self.gate = None  # running ratio of validation losses: full network / skip term alone
        self.stats = dict(proposals=0, accepted=0, rejected=0, trained=0, sweeps=0, extra_sweeps=0)
        self.log = []   # per proposal: rollout, residual before, residual after, kept
        self.reset()

    def reset(self):
        """Forget the iterate history (new potential or reordered orbitals); keep the weights,
        which go on training across potentials."""
        self.hist = []          # device copies of the last plain iterates (psi)
        self.eps_hist = []      # host copies of their eigenvalues
        self.anderson_ck = None
        self.pending = False
        self.cool = 0
        self.backoff = self.cooldown_len
        self.last_res = None

    def _setup(self, gi):
        if self.net is None:
            self.net = MLP(self.P, self.hidden, self.lr, self.seed, stream=gi.stream)
            n, m = gi.n, gi.norb
            if n % self.P:
                raise ValueError("mesh point count is not a multiple of the cell size P")
            self.ncell = n // self.P
            self.rows = m * self.ncell
            f64 = dict(dtype=torch.float64, device="cuda")
            self.X = torch.zeros(self.rows, self.net.ldx, dtype=torch.bfloat16, device="cuda")
            self.scale = torch.zeros(self.rows, dtype=torch.float32, device="cuda")
            self.dn = torch.zeros(self.rows, self.P, dtype=torch.float32, device="cuda")
            self.T = torch.zeros(self.rows, self.P, dtype=torch.float32, device="cuda")
            self.d = torch.zeros(m, n, **f64)
            self.dnext = torch.zeros(m, n, **f64)
            self.work_psi = torch.zeros(m, n, **f64)
            self.work_d = torch.zeros(m, n, **f64)
            self.backup_psi = torch.zeros(m, n, **f64)
            self.backup_eps = torch.zeros(m, **f64)
            self.dfloor = torch.zeros(m, **f64)

    def _features(self, gi, psi, d):
        L = _native.lib()
        s = ctypes.c_void_p(gi.stream.cuda_stream)
        # floor of the patch scale: a fraction of the orbital's RMS update
        self.dfloor.copy_(self.floor * torch.sqrt((d * d).mean(dim=1)))
        _native.check(L.tagi_mlp_patch_features(_p(psi), _p(d), _p(gi.eps), _p(self.dfloor), gi.norb, self.ncell,
                                                self.P, gi.n, self.net.ldx, _p(self.X), _p(self.scale), _p(self.dn),
                                                s))

    def _train(self, gi):
        psi_prev, psi_cur, psi_new = self.hist[-3], self.hist[-2], self.hist[-1]
        torch.sub(psi_cur, psi_prev, out=self.d)
        torch.sub(psi_new, psi_cur, out=self.dnext)
        self._features(gi, psi_cur, self.d)
        L = _native.lib()
        s = ctypes.c_void_p(gi.stream.cuda_stream)
        _native.check(L.tagi_mlp_patch_target(_p(self.dnext), _p(self.scale), gi.norb, self.ncell, self.P, gi.n,
                                              _p(self.T), s))
        for i in range(self.train_steps):
            loss = self.net.loss_and_grads(self.X, self.dn, self.T, self.rows)
            if i == 0:
                # the new pair is unseen: validate the network against its own skip term alone
                skip = torch.sum((self.net.params["alpha"] * self.dn - self.T) ** 2)
                ratio = float(loss) / max(float(skip), 1e-300)
                self.gate = ratio if self.gate is None else 0.7 * self.gate + 0.3 * ratio
            self.net.adam_step()
        self.stats["trained"] += 1

    def _propose(self, gi):
        """psi <- psi_t + sum of `rollout` predicted updates, Gram-Schmidt'ed; backup kept."""
        L = _native.lib()
        s = ctypes.c_void_p(gi.stream.cuda_stream)
        # Orbital mixing keeps its history across a jump: the sweep from the
        # proposal adds a genuine (input, output) pair to it.  If the jump is
        # rejected that pair is taken out again, so the plain method resumes
        # with exactly its own history.
        self.anderson_ck = gi.anderson_checkpoint() if hasattr(gi, "anderson_checkpoint") else None
        self.backup_psi.copy_(gi.psi)
        self.backup_eps.copy_(gi.eps)
        self.work_psi.copy_(gi.psi)
        # eigenvalues: the geometric (Aitken) sum of their own last two updates, same rollout
        e0, e1, e2 = self.eps_hist[-3], self.eps_hist[-2], self.eps_hist[-1]
        d1, d2 = e1 - e0, e2 - e1
        with np.errstate(divide="ignore", invalid="ignore"):
            rho = np.clip(np.where(np.abs(d1) > 0, d2 / d1, 0.0), 0.0, 0.9)
        J = self.steps
        self.eps_proposed = e2 + d2 * rho * (1.0 - rho ** J) / (1.0 - rho)
        torch.sub(self.hist[-1], self.hist[-2], out=self.work_d)
        for _ in range(J):
            self._features(gi, self.work_psi, self.work_d)
            Y = self.net.forward(self.X, self.rows)
            # the network's correction is used only while it beats its own skip term on unseen pairs
            w = self.correction if (self.gate is not None and self.gate < 0.5) else 0.0
            if w != 1.0:
                Y.mul_(w)
            _native.check(L.tagi_mlp_patch_apply(_p(self.work_psi), _p(Y), _p(self.dn), _p(self.scale),
                                                 _p(self.net.params["alpha"]), gi.norb, self.ncell, self.P, gi.n,
                                                 _p(self.work_psi), _p(self.work_d), s))
        gi.psi.copy_(self.work_psi)
        orthonormalize(gi.psi, gi.w, gi.stream)
        self.work_psi.copy_(gi.psi)  # the proposal as the next sweep starts from it
        gi.set_eigenvalues(self.eps_proposed)
        self.pending = True
        self.stats["proposals"] += 1

    def sweep(self, scf):
        """One Green-iteration sweep of scf (scf.SCF) with extrapolation; returns the residual."""
        gi = scf.gi
        self._setup(gi)
        with torch.cuda.stream(gi.stream):
            scf._gi_sweep()
            gi.stream.synchronize()
            res = float(gi.res.max().item())
            self.stats["sweeps"] += 1
            if self.pending:
                self.pending = False
                kept = self.last_res is not None and res < self.last_res
                self.log.append((self.steps, self.last_res, res, kept, self.gate))
                if kept:
                    self.steps = min(2 * self.steps, self.rollout)
                else:
                    self.steps = max(self.steps // 2, 1)
                if kept:
                    self.stats["accepted"] += 1
                    # the jump's sweep is a plain update from the proposal: restart the history there
                    self.hist = [self.work_psi.clone(), gi.psi.clone()]
                    self.eps_hist = [np.asarray(self.eps_proposed, dtype=np.float64), gi.eps.cpu().numpy()]
                    self.last_res = res
                    self.backoff = self.cooldown_len
                    return res
                # rejected: back to the plain iterate and its plain sweep
                self.stats["rejected"] += 1
                self.stats["extra_sweeps"] += 1
                gi.psi.copy_(self.backup_psi)
                gi.set_eigenvalues(self.backup_eps.cpu().numpy())
                if hasattr(gi, "anderson_restore"):
                    gi.anderson_restore(self.anderson_ck)
                self.cool = self.backoff
                self.backoff = min(2 * self.backoff + 1, 16)
                scf._gi_sweep()
                gi.stream.synchronize()
                res = float(gi.res.max().item())
                self.stats["sweeps"] += 1
            self.hist.append(gi.psi.clone())
            self.eps_hist.append(gi.eps.cpu().numpy())
            if len(self.hist) > 3:
                self.hist.pop(0)
                self.eps_hist.pop(0)
            self.last_res = res
            if len(self.hist) == 3:
                self._train(gi)
                # the plain method checks the learner as a whole too: a run in which fewer
                # than a third of the jumps survive stops proposing
                p = self.stats["proposals"]
                if p >= 6 and self.stats["accepted"] * 3 < p:
                    self.disabled = True
                if (not self.disabled and self.stats["trained"] >= self.warmup and self.cool == 0
                        and res > self.min_residual):
                    self._propose(gi)
            if self.cool > 0:
                self.cool -= 1
            gi.stream.synchronize()
        return res
