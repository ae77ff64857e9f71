"""All-electron Kohn-Sham SCF by Green iteration, on the device.

Per SCF iteration (scfFixedPoint.py:92-672, with the Slater exchange of an
LDA and no correlation, as the ring-molecule workload asks):

    V_H   = sum_j w_j rho_j / |x - y_j|  (Coulomb, Gaussian subtraction, alpha 1;
                                          no 4 pi, scfFixedPoint.py:297-303)
    V_x   = -(3/pi)^(1/3) rho^(1/3)       Slater exchange
    V_eff = V_H + V_x + V_ext + gaugeShift
    Green-iteration sweeps (gi.GreenIteration) until the orbital residual
    falls below this iteration's tolerance
    sort orbitals by eigenvalue; Fermi-Dirac occupations at 300 K (:607-617)
    rho_out = sum_m occ_m psi_m^2 scaled to N electrons (:624-636)
    Anderson mixing of rho_in / rho_out histories (densityMixingSchemes.py)
    energies: E_band, E_H = 1/2 <W, rho V_H>, E_x, total (:646-660)

Convergence: the largest change of an occupied eigenvalue between SCF
iterations below ``tol`` (Ha).  Everything per point runs in this package's
kernels; the host keeps scalars: occupations (bisection on the Fermi level),
the Anderson linear system (size <= history), the loop control.

An optional ``extrapolator`` (learned.LearnedExtrapolator) proposes an
extrapolated orbital set after a sweep; the sweep that follows checks it: a
proposal whose Green-iteration residual is not below the plain iterate's
previous residual is rolled back, so the plain method stays the fallback.
"""
import ctypes
import math
import time

import numpy as np
import torch

try:
    from . import _native
    from . import device as dev
    from .BaryTreeInterface import Kernel, Singularity
    from .gi import GreenIteration, orthonormalize
except ImportError:
    import _native
    import device as dev
    from BaryTreeInterface import Kernel, Singularity
    from gi import GreenIteration, orthonormalize

KB = 1.0 / 315774.6  # Ha per K (scfFixedPoint.py:48-50)


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def fermi_occupations(eps, n_electrons, sigma=300.0 * KB):
    """Occupations 2 / (1 + exp((eps - eF)/sigma)) with sum = n_electrons; eF by
    bisection (the reference uses brentq on the same function, :52-59)."""
    eps = np.asarray(eps, dtype=np.float64)

    def excess(ef):
        x = np.clip((eps - ef) / sigma, -700, 700)
        return 2.0 * np.sum(1.0 / (1.0 + np.exp(x))) - n_electrons

    lo, hi = float(eps.min()) - 1.0, 1.0
    if excess(hi) < 0:
        raise ValueError("not enough orbitals for the electron count")
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if excess(mid) > 0:
            hi = mid
        else:
            lo = mid
        if hi - lo < 1e-15:
            break
    ef = 0.5 * (lo + hi)
    x = np.clip((eps - ef) / sigma, -700, 700)
    return 2.0 / (1.0 + np.exp(x)), ef


def nuclear_repulsion(nuclei, charges):
    e = 0.0
    for a in range(len(charges)):
        for b in range(a):
            e += charges[a] * charges[b] / float(np.linalg.norm(np.asarray(nuclei[a]) - np.asarray(nuclei[b])))
    return e


class AndersonMixer:
    """Anderson mixing of densities with a ring history of `history` rows on
    the device; the weighted dots run in tagi_wdot_rows, the small linear
    system on the host (densityMixingSchemes.py:30-97)."""

    def __init__(self, n, weights, mixing=0.5, history=10, device="cuda", stream=None):
        self.n, self.beta, self.H = n, float(mixing), int(history)
        self.s = ctypes.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        self.w = weights
        f64 = dict(dtype=torch.float64, device=device)
        self.rin = torch.zeros(self.H, n, **f64)
        self.rout = torch.zeros(self.H, n, **f64)
        self.count = 0
        L = _native.lib()
        self.work = torch.empty(int(L.tagi_gi_workspace_doubles(n, self.H)) + 1, **f64)
        self.dots = torch.zeros(self.H, **f64)

    def _dot_rows(self, A, b):
        L = _native.lib()
        rows = A.shape[0]
        _native.check(L.tagi_wdot_rows(_p(A), self.n, _p(b), 0, _p(self.w), self.n, rows, _p(self.dots),
                                       _p(self.work), self.work.numel(), self.s))
        return self.dots[:rows].cpu().numpy().copy()

    def mix(self, rho_in, rho_out, out):
        row = self.count % self.H
        self.rin[row].copy_(rho_in)
        self.rout[row].copy_(rho_out)
        self.count += 1
        nh = min(self.count, self.H)
        older = [(row - 1 - k) % self.H for k in range(nh - 1)]
        c = np.zeros(max(nh - 1, 1))
        if nh > 1:
            F = self.rout[row] - self.rin[row]
            D = torch.stack([F - (self.rout[r] - self.rin[r]) for r in older]).contiguous()
            A = np.zeros((nh - 1, nh - 1))
            for i in range(nh - 1):
                A[i] = self._dot_rows(D, D[i].contiguous())
            rhs = self._dot_rows(D, F.contiguous())
            try:
                c = np.linalg.solve(A, rhs)
            except np.linalg.LinAlgError:
                c = np.linalg.lstsq(A, rhs, rcond=None)[0]
        rows_t = torch.as_tensor(np.asarray(older if older else [0], dtype=np.int32), device=out.device)
        c_t = torch.as_tensor(c, dtype=torch.float64, device=out.device)
        _native.check(_native.lib().tagi_anderson_combine(
            _p(self.rin), _p(self.rout), nh, row, _p(rows_t), _p(c_t), self.beta, self.n, _p(out), self.s))
        return out


class SCF:
    """Green-iteration SCF for one mesh (targets = sources = mesh points)."""

    def __init__(self, x, y, z, w, nuclei, charges, psi0, eps0, n_electrons, gauge_shift=-0.5, mixing=0.5,
                 history=10, precision="mixed", theta=0.7, degree=7, source_leaf=2000, target_leaf=2000,
                 soft=0.0, graph=True, extrapolator=None, orbital_mixing=5):
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
        self.x, self.y, self.z, self.w = t(x), t(y), t(z), t(w)
        self.n = int(self.w.numel())
        self.nuclei = np.asarray(nuclei, dtype=np.float64).reshape(-1, 3)
        self.charges = np.asarray(charges, dtype=np.float64).reshape(-1)
        self.ne = float(n_electrons)
        self.gauge = float(gauge_shift)
        self.precision = precision
        self.stream = torch.cuda.Stream()
        self.s = ctypes.c_void_p(self.stream.cuda_stream)
        torch.cuda.synchronize()
        with torch.cuda.stream(self.stream):
            self._setup(psi0, eps0, soft, theta, degree, source_leaf, target_leaf, mixing, history)
        self.stream.synchronize()
        self.use_graph = graph
        self.extrapolator = extrapolator
        if orbital_mixing:
            self.gi.enable_anderson(history=orbital_mixing)
        self.enuc = nuclear_repulsion(self.nuclei, self.charges)
        self.history = []

    def _setup(self, psi0, eps0, soft, theta, degree, source_leaf, target_leaf, mixing, history):
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
        self.plan = dev.TreecodePlan.for_mesh(self.x, self.y, self.z, self.w, theta=theta, degree=degree,
                                              source_leaf=source_leaf, target_leaf=target_leaf, stream=self.stream)
        vext = torch.zeros(self.n, dtype=torch.float64, device="cuda")
        for R, Z in zip(self.nuclei, self.charges):
            r2 = (self.x - R[0]) ** 2 + (self.y - R[1]) ** 2 + (self.z - R[2]) ** 2
            vext -= Z / torch.sqrt(r2 + soft)
        self.vext = vext
        self.psi = t(psi0).reshape(-1, self.n).clone()
        self.norb = self.psi.shape[0]
        self.veff = torch.zeros(self.n, dtype=torch.float64, device="cuda")
        self.vh = torch.zeros_like(self.veff)
        self.vx = torch.zeros_like(self.veff)
        self.ex = torch.zeros_like(self.veff)
        self.rho = torch.zeros_like(self.veff)
        self.rho_out = torch.zeros_like(self.veff)
        L = _native.lib()
        self.work = torch.empty(int(L.tagi_gi_workspace_doubles(self.n, 4)) + 1, dtype=torch.float64,
                                device="cuda")
        self.dot = torch.zeros(4, dtype=torch.float64, device="cuda")
        # orthonormal start
        orthonormalize(self.psi, self.w, self.stream)
        self.gi = GreenIteration(self.plan, self.w, self.psi, eps0, self.veff, gauge_shift=self.gauge,
                                 precision=self.precision, stream=self.stream)
        self.mixer = AndersonMixer(self.n, self.w, mixing, history, stream=self.stream)
        self.occ = np.full(self.norb, 2.0)
        occ_t = torch.as_tensor(self.occ, dtype=torch.float64, device="cuda")
        _native.check(L.tagi_scf_density(_p(self.psi), _p(occ_t), self.norb, self.n, _p(self.w), self.ne,
                                         _p(self.rho), _p(self.work), self.work.numel(), self.s))

    def _wsum(self, a, b=None):
        L = _native.lib()
        _native.check(L.tagi_wdot_rows(_p(a), 0, _p(b) if b is not None else None, 0, _p(self.w), self.n, 1,
                                       _p(self.dot), _p(self.work), self.work.numel(), self.s))
        return float(self.dot[0].item())

    def potentials(self):
        """V_H, V_x, V_eff from the current input density; energies E_H, E_x, <rho V_x>."""
        L = _native.lib()
        self.plan.convolve(self.rho, self.rho, Kernel.COULOMB, [1.0], Singularity.SUBTRACTION,
                           precision=self.precision, out=self.vh, stream=self.stream)
        _native.check(L.tagi_lda_exchange(_p(self.rho), self.n, _p(self.vx), _p(self.ex), self.s))
        _native.check(L.tagi_veff(_p(self.vh), _p(self.vx), _p(self.vext), self.gauge, self.n, _p(self.veff),
                                  self.s))
        return dict(Ehartree=0.5 * self._wsum(self.rho, self.vh), Ex=self._wsum(self.rho, self.ex),
                    Vx=self._wsum(self.rho, self.vx))

    def _gi_sweep(self):
        self.gi.step()
        if self.use_graph and self.gi._graph is None:
            self.gi.capture()
        if self.gi.anderson is not None:
            self.stream.synchronize()
            self.gi.anderson_step(float(self.gi.res.max().item()))

    def green_iterations(self, tol, max_sweeps, min_sweeps=1):
        """Sweeps until the largest orbital residual (with eigenvalue) is below tol."""
        sweeps, res = 0, float("inf")
        self.gi.reset_anderson()  # a new potential: earlier sweeps do not mix with this one's
        if self.extrapolator is not None:
            self.extrapolator.reset()  # a new potential: earlier iterates no longer predict this one
        while sweeps < max_sweeps:
            if self.extrapolator is not None:
                res = self.extrapolator.sweep(self)
            else:
                self._gi_sweep()
                self.stream.synchronize()
                res = float(self.gi.res.max().item())
            sweeps += 1
            if sweeps >= min_sweeps and res < tol:
                break
        return sweeps, res

    def run(self, tol=1e-5, max_scf=60, gi_tol0=1e-2, gi_tol_min=1e-6, gi_decay=0.3, max_sweeps=12,
            time_limit=None, verbose=False):
        """Iterate to an eigenvalue change below tol.  Returns a summary dict;
        per-iteration records in self.history."""
        with torch.cuda.stream(self.stream):
            return self._run(tol, max_scf, gi_tol0, gi_tol_min, gi_decay, max_sweeps, time_limit, verbose)

    def _run(self, tol, max_scf, gi_tol0, gi_tol_min, gi_decay, max_sweeps, time_limit, verbose):
        t0 = time.perf_counter()
        prev_eps = None
        total_sweeps = 0
        converged = False
        for it in range(max_scf):
            en = self.potentials()
            gi_tol = max(gi_tol_min, gi_tol0 * gi_decay ** it)
            sweeps, gres = self.green_iterations(gi_tol, max_sweeps)
            total_sweeps += sweeps
            # sort by eigenvalue (scfFixedPoint.py:76-88)
            eps = self.gi.eps.cpu().numpy()
            order = np.argsort(eps, kind="stable")
            if np.any(order != np.arange(self.norb)):
                idx = torch.as_tensor(order, device="cuda")
                self.psi.copy_(self.psi[idx])
                self.gi.set_eigenvalues(eps[order])
                self.gi.eps_prev.copy_(self.gi.eps)
                eps = eps[order]
                if self.extrapolator is not None:
                    self.extrapolator.reset()
            occ, ef = fermi_occupations(eps - self.gauge, self.ne)
            self.occ = occ
            occ_t = torch.as_tensor(occ, dtype=torch.float64, device="cuda")
            L = _native.lib()
            _native.check(L.tagi_scf_density(_p(self.psi), _p(occ_t), self.norb, self.n, _p(self.w), self.ne,
                                             _p(self.rho_out), _p(self.work), self.work.numel(), self.s))
            diff = self.rho_out - self.rho
            dres = math.sqrt(max(self._wsum(diff, diff), 0.0)) / max(len(self.charges), 1)
            self.mixer.mix(self.rho, self.rho_out, self.rho)
            eband = float(np.sum((eps - self.gauge) * occ))
            etot = eband - en["Ehartree"] + en["Ex"] - en["Vx"] + self.enuc
            occupied = occ > 1e-6
            de = float(np.max(np.abs(eps - prev_eps)[occupied])) if prev_eps is not None else float("inf")
            prev_eps = eps.copy()
            rec = dict(iteration=it + 1, seconds=time.perf_counter() - t0, sweeps=sweeps, gi_residual=gres,
                       eigenvalues=(eps - self.gauge).tolist(), eigenvalue_change=de, density_residual=dres,
                       Etotal=etot, Eband=eband, Ehartree=en["Ehartree"], Ex=en["Ex"], fermi=ef - 0.0)
            self.history.append(rec)
            if verbose:
                print(f"SCF {it + 1}: dE_eig {de:.3e} Etot {etot:.8f} sweeps {sweeps} gi_res {gres:.2e} "
                      f"rho_res {dres:.2e} t {rec['seconds']:.1f}s", flush=True)
            if de < tol:
                converged = True
                break
            if time_limit is not None and time.perf_counter() - t0 > time_limit:
                break
        self.stream.synchronize()
        return dict(converged=converged, iterations=len(self.history), sweeps=total_sweeps,
                    seconds=time.perf_counter() - t0,
                    eigenvalues=self.history[-1]["eigenvalues"] if self.history else None,
                    Etotal=self.history[-1]["Etotal"] if self.history else None)

    def close(self):
        self.gi.close()
        self.plan.close()
