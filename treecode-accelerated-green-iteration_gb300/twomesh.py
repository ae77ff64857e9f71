"""Two-mesh eigenvalue correction on the device.

Restates the correction step TAGI runs after its SCF converges
(3D-GreenIteration/src/Green-Iteration-Routines/twoMeshCorrection.py:83-470)
in its all-electron form: local potentials only (the nonlocal pseudopotential
terms of :352-370 are zero without pseudopotentials) and Slater exchange
without correlation, as the SCF of this package uses.

    RHOf      = interp(RHO)                                          :172-176
    V_H       = Coulomb-SS convolution, targets the coarse mesh with RHO,
                sources the fine mesh with (RHOf, Wf), theta - 0.15,
                degree + 2                                           :183-254
    E_H       = 1/2 <W, RHO V_H>                                     :271
    V_eff     = V_H + V_x(RHO) + V_ext + gaugeShift (coarse)         :289-298
    per orbital m (all orbitals here in one launch per field pass):
      psi_f   = interp(psi_m)                                        :311-313
      Veff_f  = interp(V_eff - V_ext) + V_ext(fine points)           :314-326
      f_c     = -2 psi_m V_eff,  f_f = -2 psi_f Veff_f               :375-376
      psiNew  = Yukawa-SS convolution (coarse targets f_c, fine sources
                (f_f, Wf)), k = sqrt(-2 eps_m), theta - 0.15, degree + 2,
                divided by 4 pi                                      :379-422
      dE      = -<psi_m V_eff (psi_m - psiNew)>_W / <psiNew^2>_W     :426-431
      eps'_m  = eps_m + dE                                           :441
    orbitals sorted by eps', Fermi occupations, E_band               :447-462

The interpolations, convolutions, exchange, sources, Harrison update and
weighted sums run in this package's kernels (tagi_interp_dev, the treecode
plan, tagi_lda_exchange, tagi_veff, tagi_gi_source, tagi_gi_update,
tagi_wdot_rows); V_ext and two vector sums are torch elementwise ops; the
host keeps the scalars.
"""
import ctypes
import math

import numpy as np
import torch

try:
    from . import _native
    from . import device as dev
    from .BaryTreeInterface import Kernel, Singularity
    from .scf import fermi_occupations
except ImportError:
    import _native
    import device as dev
    from BaryTreeInterface import Kernel, Singularity
    from scf import fermi_occupations


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _t(a):
    if torch.is_tensor(a):
        return a.to(device="cuda", dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def external_potential(x, y, z, nuclei, charges, soft=0.0):
    """V_ext = -sum_a Z_a / |r - R_a| (all-electron)."""
    v = torch.zeros_like(x)
    for R, Z in zip(np.asarray(nuclei, np.float64).reshape(-1, 3), np.asarray(charges, np.float64).reshape(-1)):
        v -= Z / torch.sqrt((x - R[0]) ** 2 + (y - R[1]) ** 2 + (z - R[2]) ** 2 + soft)
    return v


class TwoMeshCorrection:
    """Coarse mesh (X, Y, Z, W), fine mesh (Xf, Yf, Zf, Wf) of the same cells,
    PtsPerCellCoarse / PtsPerCellFine (int32), cell order; nuclei and charges
    for the external potential.  theta / degree are the SCF's treecode
    parameters: the correction's convolutions use theta - 0.15, degree + 2
    (twoMeshCorrection.py:252-254, :418-420)."""

    def __init__(self, X, Y, Z, W, Xf, Yf, Zf, Wf, ppc_coarse, ppc_fine, order, nuclei, charges,
                 theta=0.7, degree=7, source_leaf=2000, target_leaf=2000, precision="mixed",
                 gauge_shift=-0.5, gaussian_alpha=1.0, soft=0.0, stream=None):
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        self.s = ctypes.c_void_p(self.stream.cuda_stream)
        self.stream.wait_stream(torch.cuda.current_stream())  # mesh arrays made on the caller's stream
        with torch.cuda.stream(self.stream):
            self.X, self.Y, self.Z, self.W = (_t(a) for a in (X, Y, Z, W))
            self.Xf, self.Yf, self.Zf, self.Wf = (_t(a) for a in (Xf, Yf, Zf, Wf))
            self.ppc_c = torch.as_tensor(ppc_coarse, dtype=torch.int32, device="cuda").contiguous()
            self.ppc_f = torch.as_tensor(ppc_fine, dtype=torch.int32, device="cuda").contiguous()
            self.n, self.nf = int(self.X.numel()), int(self.Xf.numel())
            self.ncells = int(self.ppc_c.numel())
            self.order = int(order)
            self.precision = precision
            self.gauge = float(gauge_shift)
            self.alpha = float(gaussian_alpha)
            self.theta, self.degree = theta - 0.15, degree + 2
            self.plan = dev.TreecodePlan(self.X, self.Y, self.Z, self.Xf, self.Yf, self.Zf, self.Wf,
                                         theta=self.theta, degree=self.degree, source_leaf=source_leaf,
                                         target_leaf=target_leaf, stream=self.stream)
            self.vext = external_potential(self.X, self.Y, self.Z, nuclei, charges, soft)
            self.vext_f = external_potential(self.Xf, self.Yf, self.Zf, nuclei, charges, soft)

    def interpolate(self, F, out=None):
        """Coarse values [n] -> fine mesh [nf] (callInterpolator)."""
        if out is None:
            out = torch.zeros(self.nf, dtype=torch.float64, device="cuda")
        else:
            out.zero_()
        return dev.interp(self.X, self.Y, self.Z, F, self.ppc_c, self.Xf, self.Yf, self.Zf, self.ppc_f,
                          self.ncells, self.order, fineF=out, stream=self.stream)

    def hartree(self, rho):
        """V_H on the coarse mesh from RHO (coarse) and its fine interpolant."""
        rho = _t(rho)
        self.stream.wait_stream(torch.cuda.current_stream())  # inputs made on the caller's stream
        with torch.cuda.stream(self.stream):
            rho_f = self.interpolate(rho)
            vh = self.plan.convolve(rho, rho_f, Kernel.COULOMB, [self.alpha], Singularity.SUBTRACTION,
                                    precision=self.precision, stream=self.stream)
        torch.cuda.current_stream().wait_stream(self.stream)  # results ready for the caller's stream
        return vh, rho_f

    def correct(self, psi, eps, rho, n_electrons=None, sigma=None):
        """Corrected eigenvalues of the orbitals psi [norb, n] with eigenvalues
        eps [norb] and density rho [n].  Returns a dict: deltaE, eigenvalues
        (corrected, input order), order (ascending permutation), Ehartree,
        and with n_electrons: occupations, fermi_energy, Eband (sorted
        order, twoMeshCorrection.py:447-462)."""
        L = _native.lib()
        psi = _t(psi).reshape(-1, self.n)
        norb = psi.shape[0]
        eps = np.asarray(eps, dtype=np.float64).reshape(-1)
        if eps.size != norb:
            raise ValueError("one eigenvalue per orbital")
        if np.any(eps >= 0):
            raise ValueError("eigenvalues must be negative (k = sqrt(-2 eps))")
        rho = _t(rho)
        f64 = dict(dtype=torch.float64, device="cuda")
        self.stream.wait_stream(torch.cuda.current_stream())  # inputs made on the caller's stream
        with torch.cuda.stream(self.stream):
            vh, _ = self.hartree(rho)
            vx = torch.empty(self.n, **f64)
            ex = torch.empty(self.n, **f64)
            veff = torch.empty(self.n, **f64)
            _native.check(L.tagi_lda_exchange(_p(rho), self.n, _p(vx), _p(ex), self.s))
            _native.check(L.tagi_veff(_p(vh), _p(vx), _p(self.vext), self.gauge, self.n, _p(veff), self.s))
            veff_f = self.interpolate(veff - self.vext) + self.vext_f
            psi_f = torch.empty((norb, self.nf), **f64)
            for m in range(norb):
                self.interpolate(psi[m].contiguous(), out=psi_f[m])
            f_c = torch.empty_like(psi)
            f_f = torch.empty_like(psi_f)
            _native.check(L.tagi_gi_source(_p(psi), _p(veff), self.n, norb, _p(f_c), self.s))
            _native.check(L.tagi_gi_source(_p(psi_f), _p(veff_f), self.nf, norb, _p(f_f), self.s))
            kd = torch.as_tensor(np.sqrt(-2.0 * eps), **f64)
            conv = self.plan.convolve(f_c, f_f, Kernel.YUKAWA, kd, Singularity.SUBTRACTION,
                                      precision=self.precision, stream=self.stream)
            # the Harrison update on copies: only its dE is kept (the reference
            # keeps the orbitals, :441)
            psi_tmp = psi.clone()
            e_tmp = torch.as_tensor(eps, **f64)
            e_prev = torch.empty_like(e_tmp)
            k_tmp = torch.empty_like(e_tmp)
            dE = torch.zeros(norb, **f64)
            flags = torch.zeros(norb, dtype=torch.int32, device="cuda")
            work = torch.empty(int(L.tagi_gi_workspace_doubles(self.n, norb)), **f64)
            _native.check(L.tagi_gi_update(_p(psi_tmp), _p(conv), _p(veff), _p(self.W), self.n, norb,
                                           1.0 / (4.0 * math.pi), _p(e_tmp), _p(e_prev), _p(k_tmp), self.gauge,
                                           _p(dE), _p(flags), _p(work), work.numel(), self.s))
            dot = torch.zeros(1, **f64)
            _native.check(L.tagi_wdot_rows(_p(rho), 0, _p(vh), 0, _p(self.W), self.n, 1, _p(dot), _p(work),
                                           work.numel(), self.s))
            eh = 0.5 * float(dot.item())
            d = dE.cpu().numpy()
        corrected = eps + d
        order = np.argsort(corrected, kind="stable")
        out = dict(deltaE=d, eigenvalues=corrected, order=order, Ehartree=eh, veff=veff, vhartree=vh,
                   psi_new=conv / (4.0 * math.pi))
        if n_electrons is not None:
            kw = {} if sigma is None else dict(sigma=sigma)
            occ, ef = fermi_occupations(corrected[order], n_electrons, **kw)
            out.update(occupations=occ, fermi_energy=ef,
                       Eband=float(np.sum((corrected[order] - self.gauge) * occ)))
        return out

    def close(self):
        if getattr(self, "plan", None) is not None:
            self.plan.close()
            self.plan = None
