"""CPU restatement of one Green-iteration sweep and of the SCF helpers
(TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of gi.py and
scf.py; never by the product path).

Follows 3D-GreenIteration/src/Green-Iteration-Routines/greenIterationFixedPoint.py
with every orbital advanced in the same sweep, as the device sweep does:
  f = -2 psi V_eff (:155); k = sqrt(-2 eps) (:207); psi_new = conv / 4pi (:323);
  dE = -<psi V_eff (psi - psi_new)>_W / <psi_new^2>_W (:373-398);
  eps += dE, an eigenvalue >= 0 set to gaugeShift - 1.5 (:470-477 use a random
  offset); psi <- psi_new; Gram-Schmidt in orbital order (Orthogonalization.c:14,
  via the oracle's restatement); residual with weights (W, 1)
  (scfFixedPoint.py:62-67).
The convolution is the oracle's FP64 treecode (same tree and list rules as
the device), so an FP64 device sweep matches this one to rounding.

two_mesh_correction restates the eigenvalue correction of
Green-Iteration-Routines/twoMeshCorrection.py:172-441 (all-electron, local
potentials) with the oracle's interpolation and treecode.
"""
import math

import numpy as np

from . import oracle as O

YUKAWA, SUBTRACTION = 2, 2


def gi_sweep(plan, w, psi, eps, veff, gauge=-0.5):
    psi = np.array(psi, dtype=np.float64, copy=True)
    eps = np.array(eps, dtype=np.float64, copy=True)
    prev, eps_prev = psi.copy(), eps.copy()
    norb = psi.shape[0]
    k = np.sqrt(-2.0 * eps)
    for m in range(norb):
        f = -2.0 * prev[m] * veff
        c = plan.convolve(f, f, w, YUKAWA, [k[m]], SUBTRACTION)
        q = c / (4.0 * math.pi)
        num = np.sum(w * prev[m] * veff * (prev[m] - q))
        den = np.sum(w * q * q)
        e = eps[m] - num / den
        if not e < 0.0:
            e = gauge - 1.5
        eps[m] = e
        psi[m] = q
    for m in range(norb):
        U = psi[m].copy()
        O.mgs(psi, U, w, m)
    dpsi = np.sqrt(np.sum(w[None, :] * (psi - prev) ** 2, axis=1))
    res = np.sqrt(dpsi ** 2 + (eps - eps_prev) ** 2)
    return psi, eps, res, dpsi


def lda_exchange(rho):
    c = (3.0 / math.pi) ** (1.0 / 3.0)
    r = np.cbrt(np.maximum(rho, 0.0))
    return -c * r, -0.75 * c * r


def density(psi, occ, w, n_electrons):
    rho = np.sum(np.asarray(occ)[:, None] * psi ** 2, axis=0)
    return rho * (n_electrons / np.sum(w * rho))


def anderson(rin_hist, rout_hist, w, beta):
    """rin_hist/rout_hist: lists oldest .. newest (densityMixingSchemes.py:30-97)."""
    n = len(rin_hist)
    F = [o - i for i, o in zip(rin_hist, rout_hist)]
    if n > 1:
        A = np.zeros((n - 1, n - 1))
        rhs = np.zeros(n - 1)
        for m in range(n - 1):
            f = F[n - 1] - F[n - 2 - m]
            rhs[m] = np.sum(f * F[n - 1] * w)
            for k in range(n - 1):
                A[m, k] = np.sum(f * (F[n - 1] - F[n - 2 - k]) * w)
        c = np.linalg.solve(A, rhs)
    else:
        c = np.zeros(0)
    win, wout = rin_hist[-1].copy(), rout_hist[-1].copy()
    for k in range(n - 1):
        win += c[k] * (rin_hist[n - 2 - k] - rin_hist[-1])
        wout += c[k] * (rout_hist[n - 2 - k] - rout_hist[-1])
    return beta * wout + (1 - beta) * win


def two_mesh_correction(coarse, fine, ppc_c, ppc_f, order, nuclei, charges, psi, eps, rho, theta, degree,
                        source_leaf, target_leaf, gauge=-0.5, alpha=1.0):
    """Eigenvalue corrections of twoMeshCorrection.py:172-441 (all-electron,
    local potentials, Slater exchange): the oracle's interpolation and FP64
    treecode (coarse targets, fine sources, theta - 0.15, degree + 2).
    coarse = (X, Y, Z, W), fine = (Xf, Yf, Zf, Wf).  Returns (dE, V_H, E_H)."""
    X, Y, Z, W = (np.asarray(a, np.float64) for a in coarse)
    Xf, Yf, Zf, Wf = (np.asarray(a, np.float64) for a in fine)
    ncells = len(ppc_c)

    def interp(F):
        return O.interp(X, Y, Z, F, ppc_c, Xf, Yf, Zf, ppc_f, ncells, order)

    def vext(x, y, z):
        v = np.zeros_like(x)
        for R, Zc in zip(np.asarray(nuclei, np.float64).reshape(-1, 3), np.asarray(charges, np.float64)):
            v -= Zc / np.sqrt((x - R[0]) ** 2 + (y - R[1]) ** 2 + (z - R[2]) ** 2)
        return v

    plan = O.Plan(X, Y, Z, Xf, Yf, Zf, Wf, theta - 0.15, degree + 2, source_leaf, target_leaf)
    COULOMB = 1
    vh = plan.convolve(rho, interp(rho), Wf, COULOMB, [alpha], SUBTRACTION)
    eh = 0.5 * float(np.sum(W * rho * vh))
    vx, _ = lda_exchange(rho)
    ve, ve_f = vext(X, Y, Z), vext(Xf, Yf, Zf)
    veff = vh + vx + ve + gauge
    veff_f = interp(veff - ve) + ve_f
    dE = np.zeros(len(eps))
    for m in range(len(eps)):
        pf = interp(psi[m])
        c = plan.convolve(-2.0 * psi[m] * veff, -2.0 * pf * veff_f, Wf, YUKAWA, [math.sqrt(-2.0 * eps[m])],
                          SUBTRACTION) / (4.0 * math.pi)
        dE[m] = -np.sum(W * psi[m] * veff * (psi[m] - c)) / np.sum(W * c * c)
    return dE, vh, eh
