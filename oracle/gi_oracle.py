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
