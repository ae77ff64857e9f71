"""The learned extrapolator driving Green iteration against plain sweeps.

Problem: the 1s state of V = -4/r (hydrogenic, eps = -8 Ha; -8.5 with the
gauge shift of -0.5) on an adaptive 62k-point mesh, from a poor start
(e^{-2r}, eps = -5.3).  Plain sweeps converge geometrically; the extrapolator
trains on the run's own iterates and jumps ahead when the next sweep's
residual confirms the jump.  Counted: sweeps (rejected jumps included) until
the residual (psi and eps) falls below 1e-6.  Checked: both runs converge to
the same eigenvalue, the extrapolator trains, proposes and keeps jumps, and
its sweep count stays within a bound of the plain count.  It does not beat
plain sweeps here (plain 25 sweeps, learned 48 on GB300): with the mixed
precision subtraction term on the kernels' own FP32 k the plain iteration
converges without a residual floor (41 sweeps before), and the kept jumps
disturb the orbital-mixing history more than they save.
"""
import ctypes
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG, to_cuda

pytestmark = pytest.mark.gpu


class _Driver:
    """The part of scf.SCF the extrapolator drives: one sweep, captured after the first."""

    def __init__(self, gi):
        self.gi = gi

    def _gi_sweep(self):
        self.gi.step()
        if self.gi._graph is None:
            self.gi.capture()


def _solve(dev, native, gi_mod, mesh, extrapolator, tol=1e-6, max_sweeps=80):
    Z = 4.0
    r = np.sqrt(mesh.x ** 2 + mesh.y ** 2 + mesh.z ** 2)
    x, y, z, w, psi, V = to_cuda(mesh.x, mesh.y, mesh.z, mesh.w, np.exp(-0.5 * Z * r)[None, :], -Z / r - 0.5)
    psi = psi.contiguous()
    L = native.lib()
    native.check(L.tagi_mgs_dev_noalloc(ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(psi.data_ptr()),
                                        ctypes.c_void_p(w.data_ptr()), 0, mesh.n, 1, None))
    torch.cuda.synchronize()
    plan = dev.TreecodePlan.for_mesh(x, y, z, w, source_leaf=1000, target_leaf=1000)
    g = gi_mod.GreenIteration(plan, w, psi, [-0.3 * Z * Z - 0.5], V, gauge_shift=-0.5, precision="mixed")
    d = _Driver(g)
    sweeps, res = 0, 1.0
    while res >= tol and sweeps < max_sweeps:
        if extrapolator is not None:
            res = extrapolator.sweep(d)
            sweeps = extrapolator.stats["sweeps"]
        else:
            d._gi_sweep()
            g.stream.synchronize()
            res = float(g.res.max())
            sweeps += 1
    eps = float(g.eps[0])
    g.close()
    plan.close()
    return sweeps, res, eps


def test_learned_extrapolation_reaches_the_plain_result(dev, native, syn):
    gi_mod = importlib.import_module(PKG + ".gi")
    learned = importlib.import_module(PKG + ".learned")
    mesh = syn.adaptive_mesh([[0.0, 0.0, 0.0]], [4.0], 5, 6, 1.0)
    plain_sweeps, plain_res, plain_eps = _solve(dev, native, gi_mod, mesh, None)
    ex = learned.LearnedExtrapolator((5 + 1) ** 3, rollout=8)
    sweeps, res, eps = _solve(dev, native, gi_mod, mesh, ex)
    assert plain_res < 1e-6 and res < 1e-6
    # both arms converge to res < 1e-6 on the same mixed-precision operator: their
    # eigenvalues agree to a few parts in 1e6 of |eps|
    assert abs(eps - plain_eps) < 3e-6 * abs(plain_eps)
    assert ex.stats["proposals"] >= 1 and ex.stats["accepted"] >= 1 and ex.stats["trained"] >= 2
    # a regression bound, not a gain: rejected jumps counted
    assert sweeps <= 2.5 * plain_sweeps, (sweeps, plain_sweeps, ex.stats)
