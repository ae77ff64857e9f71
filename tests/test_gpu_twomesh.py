"""Two-mesh eigenvalue correction (twomesh.TwoMeshCorrection) on the GPU,
over a two-level mesh built by the device mesh generator.

Checked against the oracle's restatement (oracle/gi_oracle.py
two_mesh_correction: the oracle's interpolation and FP64 treecode with the
same tree and list rules, numpy for the rest).  Tolerances: FP64 device path
agrees to rounding (1e-10 relative on V_H and E_H, 1e-9 Ha on dE); the mixed
path within 1e-6 relative (V_H), and dE within the shift that a 1e-6
relative error of the convolution can cause (bound computed in the test).
Known answer: the Hartree potential of a normalized Gaussian is
erf(sqrt(a) r)/r; with the fine mesh as sources its error is below the
coarse-only convolution's.
"""
import importlib
import math

import numpy as np
import pytest
import torch
from scipy.special import erf

from oracle import gi_oracle as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NUC = np.array([[-0.7, 0.05, 0.0], [0.7, -0.05, 0.0]])
CHG = np.array([1.0, 1.0])
ORDER = 3


@pytest.fixture(scope="module")
def setup(pkg, native, oracle):
    M = importlib.import_module(pkg.__name__ + ".mesh")
    T = importlib.import_module(pkg.__name__ + ".twomesh")
    m = M.build_mesh(8.0, 4.0, NUC, ORDER, 1.0, 4.0, 1.0, -2.0)
    assert m.n == 11264 and m.Xf.numel() == 43520
    h = {k: getattr(m, k).cpu().numpy() for k in ("X", "Y", "Z", "W", "Xf", "Yf", "Zf", "Wf",
                                                  "PtsPerCellCoarse", "PtsPerCellFine")}
    X, Y, Z, W = h["X"], h["Y"], h["Z"], h["W"]
    r1 = np.sqrt((X - NUC[0, 0]) ** 2 + (Y - NUC[0, 1]) ** 2 + (Z - NUC[0, 2]) ** 2)
    r2 = np.sqrt((X - NUC[1, 0]) ** 2 + (Y - NUC[1, 1]) ** 2 + (Z - NUC[1, 2]) ** 2)
    psi = np.stack([np.exp(-r1) + np.exp(-r2), np.exp(-r1) - np.exp(-r2)])
    psi /= np.sqrt((psi ** 2 * W).sum(1))[:, None]
    rho = 2 * psi[0] ** 2
    eps = np.array([-0.6, -0.2])
    ref = G.two_mesh_correction((X, Y, Z, W), (h["Xf"], h["Yf"], h["Zf"], h["Wf"]), h["PtsPerCellCoarse"],
                                h["PtsPerCellFine"], ORDER, NUC, CHG, psi, eps, rho, 0.7, 7, 500, 500)
    return T, m, h, psi, eps, rho, ref


def make(T, m, precision):
    return T.TwoMeshCorrection(m.X, m.Y, m.Z, m.W, m.Xf, m.Yf, m.Zf, m.Wf, m.PtsPerCellCoarse, m.PtsPerCellFine,
                               ORDER, NUC, CHG, theta=0.7, degree=7, source_leaf=500, target_leaf=500,
                               precision=precision)


def test_fp64_matches_oracle(setup):
    T, m, h, psi, eps, rho, (dE_ref, vh_ref, eh_ref) = setup
    c = make(T, m, "fp64")
    out = c.correct(psi, eps, rho, n_electrons=2.0)
    vh = out["vhartree"].cpu().numpy()
    assert np.linalg.norm(vh - vh_ref) / np.linalg.norm(vh_ref) <= 1e-10
    assert abs(out["Ehartree"] - eh_ref) <= 1e-10 * abs(eh_ref)
    assert np.max(np.abs(out["deltaE"] - dE_ref)) <= 1e-9
    assert np.array_equal(out["eigenvalues"], eps + out["deltaE"])
    assert np.array_equal(out["order"], np.argsort(out["eigenvalues"]))
    assert abs(out["occupations"].sum() - 2.0) < 1e-9
    c.close()


def test_mixed_matches_oracle(setup):
    T, m, h, psi, eps, rho, (dE_ref, vh_ref, eh_ref) = setup
    c = make(T, m, "mixed")
    out = c.correct(psi, eps, rho)
    vh = out["vhartree"].cpu().numpy()
    assert np.linalg.norm(vh - vh_ref) / np.linalg.norm(vh_ref) <= 1e-6
    # dE = -<psi V (psi - c)>_W / <c^2>_W with c = psiNew carrying <= 1e-6
    # relative error: dE moves by up to 1e-6 (|<psi V c>_W| + 2 |dE| <c^2>_W) / <c^2>_W
    W = h["W"]
    conv = out["psi_new"].cpu().numpy()
    veff = out["veff"].cpu().numpy()
    for mm in range(len(eps)):
        c2 = np.sum(W * conv[mm] ** 2)
        bound = 1e-6 * (abs(np.sum(W * psi[mm] * veff * conv[mm])) + 2 * abs(dE_ref[mm]) * c2) / c2
        assert abs(out["deltaE"][mm] - dE_ref[mm]) <= bound, (mm, bound)
    c.close()


def test_hartree_known_answer(setup):
    """Gaussian density: the two-mesh V_H (fine sources) is closer to
    erf(sqrt(a) r)/r than the coarse-only convolution with the same parameters."""
    T, m, h, *_ = setup
    a = 1.3
    X, Y, Z = h["X"], h["Y"], h["Z"]
    g = (a / np.pi) ** 1.5 * np.exp(-a * (X ** 2 + Y ** 2 + Z ** 2))
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    exact = erf(np.sqrt(a) * r) / r
    c = make(T, m, "fp64")
    vh, rho_f = c.hartree(torch.as_tensor(g, device="cuda"))
    err2 = np.linalg.norm(vh.cpu().numpy() - exact) / np.linalg.norm(exact)
    assert err2 <= 3e-4
    dev = importlib.import_module(T.__name__.rsplit(".", 1)[0] + ".device")
    plan = dev.TreecodePlan.for_mesh(m.X, m.Y, m.Z, m.W, theta=0.55, degree=9, source_leaf=500, target_leaf=500)
    gd = torch.as_tensor(g, device="cuda")
    v1 = plan.convolve(gd, gd, 1, [1.0], 2, precision="fp64")
    err1 = np.linalg.norm(v1.cpu().numpy() - exact) / np.linalg.norm(exact)
    assert err2 < err1
    # the fine-mesh density integrates to one like the coarse one
    assert abs(float((rho_f * m.Wf).sum()) - 1.0) < 1e-3
    c.close()
    plan.close()


def test_identity_fine_mesh_is_a_harrison_step(pkg, native):
    """With no fine cells (level 0) the fine mesh is the coarse mesh, the
    interpolation copies, and dE is the Harrison update of one Green-iteration
    step at the correction's parameters (oracle gi formula on one mesh)."""
    M = importlib.import_module(pkg.__name__ + ".mesh")
    T = importlib.import_module(pkg.__name__ + ".twomesh")
    m = M.build_mesh(6.0, 3.0, NUC, ORDER, 1.0, 3.0, 1.0, 0.0)
    assert torch.equal(m.X, m.Xf) and torch.equal(m.W, m.Wf)
    X, Y, Z, W = (t.cpu().numpy() for t in (m.X, m.Y, m.Z, m.W))
    r1 = np.sqrt((X - NUC[0, 0]) ** 2 + (Y - NUC[0, 1]) ** 2 + (Z - NUC[0, 2]) ** 2)
    psi = np.exp(-1.2 * r1)[None, :]
    psi /= np.sqrt((psi ** 2 * W).sum())
    rho = 2 * psi[0] ** 2
    eps = np.array([-0.55])
    c = T.TwoMeshCorrection(m.X, m.Y, m.Z, m.W, m.Xf, m.Yf, m.Zf, m.Wf, m.PtsPerCellCoarse, m.PtsPerCellFine,
                            ORDER, NUC, CHG, theta=0.7, degree=7, source_leaf=300, target_leaf=300,
                            precision="fp64")
    out = c.correct(psi, eps, rho)
    plan = O.Plan(X, Y, Z, X, Y, Z, W, 0.55, 9, 300, 300)
    vh = plan.convolve(rho, rho, W, 1, [1.0], 2)
    vx, _ = G.lda_exchange(rho)
    vext = -sum(Zc / np.sqrt((X - R[0]) ** 2 + (Y - R[1]) ** 2 + (Z - R[2]) ** 2) for R, Zc in zip(NUC, CHG))
    veff = vh + vx + vext - 0.5
    conv = plan.convolve(-2 * psi[0] * veff, -2 * psi[0] * veff, W, 2, [math.sqrt(1.1)], 2) / (4 * math.pi)
    dE = -np.sum(W * psi[0] * veff * (psi[0] - conv)) / np.sum(W * conv * conv)
    assert abs(out["deltaE"][0] - dE) <= 1e-9
    c.close()
