"""Subsystem (e) on the GPU: weighted Gram-Schmidt and two-mesh interpolation
against the reference's own C (golden vectors) and the oracle restatement.

Tolerances: FP64 throughout; the device sums in a different order than the
reference's sequential loops, so agreement is to rounding, stated per test.
"""
import os

import numpy as np
import pytest
import torch

from conftest import rel_l2, to_cuda

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_mgs_device_matches_reference_golden(dev):
    g = np.load(os.path.join(GOLD, "mgs_reference.npz"))
    for tag in ("unitW", "randW"):
        V, W = to_cuda(g[f"{tag}_V_in"], g[f"{tag}_W"])
        for m in range(V.shape[0]):
            U = V[m].clone()
            dev.mgs(V, U, W, m)
            assert rel_l2(U.cpu().numpy(), g[f"{tag}_U_out"][m]) <= 1e-13, (tag, m)
        assert np.max(np.abs(V.cpu().numpy() - g[f"{tag}_V_out"])) <= 1e-13


def test_mgs_dropin_matches_reference_golden(pkg):
    orth = pkg.orthogonalization_wrapper
    g = np.load(os.path.join(GOLD, "mgs_reference.npz"))
    V = g["randW_V_in"].copy()
    W = g["randW_W"].copy()
    for m in range(V.shape[0]):
        U = np.copy(V[m])
        orth.callOrthogonalization(V, U, W, m, True)
        assert rel_l2(U, g["randW_U_out"][m]) <= 1e-13
    assert np.max(np.abs(V - g["randW_V_out"])) <= 1e-13


def test_mgs_large_orthonormal(dev, oracle):
    """Reference check (test_orthogonalization_wrapper.py:69,80) at 2e6 points."""
    rng = np.random.default_rng(3)
    n, m = 2_000_000, 6
    V0 = rng.random((m, n))
    Wn = rng.uniform(0.5, 1.5, n)
    V, W = to_cuda(V0, Wn)
    for t in range(m):
        U = V[t].clone()
        dev.mgs(V, U, W, t)
    Vh = V.cpu().numpy()
    G = (Vh * Wn) @ Vh.T
    assert np.max(np.abs(G - np.eye(m))) / n <= 1e-12
    # same arithmetic as the oracle restatement to rounding
    Vo = V0.copy()
    for t in range(m):
        U = Vo[t].copy()
        oracle.mgs(Vo, U, Wn, t)
    assert rel_l2(Vh, Vo) <= 1e-12


def test_mgs_rejects_bad_target(dev, native):
    V, W = to_cuda(np.ones((2, 10)), np.ones(10))
    with pytest.raises(native.TagiError):
        dev.mgs(V, V[0].clone(), W, 2)


def _case(g, p):
    return [g[p + k] for k in ("cX", "cY", "cZ", "cF", "fX", "fY", "fZ")]


@pytest.mark.parametrize("prefix", ["c175_", "mc_", "cn_"])
def test_interp_device_matches_reference_golden(dev, prefix):
    g = np.load(os.path.join(GOLD, "interp_reference.npz"))
    cX, cY, cZ, cF, fX, fY, fZ = _case(g, prefix)
    order = int(g[prefix + "order"])
    if prefix == "mc_":
        ppc_c, ppc_f, ncell, f0 = g["mc_ppc_c"], g["mc_ppc_f"], 3, g["mc_fineF0"]
    else:
        ppc_c, ppc_f, ncell, f0 = np.array([len(cX)]), np.array([len(fX)]), 1, np.zeros(len(fX))
    t = to_cuda(cX, cY, cZ, cF, fX, fY, fZ, f0)
    pc = torch.as_tensor(ppc_c.astype(np.int32), device="cuda")
    pf = torch.as_tensor(ppc_f.astype(np.int32), device="cuda")
    out = dev.interp(t[0], t[1], t[2], t[3], pc, t[4], t[5], t[6], pf, ncell, order, fineF=t[7])
    ref = g[prefix + "out"]
    assert np.max(np.abs(out.cpu().numpy() - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_interp_dropin_known_integral(pkg):
    """meshUtilities.py:1753: integral of interp(x^4 y^4) z^6 over the 8 children = 1/175."""
    interp = pkg.interpolation_wrapper
    g = np.load(os.path.join(GOLD, "interp_reference.npz"))
    cX, cY, cZ, cF, fX, fY, fZ = _case(g, "c175_")
    out = interp.callInterpolator(cX, cY, cZ, cF, np.array([len(cX)]), fX, fY, fZ,
                                  np.array([len(fX)]), 1, 6, True)
    assert abs(np.sum(out * fZ ** 6 * g["c175_fW"]) - 1 / 175) < 1e-12
    assert np.max(np.abs(out - g["c175_out"])) <= 1e-13


def test_interp_whole_mesh_copy(pkg):
    interp = pkg.interpolation_wrapper
    a = np.linspace(0, 1, 27)
    out = interp.callInterpolator(a, a, a, 3 * a, np.array([27]), a, a, a, np.array([27]), 1, 2, True)
    assert np.array_equal(out, 3 * a)


def test_interp_rejects_inconsistent_cells(pkg, native):
    interp = pkg.interpolation_wrapper
    a = np.linspace(0, 1, 27)
    b = np.linspace(0, 1, 54)
    with pytest.raises(native.TagiError):
        interp.callInterpolator(a, a, a, a, np.array([30]), b, b, b, np.array([54]), 1, 2, True)


@pytest.mark.parametrize("shuffle", [False, True])
def test_interp_tensor_and_general_paths_match_oracle(dev, oracle, shuffle):
    """Fine points on tensor grids per child block take the sum-factorised path;
    the same points in shuffled order (no tensor structure) take the per-point
    formula.  Both equal the oracle's restatement of the reference to 1e-13."""
    from oracle import mesh_oracle as MO
    pkg = __import__("importlib").import_module("treecode-accelerated-green-iteration_gb300")
    nuclei, _ = pkg.synthetic.ring_molecule()
    order = 5
    tab, pts = MO.build(20.0, 5.0, nuclei, order, 3.0, 5.0, 2.0, -2.0)
    X, Y, Z, W, Xf, Yf, Zf, Wf = pts
    F = np.exp(-np.sqrt(X ** 2 + Y ** 2 + Z ** 2) / 3.0) * (1.0 + 0.1 * X)
    ppc_c, ppc_f = tab["ppc_c"].astype(np.int32), tab["ppc_f"].astype(np.int32)
    if shuffle:   # permute the fine points inside every cell
        rng = np.random.default_rng(9)
        off = np.concatenate([[0], np.cumsum(ppc_f)])
        perm = np.concatenate([off[c] + rng.permutation(ppc_f[c]) for c in range(len(ppc_f))])
        Xf, Yf, Zf = Xf[perm], Yf[perm], Zf[perm]
    ref = oracle.interp(X, Y, Z, F, ppc_c, Xf, Yf, Zf, ppc_f, len(ppc_c), order)
    t = to_cuda(X, Y, Z, F, Xf, Yf, Zf)
    pc = torch.as_tensor(ppc_c, device="cuda")
    pf = torch.as_tensor(ppc_f, device="cuda")
    out = dev.interp(t[0], t[1], t[2], t[3], pc, t[4], t[5], t[6], pf, len(ppc_c), order).cpu().numpy()
    assert np.max(np.abs(out - ref)) <= 1e-13 * np.max(np.abs(ref))
