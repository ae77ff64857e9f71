"""The CPU oracle, pinned before it is trusted (no GPU needed).

* MGS and interpolation restatements == the reference's own C
  (oracle/_ref, compiled from the reference sources where present) and ==
  the committed golden vectors made by that C.
* Known answers: the interpolation integral 1/175 of meshUtilities.py:1753,
  the MGS tolerances of test_orthogonalization_wrapper.py:69,80, closed-form
  Coulomb/Yukawa convolutions for the direct sum.
* Treecode restatement vs direct sum (approximation error) and list
  invariants.  Treecode parity against BaryTree itself is unpinned: BaryTree
  is not part of the reference.
"""
import os

import numpy as np
import pytest
from scipy.special import erf

from conftest import rel_l2

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_mgs_matches_reference_golden(oracle):
    g = np.load(os.path.join(GOLD, "mgs_reference.npz"))
    for tag in ("unitW", "randW"):
        V = g[f"{tag}_V_in"].copy()
        W = g[f"{tag}_W"]
        for m in range(V.shape[0]):
            U = V[m].copy()
            oracle.mgs(V, U, W, m)
            assert np.array_equal(U, g[f"{tag}_U_out"][m]), (tag, m)
        assert np.array_equal(V, g[f"{tag}_V_out"]), tag


def test_mgs_reference_tolerances(oracle):
    """test_orthogonalization_wrapper.py:69,80: overlaps/N and (norm-1)/N <= 1e-12."""
    rng = np.random.default_rng(0)
    n, m = 2000, 8
    V = rng.random((m, n))
    W = np.ones(n)
    for t in range(m):
        U = V[t].copy()
        oracle.mgs(V, U, W, t)
    G = V @ V.T
    assert np.max(np.abs(G - np.diag(np.diag(G)))) / n <= 1e-12
    assert np.max(np.abs(np.diag(G) - 1)) / n <= 1e-12


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLD), "..", "oracle", "_ref",
                                                    "libref_orth.so")),
                    reason="reference C not compiled here (reference tree absent)")
def test_mgs_matches_compiled_reference(oracle):
    rng = np.random.default_rng(1)
    V1 = rng.normal(size=(5, 777))
    V2 = V1.copy()
    W = rng.uniform(0.1, 3, 777)
    for m in range(5):
        U1, U2 = V1[m].copy(), V2[m].copy()
        oracle.mgs(V1, U1, W, m)
        oracle.ref_mgs(V2, U2, W, m)
        assert np.array_equal(U1, U2)
    assert np.array_equal(V1, V2)


def _interp_case(g, p):
    return dict(cX=g[p + "cX"], cY=g[p + "cY"], cZ=g[p + "cZ"], cF=g[p + "cF"], fX=g[p + "fX"],
                fY=g[p + "fY"], fZ=g[p + "fZ"])


def test_interp_matches_reference_golden(oracle):
    g = np.load(os.path.join(GOLD, "interp_reference.npz"))
    c = _interp_case(g, "c175_")
    out = oracle.interp(c["cX"], c["cY"], c["cZ"], c["cF"], [len(c["cX"])], c["fX"], c["fY"],
                        c["fZ"], [len(c["fX"])], 1, int(g["c175_order"]))
    assert np.array_equal(out, g["c175_out"])
    c = _interp_case(g, "mc_")
    out = oracle.interp(c["cX"], c["cY"], c["cZ"], c["cF"], g["mc_ppc_c"], c["fX"], c["fY"],
                        c["fZ"], g["mc_ppc_f"], 3, int(g["mc_order"]), fineF=g["mc_fineF0"])
    assert np.array_equal(out, g["mc_out"])
    c = _interp_case(g, "cn_")  # fine points on coarse nodes (exact-node branches)
    out = oracle.interp(c["cX"], c["cY"], c["cZ"], c["cF"], [len(c["cX"])], c["fX"], c["fY"],
                        c["fZ"], [len(c["fX"])], 1, int(g["cn_order"]))
    assert np.array_equal(out, g["cn_out"])


def test_interp_known_integral(oracle):
    """meshUtilities.py:1682-1794: integral of interp(x^4 y^4) * z^6 over [0,1]^3 = 1/175."""
    g = np.load(os.path.join(GOLD, "interp_reference.npz"))
    c = _interp_case(g, "c175_")
    out = oracle.interp(c["cX"], c["cY"], c["cZ"], c["cF"], [len(c["cX"])], c["fX"], c["fY"],
                        c["fZ"], [len(c["fX"])], 1, 6)
    integral = np.sum(out * g["c175_fZ"] ** 6 * g["c175_fW"])
    assert abs(integral - 1 / 175) < 1e-12


def test_interp_whole_mesh_copy(oracle):
    """TwoMeshInterpolation.c:175-180: equal sizes copy (overwrite) and return."""
    a = np.arange(10.0)
    out = oracle.interp(a, a, a, a * 2, [10], a, a, a, [10], 1, 1, fineF=np.ones(10))
    assert np.array_equal(out, a * 2)


def test_mesh_points_weights_match_reference(syn):
    g = np.load(os.path.join(GOLD, "mesh_reference.npz"))
    for order in range(2, 10):
        assert np.allclose(syn.cheb1_points(-1.5, 2.5, order), g[f"points_{order}"], rtol=0, atol=1e-14)
        assert np.allclose(syn.cheb1_weights_unscaled(order), g[f"weights_{order}"], rtol=0, atol=1e-14)
        x, y, z, w = syn.cell_points(np.array([[0.0, -1.0, 3.0]]), np.array([[1.0, 2.0, 3.5]]), order)
        assert np.allclose(w, g[f"w3d_{order}"].ravel(), rtol=1e-13, atol=0)


def test_direct_sum_coulomb_gaussian(oracle, syn):
    """Coulomb potential of a normalized Gaussian is erf(sqrt(a) r)/r."""
    mesh, f, rho = syn.single_atom(factor=1.0, max_depth=5)
    a = 1.3
    r2 = mesh.x ** 2 + mesh.y ** 2 + mesh.z ** 2
    g = (a / np.pi) ** 1.5 * np.exp(-a * r2)
    sub = np.arange(0, mesh.n, 211)
    V = oracle.direct(mesh.x, mesh.y, mesh.z, g, mesh.x, mesh.y, mesh.z, g, mesh.w, 1, [1.0], 2,
                      subset=sub)
    r = np.sqrt(r2[sub])
    exact = erf(np.sqrt(a) * r) / r
    assert rel_l2(V, exact) < 5e-4


def test_direct_sum_hydrogen_fixed_point(oracle, syn):
    """psi = e^-r/sqrt(pi), V = -1/r, k = 1: (1/4pi) G_k * (-2 V psi) = psi."""
    mesh, _, _ = syn.single_atom(factor=1.0, max_depth=5)
    r = np.sqrt(mesh.x ** 2 + mesh.y ** 2 + mesh.z ** 2)
    psi = np.exp(-r) / np.sqrt(np.pi)
    f = 2.0 / r * psi
    sub = np.arange(0, mesh.n, 211)
    phi = oracle.direct(mesh.x, mesh.y, mesh.z, f, mesh.x, mesh.y, mesh.z, f, mesh.w, 2, [1.0], 2,
                        subset=sub)
    assert rel_l2(phi / (4 * np.pi), psi[sub]) < 1e-2


def test_treecode_oracle_vs_direct(oracle, small_mesh):
    mesh, f, rho = small_mesh
    p = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, 7, 300, 300, 1.0)
    assert p.n_far > 0
    sub = np.arange(0, mesh.n, 13)
    for kern, q in ((2, f), (1, rho)):
        tc = p.convolve(q, q, mesh.w, kern, [1.0], 2)
        d = oracle.direct(mesh.x, mesh.y, mesh.z, q, mesh.x, mesh.y, mesh.z, q, mesh.w, kern, [1.0], 2,
                          subset=sub)
        assert rel_l2(tc[sub], d) < 1e-6


def test_theta_zero_is_direct_sum(oracle, small_mesh):
    mesh, f, rho = small_mesh
    p = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.0, 3, 300, 300, 1.0)
    assert p.n_far == 0
    tc = p.convolve(f, f, mesh.w, 2, [1.3], 2)
    d = oracle.direct(mesh.x, mesh.y, mesh.z, f, mesh.x, mesh.y, mesh.z, f, mesh.w, 2, [1.3], 2)
    assert rel_l2(tc, d) < 1e-13


def test_oracle_lists_partition_sources(oracle, small_mesh):
    mesh = small_mesh[0]
    p = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, 5, 100, 100, 1.0)
    st, L = p.tree(0), p.lists()
    for b in range(p.n_batches):
        cover = np.zeros(mesh.n, np.int32)
        for e in range(L["near_off"][b], L["near_off"][b + 1]):
            c = L["near_list"][e]
            cover[st["begin"][c]:st["end"][c]] += 1
        for e in range(L["far_off"][b], L["far_off"][b + 1]):
            c = L["far_list"][e]
            cover[st["begin"][c]:st["end"][c]] += 1
        assert cover.min() == 1 and cover.max() == 1
