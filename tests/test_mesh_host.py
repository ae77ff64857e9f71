"""Mesh generation on the host side (no GPU): the oracle's restatement of the
reference's two-level mesh is pinned against the reference itself
(tests/golden/mesh_build_reference.npz, made by make_golden.py from the
reference's own divide rule and cell-point functions), bit for bit; the
package's host helpers (base cells, 1-D tables) equal the oracle's."""
import hashlib
import importlib
import os

import numpy as np
import pytest

from oracle import mesh_oracle as MO

GOLD = os.path.join(os.path.dirname(__file__), "golden", "mesh_build_reference.npz")
CASES = ("a", "b", "c")


def digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).digest(), np.uint8)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def M(pkg):
    return importlib.import_module(pkg.__name__ + ".mesh")


def case(g, t):
    XL, side, order, h, H, r, level = g[f"{t}_params"]
    return float(XL), float(side), int(order), float(h), float(H), float(r), float(level)


@pytest.mark.parametrize("t", CASES)
def test_oracle_cells_match_reference(gold, t):
    XL, side, order, h, H, r, level = case(gold, t)
    base = MO.base_cells(XL, XL, XL, side)
    assert np.array_equal(base, gold[f"{t}_base"])
    leaves = MO.refine(base, gold[f"{t}_atoms"], h, H, r, level)
    tab = MO.cell_table(leaves, order)
    for k in ("cx", "cy", "cz", "dx", "dy", "dz", "ppc_f"):
        assert np.array_equal(tab[k], gold[f"{t}_{k}"]), k


@pytest.mark.parametrize("t", CASES)
def test_oracle_points_match_reference(gold, t):
    XL, side, order, h, H, r, level = case(gold, t)
    tab = {k: gold[f"{t}_{k}"] for k in ("cx", "cy", "cz", "dx", "dy", "dz", "ppc_f")}
    pts = MO.points(tab, order, gold[f"{t}_u"], gold[f"{t}_W"])
    for name, a in zip(("x", "y", "z", "w", "xf", "yf", "zf", "wf"), pts):
        assert len(a) == int(gold[f"{t}_{name}_len"]), name
        assert np.array_equal(a[::97], gold[f"{t}_{name}_every97"]), name
        assert np.array_equal(digest(a), gold[f"{t}_{name}_sha256"]), name


def test_fixture_covers_the_rule(gold):
    """The fixture holds unrefined and fine cells of 8 and 27 children and a
    level >= 1 case (the r/2 branch)."""
    ppc = {t: set(np.unique(gold[f"{t}_ppc_f"] // (case(gold, t)[2] + 1) ** 3)) for t in CASES}
    assert ppc["a"] == {1, 8} and ppc["b"] == {1, 27} and ppc["c"] == {1}
    assert case(gold, "c")[6] >= 1


@pytest.mark.parametrize("t", CASES)
def test_weights_sum_to_volume(gold, t):
    """mpiMeshBuilding.py:456-459 checks the cell volumes; the quadrature weights
    integrate 1 exactly, so both meshes' weights sum to the domain volume."""
    XL, side, order, h, H, r, level = case(gold, t)
    tab = {k: gold[f"{t}_{k}"] for k in ("cx", "cy", "cz", "dx", "dy", "dz", "ppc_f")}
    x, y, z, w, xf, yf, zf, wf = MO.points(tab, order)
    vol = (2 * XL) ** 3
    assert abs(w.sum() - vol) / vol < 1e-12 and abs(wf.sum() - vol) / vol < 1e-12
    assert abs(np.sum(tab["dx"] * tab["dy"] * tab["dz"]) - vol) / vol < 1e-14


@pytest.mark.parametrize("t", CASES)
def test_package_host_helpers_match_oracle(M, gold, t):
    XL, side, order, *_ = case(gold, t)
    assert np.array_equal(M.base_cells(XL, XL, XL, side), MO.base_cells(XL, XL, XL, side))
    u, W = M.unit_tables(order)
    assert np.array_equal(u, MO.unit_nodes(order)) and np.array_equal(W, MO.unit_weights(order))
    # here (where the fixture was made) they are the reference's tables too
    assert np.array_equal(u, gold[f"{t}_u"]) and np.array_equal(W, gold[f"{t}_W"])


def test_base_cells_uneven_domain(M):
    """Non-cubic domain and a side that does not divide it (ceil rule, linspace)."""
    b = M.base_cells(7.0, 5.0, 3.0, 2.5)
    assert b.shape == (6 * 4 * 3, 6)
    assert np.array_equal(b, MO.base_cells(7.0, 5.0, 3.0, 2.5))


def test_oracle_rejects_depth_overflow():
    with pytest.raises(ValueError):
        MO.refine(MO.base_cells(4.0, 4.0, 4.0, 8.0), [[0.1, 0.2, 0.3]], 0.01, 8.0, 1.0, -2.0, max_depth=3)


def test_two_mesh_oracle_identity_mesh(oracle):
    """The oracle's two-mesh correction with fine mesh == coarse mesh (no fine
    cells) is one Harrison update at theta - 0.15, degree + 2."""
    import math
    from oracle import gi_oracle as G
    nuc, chg = np.array([[0.3, -0.2, 0.1]]), np.array([1.0])
    tab, (X, Y, Z, W, Xf, Yf, Zf, Wf) = MO.build(4.0, 4.0, nuc, 2, 1.0, 4.0, 1.0, 0.0)
    assert np.array_equal(X, Xf) and np.array_equal(W, Wf)
    r = np.sqrt((X - 0.3) ** 2 + (Y + 0.2) ** 2 + (Z - 0.1) ** 2)
    psi = np.exp(-r)[None, :]
    psi /= np.sqrt((psi ** 2 * W).sum())
    rho = 2 * psi[0] ** 2
    dE, vh, eh = G.two_mesh_correction((X, Y, Z, W), (Xf, Yf, Zf, Wf), tab["ppc_c"], tab["ppc_f"], 2, nuc, chg,
                                       psi, np.array([-0.5]), rho, 0.7, 5, 200, 200)
    plan = oracle.Plan(X, Y, Z, X, Y, Z, W, 0.55, 7, 200, 200)
    vh1 = plan.convolve(rho, rho, W, 1, [1.0], 2)
    assert np.array_equal(vh, vh1)
    veff = vh1 + G.lda_exchange(rho)[0] - 1.0 / r - 0.5
    c = plan.convolve(-2 * psi[0] * veff, -2 * psi[0] * veff, W, 2, [1.0], 2) / (4 * math.pi)
    d = -np.sum(W * psi[0] * veff * (psi[0] - c)) / np.sum(W * c * c)
    assert abs(dE[0] - d) <= 1e-12 * max(1.0, abs(d))


def _level_sync_order(base, atoms, h, H, r, level, min_depth=0, depth_bits=16):
    """The device refinement's ordering scheme, restated: cells emitted level by
    level, each carrying a path key (base index << 48 | 3-bit child digit per
    level), leaves sorted by key at the end."""
    atoms = [tuple(a) for a in np.asarray(atoms, np.float64).reshape(-1, 3)]
    cells = [tuple(map(float, b)) for b in base]
    keys = [i << 48 for i in range(len(cells))]
    leaves, depth = [], 0
    while cells:
        nxt, nkeys = [], []
        for c, k in zip(cells, keys):
            div, fine = (True, 1) if depth < min_depth else MO.divide_rule(c, atoms, h, H, r, level)
            if not div:
                leaves.append((k, c, fine))
                continue
            xb = [c[0], (c[1] + c[0]) / 2, c[1]]
            yb = [c[2], (c[3] + c[2]) / 2, c[3]]
            zb = [c[4], (c[5] + c[4]) / 2, c[5]]
            for q in range(8):
                i, j, kk = q >> 2, (q >> 1) & 1, q & 1
                nxt.append((xb[i], xb[i + 1], yb[j], yb[j + 1], zb[kk], zb[kk + 1]))
                nkeys.append(k | (q << (3 * (depth_bits - 1 - depth))))
        cells, keys, depth = nxt, nkeys, depth + 1
    leaves.sort(key=lambda t: t[0])
    return [(c, f) for _, c, f in leaves]


@pytest.mark.parametrize("level,min_depth", [(-2.0, 0), (0.0, 2), (2.0, 0)])
def test_path_key_order_is_depth_first(syn, level, min_depth):
    """Sorting leaves by padded path key gives the reference's uniqueID
    (depth-first, x-major) order: a leaf is never a prefix of another leaf."""
    nuclei, _ = syn.ring_molecule()
    base = MO.base_cells(12.0, 12.0, 12.0, 4.0)
    a = _level_sync_order(base, nuclei, 1.5, 4.0, 1.5, level, min_depth)
    b = MO.refine(base, nuclei, 1.5, 4.0, 1.5, level, min_depth)
    assert len(a) == len(b)
    assert all(x[0] == tuple(y[0]) and x[1] == y[1] for x, y in zip(a, b))


def test_high_multiply_index_split_is_exact():
    """The points kernel splits q = i p^2 + j p + k with high multiplies by
    ceil(2^32 / d) (d = p, p^2; 0 for d = 1, where q is always 0): exact for
    every order 0..15 and every q < (order+1)^3."""
    for p1 in range(1, 17):
        p2, p3 = p1 * p1, p1 * p1 * p1
        m1 = -(-(1 << 32) // p1) if p1 > 1 else 0
        m2 = -(-(1 << 32) // p2) if p2 > 1 else 0
        assert m1 < (1 << 32) and m2 < (1 << 32)
        q = np.arange(p3, dtype=np.uint64)
        hi = lambda a, m: (a * np.uint64(m)) >> np.uint64(32)
        t = hi(q, m1)
        i, j, k = hi(q, m2), t - hi(t, m1) * np.uint64(p1), q - t * np.uint64(p1)
        assert np.array_equal(i, q // p2) and np.array_equal(j, (q // p1) % p1) and np.array_equal(k, q % p1)
