"""Device mesh generation (tagi_mesh_refine / tagi_mesh_points) on the GPU.

Bit-exact throughout: the cells and points are integer decisions and FP64
round-to-nearest arithmetic in the reference's order, so they must equal the
reference's own (golden fixture, made from the reference's functions) and
the oracle's restatement exactly, given the same 1-D node/weight tables.
"""
import ctypes
import hashlib
import importlib
import os

import numpy as np
import pytest
import torch

from oracle import mesh_oracle as MO

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "mesh_build_reference.npz")
NAMES = ("x", "y", "z", "w", "xf", "yf", "zf", "wf")


def digest(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).digest(), np.uint8)


@pytest.fixture(scope="module")
def M(native, pkg):
    return importlib.import_module(pkg.__name__ + ".mesh")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def case(g, t):
    XL, side, order, h, H, r, level = g[f"{t}_params"]
    return float(XL), float(side), int(order), float(h), float(H), float(r), float(level)


def host(m):
    return [t.cpu().numpy() for t in (m.X, m.Y, m.Z, m.W, m.Xf, m.Yf, m.Zf, m.Wf)]


@pytest.mark.parametrize("t", ("a", "b", "c"))
def test_device_mesh_matches_reference(M, gold, t):
    XL, side, order, h, H, r, level = case(gold, t)
    m = M.build_mesh(XL, side, gold[f"{t}_atoms"], order, h, H, r, level,
                     tables=(gold[f"{t}_u"], gold[f"{t}_W"]))
    for k, v in (("cx", m.cellX), ("cy", m.cellY), ("cz", m.cellZ), ("dx", m.cellDX), ("dy", m.cellDY),
                 ("dz", m.cellDZ), ("ppc_f", m.PtsPerCellFine)):
        assert np.array_equal(v.cpu().numpy(), gold[f"{t}_{k}"]), k
    assert np.all(m.PtsPerCellCoarse.cpu().numpy() == (order + 1) ** 3)
    for name, a in zip(NAMES, host(m)):
        assert len(a) == int(gold[f"{t}_{name}_len"]), name
        assert np.array_equal(a[::97], gold[f"{t}_{name}_every97"]), name
        assert np.array_equal(digest(a), gold[f"{t}_{name}_sha256"]), name


@pytest.mark.parametrize("level,min_depth", [(-2.0, 0), (-4.0, 1), (2.0, 0), (0.0, 2)])
def test_device_mesh_matches_oracle(M, syn, level, min_depth):
    """Ring molecule, 12 nuclei; fine meshes of 8 and 64 children, the r/4
    branch (level 2), forced refinement to a minimum depth."""
    nuclei, _ = syn.ring_molecule()
    XL, side, order, h, H, r = 12.0, 4.0, 2, 1.5, 4.0, 1.5
    tables = M.unit_tables(order)
    m = M.build_mesh(XL, side, nuclei, order, h, H, r, level, min_depth=min_depth, tables=tables)
    base = MO.base_cells(XL, XL, XL, side)
    tab = MO.cell_table(MO.refine(base, nuclei, h, H, r, level, min_depth), order)
    for k, v in (("cx", m.cellX), ("cy", m.cellY), ("cz", m.cellZ), ("dx", m.cellDX), ("dy", m.cellDY),
                 ("dz", m.cellDZ), ("ppc_c", m.PtsPerCellCoarse), ("ppc_f", m.PtsPerCellFine)):
        assert np.array_equal(v.cpu().numpy(), tab[k]), k
    for name, a, b in zip(NAMES, host(m), MO.points(tab, order, *tables)):
        assert np.array_equal(a, b), name


def test_large_mesh_properties(M, syn):
    """The 16.9M-point ring mesh of the mesh benchmark: both meshes' weights sum
    to the domain volume, cells tile the domain, every point lies in its cell,
    and a sample of cells equals the oracle's points."""
    nuclei, _ = syn.ring_molecule()
    XL, order = 20.0, 7
    m = M.build_mesh(XL, 5.0, nuclei, order, 1.0, 5.0, 2.0, -2.0)
    vol = (2 * XL) ** 3
    assert m.num_cells == 5104 and m.n == 5104 * 512 and m.Xf.numel() == 14282752
    for w in (m.W, m.Wf):
        assert abs(w.sum().item() - vol) / vol < 1e-12
    cv = (m.cellDX * m.cellDY * m.cellDZ).sum().item()
    assert abs(cv - vol) / vol < 1e-14
    p3 = (order + 1) ** 3
    cell = torch.arange(m.num_cells, device="cuda").repeat_interleave(p3)
    for P, c, d in ((m.X, m.cellX, m.cellDX), (m.Y, m.cellY, m.cellDY), (m.Z, m.cellZ, m.cellDZ)):
        assert bool(((P - c[cell]).abs() < d[cell] / 2).all())
    tab = {k: v.cpu().numpy() for k, v in (("cx", m.cellX), ("cy", m.cellY), ("cz", m.cellZ), ("dx", m.cellDX),
                                           ("dy", m.cellDY), ("dz", m.cellDZ), ("ppc_f", m.PtsPerCellFine))}
    tab_sub = {k: v[-40:] for k, v in tab.items()}
    ref = MO.points(tab_sub, order, *M.unit_tables(order))
    off_f = int(tab["ppc_f"][:-40].sum())
    got = host(m)
    for i, (a, b) in enumerate(zip(got, ref)):
        start = (m.num_cells - 40) * p3 if i < 4 else off_f
        assert np.array_equal(a[start:], b), NAMES[i]


def test_coarse_only_and_query(M, native, syn):
    nuclei, _ = syn.ring_molecule()
    m = M.build_mesh(10.0, 5.0, nuclei, 3, 1.0, 5.0, 2.0, -3.0, fine=False)
    assert m.Xf is None and m.n == m.num_cells * 64
    L = native.lib()
    base = torch.as_tensor(M.base_cells(10.0, 10.0, 10.0, 5.0), device="cuda")
    atoms = torch.as_tensor(np.ascontiguousarray(nuclei, np.float64), device="cuda")
    n, nc, nf = ctypes.c_int(0), ctypes.c_longlong(0), ctypes.c_longlong(0)
    null = [ctypes.c_void_p(0)] * 8
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = (ctypes.c_void_p(base.data_ptr()), base.shape[0], ctypes.c_void_p(atoms.data_ptr()), atoms.shape[0], 3,
            1.0, 5.0, 2.0, -3.0, 0, 16)
    assert L.tagi_mesh_refine(*args, *null, 0, ctypes.byref(n), ctypes.byref(nc), ctypes.byref(nf), s) == 0
    assert n.value == m.num_cells and nc.value == m.n
    assert nf.value == int(m.PtsPerCellFine.sum().item())
    # capacity too small: an error, with the count reported
    cells = [torch.empty(n.value - 1, dtype=torch.float64, device="cuda") for _ in range(6)]
    outs = [ctypes.c_void_p(c.data_ptr()) for c in cells] + [ctypes.c_void_p(0)] * 2
    rc = L.tagi_mesh_refine(*args, *outs, n.value - 1, ctypes.byref(n), ctypes.byref(nc), ctypes.byref(nf), s)
    assert rc == native.TAGI_ERR_ARG and n.value == m.num_cells


def test_rejected_inputs(M, native, pkg):
    err = pkg._native.TagiError
    atoms = [[0.1, 0.2, 0.3]]
    with pytest.raises(err, match="children"):          # 5^3 fine children: the reference exits too
        M.build_mesh(4.0, 4.0, atoms, 2, 1.0, 4.0, 1.0, -5.0)
    with pytest.raises(err, match="maxDepth"):          # the rule would refine below maxDepth
        M.build_mesh(4.0, 8.0, atoms, 2, 0.01, 8.0, 1.0, -2.0, max_depth=3)
    with pytest.raises(err, match="order"):
        M.build_mesh(4.0, 4.0, atoms, 16, 1.0, 4.0, 1.0, -2.0)
    m = M.build_mesh(4.0, 4.0, atoms, 2, 1.0, 4.0, 1.0, -2.0, fine=False)
    bad = m.PtsPerCellFine.clone()
    bad[0] = 2 * 27                                     # neither 1, 8, 27 nor 64 cells of 27 points
    cells = [m.cellX, m.cellY, m.cellZ, m.cellDX, m.cellDY, m.cellDZ]
    with pytest.raises(err, match="fine cell"):
        M.mesh_points(cells, bad, 2, int(bad.sum().item()))
    with pytest.raises(err, match="sums to"):
        M.mesh_points(cells, m.PtsPerCellFine, 2, int(m.PtsPerCellFine.sum().item()) + 27)


def test_default_tables_close_to_numpy(M, native):
    """NULL tables: the library's libm nodes/weights agree with numpy's to
    rounding (the bit pattern of a given numpy build needs the explicit tables)."""
    m = M.build_mesh(4.0, 4.0, [[0.1, 0.2, 0.3]], 5, 1.0, 4.0, 1.0, -2.0)
    cells = [m.cellX, m.cellY, m.cellZ, m.cellDX, m.cellDY, m.cellDZ]
    n = m.num_cells
    C = [torch.empty(n * 216, dtype=torch.float64, device="cuda") for _ in range(4)]
    p = [ctypes.c_void_p(c.data_ptr()) for c in cells]
    null = ctypes.POINTER(ctypes.c_double)()
    rc = native.lib().tagi_mesh_points(*p, ctypes.c_void_p(0), n, 5, null, null,
                                       *[ctypes.c_void_p(c.data_ptr()) for c in C], n * 216,
                                       *[ctypes.c_void_p(0)] * 4, 0,
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    for a, b in zip(C, (m.X, m.Y, m.Z, m.W)):
        assert torch.allclose(a, b, rtol=1e-14, atol=1e-14)
