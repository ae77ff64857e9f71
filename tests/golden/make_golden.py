"""Generate the golden vectors in this directory from the REFERENCE itself.

Run here, where the reference tree is mounted (it is not on the GPU machine):
    python tests/golden/make_golden.py
It needs oracle/_ref (``make -C oracle ref``: the reference's own
Orthogonalization.c and TwoMeshInterpolation.c compiled from their sources)
and imports the reference's Python meshUtilities.py for the Chebyshev
first-kind points and weights, and mpiMeshBuilding.py / CellStruct_CC.py for
the two-level mesh (refinement rule and cell points).  Outputs (small .npz
files) are committed.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_ROOT = os.environ.get("TAGI_REFERENCE", "/root/reference")   # the reference repository's root
REF_UTIL = os.path.join(REF_ROOT, "3D-GreenIteration", "src", "utilities")
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def reference_mesh_utilities():
    """Import meshUtilities.py with its unused heavy imports stubbed out."""
    sys.modules.setdefault("vtk", types.ModuleType("vtk"))
    sys.modules.setdefault("interpolation_wrapper", types.ModuleType("interpolation_wrapper"))
    sys.path.insert(0, REF_UTIL)
    import meshUtilities
    return meshUtilities


def mgs_golden():
    """Sequential MGS of 6 random vectors (uniform weights like
    test_orthogonalization_wrapper.py:31, and random weights) with the reference C."""
    rng = np.random.default_rng(20240601)
    out = {}
    for tag, W in (("unitW", np.ones(400)), ("randW", rng.uniform(0.1, 2.0, 400))):
        V0 = rng.random((6, 400))
        V = V0.copy()
        Us = []
        for m in range(6):
            U = V[m].copy()
            O.ref_mgs(V, U, W, m)
            Us.append(U.copy())
        out[f"{tag}_V_in"] = V0
        out[f"{tag}_W"] = W
        out[f"{tag}_V_out"] = V
        out[f"{tag}_U_out"] = np.array(Us)
    np.savez_compressed(os.path.join(HERE, "mgs_reference.npz"), **out)


def _cell(lo, hi, order, mu):
    x = mu.ChebyshevPointsFirstKind(lo[0], hi[0], order)
    y = mu.ChebyshevPointsFirstKind(lo[1], hi[1], order)
    z = mu.ChebyshevPointsFirstKind(lo[2], hi[2], order)
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    w = mu.weights3DFirstKind(lo[0], hi[0], order, lo[1], hi[1], order, lo[2], hi[2], order)
    return X.ravel(), Y.ravel(), Z.ravel(), np.asarray(w).ravel()


def interp_golden(mu):
    """(1) meshUtilities.py:1682-1794: order 6, unit cube, one coarse cell -> 8
    children, f = x^4 y^4, known integral of f*z^6 = 1/175.  (2) a 3-cell mesh
    mixing an unrefined cell, an 8-child cell and a 27-child cell, order 4."""
    out = {}
    order = 6
    cx, cy, cz, cw = _cell((0, 0, 0), (1, 1, 1), order, mu)
    fx, fy, fz, fw = [], [], [], []
    for i in range(2):
        for j in range(2):
            for k in range(2):
                lo = (0.5 * i, 0.5 * j, 0.5 * k)
                hi = (0.5 + 0.5 * i, 0.5 + 0.5 * j, 0.5 + 0.5 * k)
                a = _cell(lo, hi, order, mu)
                fx.append(a[0]); fy.append(a[1]); fz.append(a[2]); fw.append(a[3])
    fx, fy, fz, fw = map(np.concatenate, (fx, fy, fz, fw))
    cF = cx ** 4 * cy ** 4
    res = O.ref_interp(cx, cy, cz, cF, [len(cx)], fx, fy, fz, [len(fx)], 1, order)
    out.update(c175_cX=cx, c175_cY=cy, c175_cZ=cz, c175_cF=cF, c175_fX=fx, c175_fY=fy, c175_fZ=fz,
               c175_fW=fw, c175_out=res, c175_order=order)
    # multi-cell mesh
    order = 4
    rng = np.random.default_rng(3)
    cells = [((0, 0, 0), (1, 1, 1), 1), ((1, 0, 0), (2, 1, 1), 8), ((0, 1, 0), (1, 2, 1), 27)]
    CX, CY, CZ, FX, FY, FZ, ppc_c, ppc_f = [], [], [], [], [], [], [], []
    for lo, hi, nch in cells:
        a = _cell(lo, hi, order, mu)
        CX.append(a[0]); CY.append(a[1]); CZ.append(a[2]); ppc_c.append(len(a[0]))
        m = round(nch ** (1 / 3))
        fxs, fys, fzs = [], [], []
        for i in range(m):
            for j in range(m):
                for k in range(m):
                    l2 = tuple(lo[d] + (hi[d] - lo[d]) * (i, j, k)[d] / m for d in range(3))
                    h2 = tuple(lo[d] + (hi[d] - lo[d]) * ((i, j, k)[d] + 1) / m for d in range(3))
                    b = _cell(l2, h2, order, mu)
                    fxs.append(b[0]); fys.append(b[1]); fzs.append(b[2])
        FX.append(np.concatenate(fxs)); FY.append(np.concatenate(fys)); FZ.append(np.concatenate(fzs))
        ppc_f.append(len(FX[-1]))
    CX, CY, CZ, FX, FY, FZ = map(np.concatenate, (CX, CY, CZ, FX, FY, FZ))
    CF = np.sin(CX) * np.cos(2 * CY) + CZ ** 3 + rng.normal(0, 0.01, len(CX))
    fineF0 = rng.normal(0, 1, len(FX))
    res = O.ref_interp(CX, CY, CZ, CF, ppc_c, FX, FY, FZ, ppc_f, 3, order, fineF=fineF0)
    out.update(mc_cX=CX, mc_cY=CY, mc_cZ=CZ, mc_cF=CF, mc_ppc_c=np.array(ppc_c, np.int32), mc_fX=FX,
               mc_fY=FY, mc_fZ=FZ, mc_ppc_f=np.array(ppc_f, np.int32), mc_fineF0=fineF0, mc_out=res,
               mc_order=order)
    # coincident nodes: fine points sharing x (or z, or x and z) with coarse
    # nodes exercise the exact-node branches (TwoMeshInterpolation.c:124-140)
    order = 3
    cx, cy, cz, _ = _cell((0, 0, 0), (1, 1, 1), order, mu)
    nodes = mu.ChebyshevPointsFirstKind(0, 1, order)
    rng2 = np.random.default_rng(9)
    px = rng2.uniform(0, 1, 64)
    py = rng2.uniform(0, 1, 64)
    pz = rng2.uniform(0, 1, 64)
    px[:16] = nodes[rng2.integers(0, order + 1, 16)]
    pz[16:32] = nodes[rng2.integers(0, order + 1, 16)]
    px[32:40] = nodes[1]
    pz[32:40] = nodes[2]
    py[40:48] = nodes[0]
    cF = np.cos(cx) + cy * cz + 0.1 * cx * cz
    res = O.ref_interp(cx, cy, cz, cF, [len(cx)], px, py, pz, [64], 1, order)
    out.update(cn_cX=cx, cn_cY=cy, cn_cZ=cz, cn_cF=cF, cn_fX=px, cn_fY=py, cn_fZ=pz, cn_out=res,
               cn_order=order)
    np.savez_compressed(os.path.join(HERE, "interp_reference.npz"), **out)


def mesh_golden(mu):
    """First-kind Chebyshev points / weights of the reference (meshUtilities.py:839-883)."""
    out = {}
    for order in range(2, 10):
        out[f"points_{order}"] = mu.ChebyshevPointsFirstKind(-1.5, 2.5, order)
        out[f"weights_{order}"] = mu.unscaledWeightsFirstKind(order)
        out[f"w3d_{order}"] = np.asarray(mu.weights3DFirstKind(0, 1, order, -1, 2, order, 3, 3.5, order))
    np.savez_compressed(os.path.join(HERE, "mesh_reference.npz"), **out)


REF_DATA = os.path.join(REF_ROOT, "3D-GreenIteration", "src", "dataStructures")


def reference_mesh_building():
    """Import the reference's mpiMeshBuilding.py and CellStruct_CC.py on one
    rank: mpi4py is a one-rank stand-in; the tree, atom, Zoltan, memory
    tracker and grid-point modules, which the imported functions do not use
    here, are empty stand-ins."""
    class _Comm:
        def Get_rank(self):
            return 0

        def Get_size(self):
            return 1

        def barrier(self):
            pass

        def allreduce(self, v):
            return v

    mpi = types.ModuleType("mpi4py")
    mpi.MPI = types.SimpleNamespace(COMM_WORLD=_Comm(), Wtime=lambda: 0.0)
    sys.modules["mpi4py"] = mpi
    sys.modules["mpi4py.MPI"] = mpi.MPI
    for name in ("pympler", "TreeStruct_CC", "AtomStruct", "zoltan_wrapper", "GridpointStruct"):
        m = types.ModuleType(name)
        m.tracker = m.classtracker = m.Tree = m.Atom = m.callZoltan = None
        m.GridPoint = lambda *a, **k: None
        sys.modules[name] = m
    sys.modules.setdefault("vtk", types.ModuleType("vtk"))
    sys.modules.setdefault("interpolation_wrapper", types.ModuleType("interpolation_wrapper"))
    import scipy.special
    if not hasattr(scipy.special, "sph_harm"):
        scipy.special.sph_harm = None
    sys.path[:0] = [REF_UTIL, REF_DATA]
    import CellStruct_CC
    import mpiMeshBuilding
    return mpiMeshBuilding, CellStruct_CC


def mesh_build_golden():
    """A whole two-level mesh made by the reference's own functions:
    base cells by inializeBaseMesh_distributed (mpiMeshBuilding.py:68-124),
    each cell's decision by Cell.refineCoarseningUniform_TwoLevel
    (CellStruct_CC.py:2344-2491) on a stand-in cell object, and the points by
    coarse/fineQuadraturePointsSingleCell (mpiMeshBuilding.py:725-840).  The
    recursion driving the rule restates recursiveDivide
    (TreeStruct_CC.py:1049-1140): midpoint split, children x-major, depth
    first, which is the uniqueID order extractCellXYZ walks."""
    mb, cs = reference_mesh_building()
    out = {}
    cases = {
        # domain, base side, atoms, order, h, H, r, level
        "a": (8.0, 4.0, [[0.3, -0.2, 0.1], [-2.6, 1.45, 2.05]], 3, 1.0, 4.0, 1.0, -2.0),
        "b": (6.0, 3.0, [[0.05, 0.4, -1.3]], 2, 0.75, 3.0, 1.5, -3.0),
        "c": (5.0, 2.5, [[1.1, -0.7, 0.2], [-1.9, 0.3, -2.2], [0.0, 2.4, 1.0]], 2, 0.6, 2.5, 0.8, 1.0),
    }
    for tag, (XL, side, atoms, order, h, H, r, level) in cases.items():
        _, _, _, cells = mb.inializeBaseMesh_distributed(XL, XL, XL, side, verbose=0)
        atom_objs = [types.SimpleNamespace(x=a[0], y=a[1], z=a[2]) for a in atoms]
        tree = types.SimpleNamespace(atoms=atom_objs)
        uw = mb.unscaledWeightsFirstKind(order)
        leaves = []

        def visit(b, depth):
            c = types.SimpleNamespace(xmin=b[0], xmax=b[1], ymin=b[2], ymax=b[3], zmin=b[4], zmax=b[5],
                                      px=order, py=order, pz=order, tree=tree, unscaledW=uw,
                                      numCoarsePoints=(order + 1) ** 3)
            c.w = mb.weights3DFirstKind(b[0], b[1], order, b[2], b[3], order, b[4], b[5], order, uw)
            cs.Cell.refineCoarseningUniform_TwoLevel(c, h, H, r, level)
            if not c.divideFlag:
                leaves.append((b, int(c.numFinePoints) if c.fineMesh else int(c.numCoarsePoints)))
                return
            xd, yd, zd = (b[1] + b[0]) / 2, (b[3] + b[2]) / 2, (b[5] + b[4]) / 2
            xb = np.array([b[0], float(xd), b[1]])
            yb = np.array([b[2], float(yd), b[3]])
            zb = np.array([b[4], float(zd), b[5]])
            for i in range(2):
                for j in range(2):
                    for k in range(2):
                        visit((xb[i], xb[i + 1], yb[j], yb[j + 1], zb[k], zb[k + 1]), depth + 1)

        for row in cells:
            visit(tuple(row), 0)
        cx = np.array([(b[0] + b[1]) / 2 for b, _ in leaves])
        cy = np.array([(b[2] + b[3]) / 2 for b, _ in leaves])
        cz = np.array([(b[4] + b[5]) / 2 for b, _ in leaves])
        dx = np.array([b[1] - b[0] for b, _ in leaves])
        dy = np.array([b[3] - b[2] for b, _ in leaves])
        dz = np.array([b[5] - b[4] for b, _ in leaves])
        ppc_f = np.array([n for _, n in leaves], np.int32)
        C, F = [[], [], [], []], [[], [], [], []]
        for c in range(len(leaves)):
            xl, xh = cx[c] - dx[c] / 2, cx[c] + dx[c] / 2
            yl, yh = cy[c] - dy[c] / 2, cy[c] + dy[c] / 2
            zl, zh = cz[c] - dz[c] / 2, cz[c] + dz[c] / 2
            pc = mb.coarseQuadraturePointsSingleCell(xl, xh, yl, yh, zl, zh, order)
            if ppc_f[c] == (order + 1) ** 3:
                pf = tuple(np.copy(a) for a in pc)
            else:
                pf = mb.fineQuadraturePointsSingleCell(xl, xh, yl, yh, zl, zh, order, int(ppc_f[c]))
            for a, v in zip(C, pc):
                a.append(v)
            for a, v in zip(F, pf):
                a.append(v)
        C = [np.concatenate(a) for a in C]
        F = [np.concatenate(a) for a in F]
        ends = np.linspace(np.pi, 0, order + 2)
        out.update({f"{tag}_params": np.array([XL, side, order, h, H, r, level]),
                    f"{tag}_atoms": np.array(atoms, np.float64), f"{tag}_base": np.asarray(cells, np.float64),
                    f"{tag}_u": np.cos((ends[1:] + ends[:-1]) / 2), f"{tag}_W": uw,
                    f"{tag}_cx": cx, f"{tag}_cy": cy, f"{tag}_cz": cz, f"{tag}_dx": dx, f"{tag}_dy": dy,
                    f"{tag}_dz": dz, f"{tag}_ppc_f": ppc_f})
        # The meshes themselves as SHA-256 digests of their float64 bytes,
        # plus every 97th point, to keep the file small.
        for name, arr in zip(("x", "y", "z", "w", "xf", "yf", "zf", "wf"), C + F):
            out[f"{tag}_{name}_sha256"] = np.frombuffer(
                __import__("hashlib").sha256(np.ascontiguousarray(arr, np.float64).tobytes()).digest(),
                np.uint8)
            out[f"{tag}_{name}_every97"] = arr[::97]
            out[f"{tag}_{name}_len"] = np.array(len(arr))
    np.savez_compressed(os.path.join(HERE, "mesh_build_reference.npz"), **out)


if __name__ == "__main__":
    O.build(ref=True)
    if not O.ref_available():
        sys.exit("oracle/_ref is missing: the reference tree must be present")
    mu = reference_mesh_utilities()
    mgs_golden()
    interp_golden(mu)
    mesh_golden(mu)
    mesh_build_golden()
    print("golden vectors written to", HERE)
