"""Generate the golden vectors in this directory from the REFERENCE itself.

Run here, where the reference tree is mounted (it is not on the GPU machine):
    python tests/golden/make_golden.py
It needs oracle/_ref (``make -C oracle ref``: the reference's own
Orthogonalization.c and TwoMeshInterpolation.c compiled from their sources)
and imports the reference's Python meshUtilities.py for the Chebyshev
first-kind points and weights.  Outputs (small .npz files) are committed.
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_UTIL = "/root/reference/3D-GreenIteration/src/utilities"
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


if __name__ == "__main__":
    O.build(ref=True)
    if not O.ref_available():
        sys.exit("oracle/_ref is missing: the reference tree must be present")
    mu = reference_mesh_utilities()
    mgs_golden()
    interp_golden(mu)
    mesh_golden(mu)
    print("golden vectors written to", HERE)
