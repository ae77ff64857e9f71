"""CPU restatement of the reference's mesh construction for the
``coarsenedUniformTwoLevel`` divide criterion (TEST INFRASTRUCTURE ONLY:
imported by tests/ as the checker of the device mesh builder; never by the
product path).

Pinned against tests/golden/mesh_build_reference.npz, which
tests/golden/make_golden.py makes by calling the reference's own rule method
and point functions.  Follows, in 3D-GreenIteration/src:
  base cells        utilities/mpiMeshBuilding.py:68-124 (inializeBaseMesh_distributed,
                    one rank: every cell, x-major)
  recursion         dataStructures/TreeStruct_CC.py:1049-1140 (recursiveDivide:
                    level < minDepth divides; children split at the midpoints,
                    CellStruct_CC.py:3060-3100, visited (i, j, k) x-major)
  leaf order        TreeStruct_CC.py:2387 walks masterList, kept sorted by
                    uniqueID (CellStruct_CC.py:220-221, digits i+1, j+1, k+1):
                    depth-first, children x-major; base cells in order
  divide rule       dataStructures/CellStruct_CC.py:2344-2491
                    (refineCoarseningUniform_TwoLevel)
  cell centre/width TreeStruct_CC.py:2392-2398 (extractCellXYZ)
  coarse points     utilities/mpiMeshBuilding.py:725-752
  fine points       utilities/mpiMeshBuilding.py:755-840
  1-D nodes/weights utilities/meshUtilities.py:835-883

Squares are written ``d * d``; the reference's scalar ``d**2`` is the same
correctly rounded product.  ``max_depth`` is this restatement's guard (the
reference has none): a cell at that depth that the rule would divide raises.
"""
import math

import numpy as np


def base_cells(XL, YL, ZL, max_side):
    """[n, 6] rows (xmin, xmax, ymin, ymax, zmin, zmax) (mpiMeshBuilding.py:82-108)."""
    nx = int(-((-2 * XL) // max_side))
    ny = int(-((-2 * YL) // max_side))
    nz = int(-((-2 * ZL) // max_side))
    x = np.linspace(-XL, XL, nx + 1)
    y = np.linspace(-YL, YL, ny + 1)
    z = np.linspace(-ZL, ZL, nz + 1)
    rows = []
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                rows.append([x[i], x[i + 1], y[j], y[j + 1], z[k], z[k + 1]])
    return np.array(rows, dtype=np.float64).reshape(-1, 6)


def unit_nodes(order):
    """u_i = cos(theta_i) of meshUtilities.py:878-881 (x = lo + (hi-lo)/2 (u+1))."""
    ends = np.linspace(np.pi, 0, order + 2)
    theta = (ends[1:] + ends[:-1]) / 2
    return np.cos(theta)


def unit_weights(order):
    """meshUtilities.py:835-853 (unscaledWeightsFirstKind)."""
    N = order
    lam = np.ones((N + 1, N + 1))
    for i in range(N + 1):
        for j in range(N + 1):
            lam[i, j] = 2 / (N + 1) * np.cos(i * (j + 1 / 2) * np.pi / (N + 1))
    W = np.zeros(N + 1)
    for i in range(N + 1):
        if i == 0:
            W[i] = 1
        elif i % 2 == 0:
            W[i] = 2 / (1 - i ** 2)
    return np.dot(np.transpose(lam), W)


def divide_rule(b, atoms, h, H, r, level):
    """(divide, fine_children) of one cell with bounds b (CellStruct_CC.py:2344-2439)."""
    xmin, xmax, ymin, ymax, zmin, zmax = (float(v) for v in b)
    dist = 10 + H
    for ax, ay, az in atoms:
        if ax < xmax and ay < ymax and az < zmax and ax > xmin and ay > ymin and az > zmin:
            dist = 0.0
        else:
            for x in (xmax, xmin):
                for y in (ymin, ymax):
                    for z in (zmin, zmax):
                        dx, dy, dz = x - ax, y - ay, z - az
                        d = math.sqrt(dx * dx + dy * dy + dz * dz)
                        dist = min(dist, d)
    side = max(zmax - zmin, xmax - xmin, ymax - ymin)
    divide = False
    if side > H:
        divide = True
    elif level >= 2 and dist < r / 4:
        divide = side > h / 4
    elif level >= 1 and dist < r / 2:
        divide = side > h / 2
    elif dist < r:
        divide = side > h
    elif dist < r + 2 * h * 1.0:
        divide = side > 2 * h
    elif dist < r + (2 * h + 4 * h) * 1.0:
        divide = side > 4 * h
    elif dist < r + (2 * h + 4 * h + 8 * h) * 1.0:
        divide = side > 8 * h
    fine = 1
    if not divide and level < -1 and dist < r * 1.5:
        m = -int(level)
        fine = m * m * m
    return divide, fine


def refine(base, atoms, h, H, r, level, min_depth=0, max_depth=16):
    """Leaves depth-first: list of (bounds[6], fine_children)."""
    atoms = [tuple(float(v) for v in a) for a in np.asarray(atoms, dtype=np.float64).reshape(-1, 3)]
    out = []

    def visit(b, depth):
        if depth < min_depth:
            divide, fine = True, 1
        else:
            divide, fine = divide_rule(b, atoms, h, H, r, level)
        if not divide:
            out.append((b, fine))
            return
        if depth >= max_depth:
            raise ValueError("refinement below max_depth %d" % max_depth)
        xb = [b[0], (b[1] + b[0]) / 2, b[1]]
        yb = [b[2], (b[3] + b[2]) / 2, b[3]]
        zb = [b[4], (b[5] + b[4]) / 2, b[5]]
        for i in range(2):
            for j in range(2):
                for k in range(2):
                    visit((xb[i], xb[i + 1], yb[j], yb[j + 1], zb[k], zb[k + 1]), depth + 1)

    for row in np.asarray(base, dtype=np.float64).reshape(-1, 6):
        visit(tuple(float(v) for v in row), 0)
    return out


def cell_table(leaves, order):
    """Centre, width and points per cell as extractCellXYZ returns them."""
    p3 = (order + 1) ** 3
    b = np.array([l[0] for l in leaves], dtype=np.float64).reshape(-1, 6)
    fine = np.array([l[1] for l in leaves], dtype=np.int64)
    return dict(cx=(b[:, 0] + b[:, 1]) / 2, cy=(b[:, 2] + b[:, 3]) / 2, cz=(b[:, 4] + b[:, 5]) / 2,
                dx=b[:, 1] - b[:, 0], dy=b[:, 3] - b[:, 2], dz=b[:, 5] - b[:, 4],
                ppc_c=np.full(len(b), p3, np.int32), ppc_f=(fine * p3).astype(np.int32))


def _cell_points(xl, xh, yl, yh, zl, zh, u, W):
    """coarseQuadraturePointsSingleCell with the 1-D tables u, W."""
    hx, hy, hz = (xh - xl) / 2, (yh - yl) / 2, (zh - zl) / 2
    xv, yv, zv = xl + hx * (u + 1), yl + hy * (u + 1), zl + hz * (u + 1)
    xw, yw, zw = hx * W, hy * W, hz * W
    n1 = len(u)
    X = np.broadcast_to(xv[:, None, None], (n1, n1, n1)).ravel()
    Y = np.broadcast_to(yv[None, :, None], (n1, n1, n1)).ravel()
    Z = np.broadcast_to(zv[None, None, :], (n1, n1, n1)).ravel()
    Wt = np.outer(np.outer(xw, yw), zw).ravel()
    return X, Y, Z, Wt


def _child_bounds(lo, hi, m):
    """mpiMeshBuilding.py:766-800."""
    if m == 1:
        return [lo, hi]
    if m == 2:
        return [lo, (lo + hi) / 2, hi]
    if m == 3:
        return [lo, (2 * lo + hi) / 3, (2 * hi + lo) / 3, hi]
    if m == 4:
        return [lo, (3 * lo + hi) / 4, (lo + hi) / 2, (3 * hi + lo) / 4, hi]
    raise ValueError("fine children per side must be 1..4")


def points(table, order, u=None, W=None, fine=True):
    """Coarse (and fine) meshes of the cell table: (x, y, z, w[, xf, yf, zf, wf])."""
    u = unit_nodes(order) if u is None else np.asarray(u, np.float64)
    W = unit_weights(order) if W is None else np.asarray(W, np.float64)
    p3 = (order + 1) ** 3
    C = [[], [], [], []]
    F = [[], [], [], []]
    for c in range(len(table["cx"])):
        xl = table["cx"][c] - table["dx"][c] / 2
        xh = table["cx"][c] + table["dx"][c] / 2
        yl = table["cy"][c] - table["dy"][c] / 2
        yh = table["cy"][c] + table["dy"][c] / 2
        zl = table["cz"][c] - table["dz"][c] / 2
        zh = table["cz"][c] + table["dz"][c] / 2
        pts = _cell_points(xl, xh, yl, yh, zl, zh, u, W)
        for a, v in zip(C, pts):
            a.append(v)
        if not fine:
            continue
        nch = int(table["ppc_f"][c]) // p3
        m = round(nch ** (1.0 / 3.0))
        if m * m * m != nch:
            raise ValueError("fine children must be 1, 8, 27 or 64")
        xb, yb, zb = _child_bounds(xl, xh, m), _child_bounds(yl, yh, m), _child_bounds(zl, zh, m)
        for ii in range(m):
            for jj in range(m):
                for kk in range(m):
                    q = _cell_points(xb[ii], xb[ii + 1], yb[jj], yb[jj + 1], zb[kk], zb[kk + 1], u, W)
                    for a, v in zip(F, q):
                        a.append(v)
    out = [np.concatenate(a) if a else np.zeros(0) for a in C]
    if fine:
        out += [np.concatenate(a) if a else np.zeros(0) for a in F]
    return tuple(out)


def build(XL, max_side, atoms, order, h, H, r, level, min_depth=0, max_depth=16, fine=True):
    """Whole mesh of a cubic domain [-XL, XL]^3: (table, points)."""
    base = base_cells(XL, XL, XL, max_side)
    leaves = refine(base, atoms, h, H, r, level, min_depth, max_depth)
    table = cell_table(leaves, order)
    return table, points(table, order, fine=fine)
