"""Two-level quadrature mesh built on the GPU (tagi_mesh_refine / tagi_mesh_points).

Host-side mirror of the reference's mesh setup for the
"coarsenedUniformTwoLevel" divide criterion on one rank
(3D-GreenIteration/src/utilities/mpiMeshBuilding.py:250-575,
buildMeshFromMinimumDepthCells):

  base cells        inializeBaseMesh_distributed (mpiMeshBuilding.py:68-124):
                    computed here on the host (a few hundred rows)
  refinement        refineCellReturnCells per base cell -> one device call
  load balancing    callZoltan (mpiMeshBuilding.py:464): not done; one GPU
                    holds every cell, in the order the refinement emits them
  points            the per-cell loop of mpiMeshBuilding.py:517-556 -> one
                    device call

Names follow the reference: X, Y, Z, W (coarse mesh), Xf, Yf, Zf, Wf (fine
mesh), PtsPerCellCoarse / PtsPerCellFine (int32 per cell).
"""
import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _native
from .device import _dev, _stream


def base_cells(XL, YL, ZL, max_side_length):
    """[n, 6] rows (xmin, xmax, ymin, ymax, zmin, zmax), x-major, as
    inializeBaseMesh_distributed builds them on one rank (mpiMeshBuilding.py:82-108)."""
    nx = int(-((-2 * XL) // max_side_length))
    ny = int(-((-2 * YL) // max_side_length))
    nz = int(-((-2 * ZL) // max_side_length))
    x = np.linspace(-XL, XL, nx + 1)
    y = np.linspace(-YL, YL, ny + 1)
    z = np.linspace(-ZL, ZL, nz + 1)
    X, Y, Z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = X.ravel(), Y.ravel(), Z.ravel()
    return np.ascontiguousarray(np.stack([x[i], x[i + 1], y[j], y[j + 1], z[k], z[k + 1]], axis=1))


def unit_tables(order):
    """(u, W): first-kind nodes cos(theta_i) on [-1, 1] and unscaled weights,
    evaluated by the same numpy expressions as meshUtilities.py:835-883."""
    ends = np.linspace(np.pi, 0, order + 2)
    u = np.cos((ends[1:] + ends[:-1]) / 2)
    N = order
    lam = np.ones((N + 1, N + 1))
    for i in range(N + 1):
        for j in range(N + 1):
            lam[i, j] = 2 / (N + 1) * np.cos(i * (j + 1 / 2) * np.pi / (N + 1))
    Wv = np.zeros(N + 1)
    for i in range(N + 1):
        if i == 0:
            Wv[i] = 1
        elif i % 2 == 0:
            Wv[i] = 2 / (1 - i ** 2)
    return np.ascontiguousarray(u), np.ascontiguousarray(np.dot(np.transpose(lam), Wv))


@dataclass
class DeviceMesh:
    """Cell table and meshes on the GPU (float64 / int32 tensors)."""
    order: int
    cellX: torch.Tensor
    cellY: torch.Tensor
    cellZ: torch.Tensor
    cellDX: torch.Tensor
    cellDY: torch.Tensor
    cellDZ: torch.Tensor
    PtsPerCellCoarse: torch.Tensor
    PtsPerCellFine: torch.Tensor
    X: torch.Tensor
    Y: torch.Tensor
    Z: torch.Tensor
    W: torch.Tensor
    Xf: torch.Tensor = None
    Yf: torch.Tensor = None
    Zf: torch.Tensor = None
    Wf: torch.Tensor = None

    @property
    def num_cells(self):
        return int(self.cellX.numel())

    @property
    def n(self):
        return int(self.X.numel())


def refine_cells(base, atoms, order, h, H, r, level, min_depth=0, max_depth=16, device="cuda",
                 stream=None):
    """Leaf cell table of the two-level rule (tagi_mesh_refine).  base: [n, 6]
    host or device rows; atoms: [natoms, 3].  Returns the six float64 cell
    arrays and the two int32 points-per-cell arrays, on the device."""
    L = _native.lib()
    base_d = torch.as_tensor(np.asarray(base, np.float64).reshape(-1, 6) if not torch.is_tensor(base) else base,
                             dtype=torch.float64, device=device).contiguous()
    atoms_d = torch.as_tensor(np.asarray(atoms, np.float64).reshape(-1, 3) if not torch.is_tensor(atoms) else atoms,
                              dtype=torch.float64, device=device).contiguous()
    nb, na = base_d.shape[0], atoms_d.shape[0]
    if stream is not None:
        stream.wait_stream(torch.cuda.current_stream())  # base_d / atoms_d were made there
    ncell, ncp, nfp = ctypes.c_int(0), ctypes.c_longlong(0), ctypes.c_longlong(0)
    args = (_dev(base_d, "base"), nb, _dev(atoms_d, "atoms") if na else ctypes.c_void_p(0), na, int(order),
            float(h), float(H), float(r), float(level), int(min_depth), int(max_depth))
    s = _stream(stream)
    null = [ctypes.c_void_p(0)] * 8
    _native.check(L.tagi_mesh_refine(*args, *null, 0, ctypes.byref(ncell), ctypes.byref(ncp), ctypes.byref(nfp), s))
    n = ncell.value
    f64 = dict(dtype=torch.float64, device=device)
    cells = [torch.empty(n, **f64) for _ in range(6)]
    ppc_c = torch.empty(n, dtype=torch.int32, device=device)
    ppc_f = torch.empty(n, dtype=torch.int32, device=device)
    outs = [_dev(c, "cell") for c in cells] + [_dev(ppc_c, "ppc_c", torch.int32), _dev(ppc_f, "ppc_f", torch.int32)]
    _native.check(L.tagi_mesh_refine(*args, *outs, n, ctypes.byref(ncell), ctypes.byref(ncp), ctypes.byref(nfp), s))
    return cells, ppc_c, ppc_f, int(nfp.value)


def mesh_points(cells, ppc_f, order, num_fine=None, tables=None, device="cuda", stream=None):
    """Coarse (and, with num_fine, fine) points of a cell table (tagi_mesh_points).
    tables: (u, W) 1-D tables; default unit_tables(order)."""
    u, Wt = unit_tables(order) if tables is None else (np.ascontiguousarray(tables[0], np.float64),
                                                       np.ascontiguousarray(tables[1], np.float64))
    if len(u) != order + 1 or len(Wt) != order + 1:
        raise ValueError("tables need order+1 entries each")
    n = int(cells[0].numel())
    p3 = (order + 1) ** 3
    f64 = dict(dtype=torch.float64, device=device)
    C = [torch.empty(n * p3, **f64) for _ in range(4)]
    F = [torch.empty(int(num_fine), **f64) for _ in range(4)] if num_fine is not None else None
    dp = ctypes.POINTER(ctypes.c_double)
    if stream is not None:
        stream.wait_stream(torch.cuda.current_stream())  # output buffers were made there
    cargs = [_dev(c, "cell") for c in cells]
    fine_args = [_dev(a, "fine") for a in F] if F is not None else [ctypes.c_void_p(0)] * 4
    _native.check(_native.lib().tagi_mesh_points(
        *cargs, _dev(ppc_f, "ppc_f", torch.int32) if F is not None else ctypes.c_void_p(0), n, int(order),
        u.ctypes.data_as(dp), Wt.ctypes.data_as(dp), *[_dev(a, "coarse") for a in C], n * p3, *fine_args,
        int(num_fine) if num_fine is not None else 0, _stream(stream)))
    return C, F


def build_mesh(XL, max_side_length, atoms, order, h, H, r, level, min_depth=0, max_depth=16, fine=True,
               YL=None, ZL=None, tables=None, device="cuda", stream=None):
    """Whole mesh on the GPU: base cells of [-XL, XL] x [-YL, YL] x [-ZL, ZL],
    refinement, coarse and (fine=True) two-level fine points."""
    base = base_cells(XL, XL if YL is None else YL, XL if ZL is None else ZL, max_side_length)
    cells, ppc_c, ppc_f, nfine = refine_cells(base, atoms, order, h, H, r, level, min_depth, max_depth,
                                              device, stream)
    C, F = mesh_points(cells, ppc_f, order, nfine if fine else None, tables, device, stream)
    F = F if F is not None else [None] * 4
    return DeviceMesh(order, *cells, ppc_c, ppc_f, *C, *F)
