"""Seeded synthetic meshes and charge vectors for the treecode workloads.

The reference builds its real-space mesh from cells of first-kind Chebyshev
quadrature points.  This module restates that construction so the treecode
has inputs of the same shape and structure; the refinement rule and the
charge densities are project-defined stand-ins for the reference's atomic
data (which is not available), all seeded.

Restated from the reference:
  * first-kind Chebyshev points    meshUtilities.py:874-883
  * first-kind (Fejer-1) weights   meshUtilities.py:839-872
  * per-cell point order i,j,k (x-major) and weights scaled by cell size
                                   mpiMeshBuilding.py:725-756
"""
from dataclasses import dataclass, field

import numpy as np


def cheb1_points(lo, hi, n):
    """n+1 open Chebyshev points on [lo, hi], ascending (meshUtilities.py:874-883)."""
    ends = np.linspace(np.pi, 0.0, n + 2)
    theta = 0.5 * (ends[1:] + ends[:-1])
    return lo + 0.5 * (hi - lo) * (np.cos(theta) + 1.0)


def cheb1_weights_unscaled(n):
    """Quadrature weights on [-1, 1] for cheb1_points (meshUtilities.py:839-857)."""
    i = np.arange(n + 1)[:, None]
    j = np.arange(n + 1)[None, :]
    lam = 2.0 / (n + 1) * np.cos(i * (j + 0.5) * np.pi / (n + 1))
    W = np.zeros(n + 1)
    W[0] = 1.0
    for k in range(2, n + 1, 2):
        W[k] = 2.0 / (1.0 - k * k)
    return lam.T @ W


@dataclass
class Mesh:
    """Flat SoA mesh: points in cell order, cell after cell (like the reference)."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    w: np.ndarray
    order: int
    cell_lo: np.ndarray          # (ncells, 3)
    cell_hi: np.ndarray          # (ncells, 3)
    nuclei: np.ndarray           # (natoms, 3)
    charges: np.ndarray          # (natoms,)
    meta: dict = field(default_factory=dict)

    @property
    def n(self):
        return len(self.x)

    @property
    def points_per_cell(self):
        return np.full(len(self.cell_lo), (self.order + 1) ** 3, dtype=np.int32)


def cell_points(lo, hi, order):
    """Points and weights of many cells at once; ordering per mpiMeshBuilding.py:739-752."""
    lo = np.atleast_2d(lo)
    hi = np.atleast_2d(hi)
    n1 = order + 1
    wref = cheb1_weights_unscaled(order)
    half = 0.5 * (hi - lo)
    # Nodes mapped as lo + (hi-lo)/2*(u+1), exactly as cheb1_points does.
    ends = np.linspace(np.pi, 0.0, order + 2)
    u = np.cos(0.5 * (ends[1:] + ends[:-1]))
    px = lo[:, 0:1] + half[:, 0:1] * (u[None, :] + 1.0)
    py = lo[:, 1:2] + half[:, 1:2] * (u[None, :] + 1.0)
    pz = lo[:, 2:3] + half[:, 2:3] * (u[None, :] + 1.0)
    wx = half[:, 0:1] * wref[None, :]
    wy = half[:, 1:2] * wref[None, :]
    wz = half[:, 2:3] * wref[None, :]
    m = len(lo)
    X = np.broadcast_to(px[:, :, None, None], (m, n1, n1, n1)).reshape(-1)
    Y = np.broadcast_to(py[:, None, :, None], (m, n1, n1, n1)).reshape(-1)
    Z = np.broadcast_to(pz[:, None, None, :], (m, n1, n1, n1)).reshape(-1)
    W = (wx[:, :, None, None] * wy[:, None, :, None] * wz[:, None, None, :]).reshape(-1)
    return (np.ascontiguousarray(X), np.ascontiguousarray(Y), np.ascontiguousarray(Z),
            np.ascontiguousarray(W))


def refine_cells(nuclei, half_width=20.0, max_depth=5, factor=4.0, min_depth=0):
    """Octree cells of [-L, L]^3: refine a cell while its center lies within
    ``factor`` cell widths of a nucleus, down to ``max_depth`` (project rule
    standing in for the reference's density-based divide criteria)."""
    nuclei = np.atleast_2d(np.asarray(nuclei, dtype=np.float64))
    centers = np.zeros((1, 3))
    width = np.array([2.0 * half_width])
    out_c, out_w = [], []
    offs = np.array([[i, j, k] for i in (-1, 1) for j in (-1, 1) for k in (-1, 1)], dtype=np.float64)
    for depth in range(max_depth + 1):
        d = np.sqrt(((centers[:, None, :] - nuclei[None, :, :]) ** 2).sum(-1)).min(axis=1)
        split = ((d < factor * width) | (depth < min_depth)) & (depth < max_depth)
        out_c.append(centers[~split])
        out_w.append(width[~split])
        c = centers[split]
        w = width[split]
        if len(c) == 0:
            break
        centers = (c[:, None, :] + 0.25 * w[:, None, None] * offs[None, :, :]).reshape(-1, 3)
        width = np.repeat(0.5 * w, 8)
    centers = np.concatenate(out_c)
    width = np.concatenate(out_w)
    lo = centers - 0.5 * width[:, None]
    hi = centers + 0.5 * width[:, None]
    return lo, hi


def adaptive_mesh(nuclei, charges, order, max_depth, factor, half_width=20.0, min_depth=0):
    lo, hi = refine_cells(nuclei, half_width, max_depth, factor, min_depth)
    x, y, z, w = cell_points(lo, hi, order)
    return Mesh(x, y, z, w, order, lo, hi, np.atleast_2d(np.asarray(nuclei, float)),
                np.asarray(charges, float),
                meta=dict(max_depth=max_depth, factor=factor, half_width=half_width))


def mesh_with_points(nuclei, charges, order, max_depth, target_points, half_width=20.0,
                     min_depth=0):
    """Pick the refinement factor (bisection) whose mesh is closest to ``target_points``."""
    lo_f, hi_f = 0.05, 64.0
    best = None
    for _ in range(40):
        f = np.sqrt(lo_f * hi_f)
        lo, hi = refine_cells(nuclei, half_width, max_depth, f, min_depth)
        npts = len(lo) * (order + 1) ** 3
        if best is None or abs(npts - target_points) < abs(best[1] - target_points):
            best = (f, npts)
        if npts < target_points:
            lo_f = f
        else:
            hi_f = f
        if hi_f / lo_f < 1.0005:
            break
    return adaptive_mesh(nuclei, charges, order, max_depth, best[0], half_width, min_depth)


# ---------------------------------------------------------------------------
# Workloads (seeded).  Each returns the mesh plus the charge vector(s).
# ---------------------------------------------------------------------------
def nuclear_potential(mesh, soft=0.01):
    V = np.zeros(mesh.n)
    for R, Z in zip(mesh.nuclei, mesh.charges):
        r2 = (mesh.x - R[0]) ** 2 + (mesh.y - R[1]) ** 2 + (mesh.z - R[2]) ** 2
        V -= Z / np.sqrt(r2 + soft)
    return V


def hydrogenic_orbital(mesh, center=(0.0, 0.0, 0.0)):
    r = np.sqrt((mesh.x - center[0]) ** 2 + (mesh.y - center[1]) ** 2 + (mesh.z - center[2]) ** 2)
    return np.exp(-r) / np.sqrt(np.pi)


def single_atom(factor=1.0, max_depth=5, order=5, Z=4.0):
    """One Z=4 nucleus at the origin in [-20,20]^3, 6^3-point cells, depth <= 5.
    f = V*psi with psi = exp(-r)/sqrt(pi), V = -Z/sqrt(r^2+0.01); rho = 2 psi^2.
    factor=4 is the literal refinement rule (~957k points); factor=1 gives the
    ~50k-point mesh the CPU-runnable case is sized for."""
    mesh = adaptive_mesh([[0.0, 0.0, 0.0]], [Z], order, max_depth, factor)
    psi = hydrogenic_orbital(mesh)
    V = nuclear_potential(mesh)
    f = V * psi
    rho = 2.0 * psi * psi
    return mesh, f, rho


def gaussian_density(mesh, rng, n_gauss=3, expo=(0.1, 10.0)):
    """rho = sum over nuclei of n_gauss normalized Gaussians carrying Z/n_gauss each."""
    rho = np.zeros(mesh.n)
    params = []
    for R, Z in zip(mesh.nuclei, mesh.charges):
        a = np.exp(rng.uniform(np.log(expo[0]), np.log(expo[1]), n_gauss))
        for ai in a:
            r2 = (mesh.x - R[0]) ** 2 + (mesh.y - R[1]) ** 2 + (mesh.z - R[2]) ** 2
            rho += (Z / n_gauss) * (ai / np.pi) ** 1.5 * np.exp(-ai * r2)
            params.append((R.copy(), Z / n_gauss, ai))
    return rho, params


def hartree_system(seed=2, target_points=1_500_000, order=7, max_depth=7, natoms=4, box=6.0):
    """Coulomb Hartree workload: natoms nuclei uniform in a box x box x box cube,
    Z from {1,6,8}, density = 3 normalized Gaussians per nucleus."""
    rng = np.random.default_rng(seed)
    nuclei = rng.uniform(-box / 2, box / 2, (natoms, 3))
    Z = rng.choice([1.0, 6.0, 8.0], natoms)
    mesh = mesh_with_points(nuclei, Z, order, max_depth, target_points)
    rho, params = gaussian_density(mesh, rng)
    mesh.meta.update(seed=seed, gaussians=params)
    return mesh, rho


def orbital_batch(mesh, n_orb, rng, k_range=(0.4, 3.0), expo=(0.1, 10.0), n_gauss=4):
    """n_orb orbitals psi_i = random signed sums of n_gauss Gaussians on the nuclei;
    charge vectors f_i = -2 V psi_i (Green-iteration source); k_i ~ U[k_range]."""
    V = nuclear_potential(mesh)
    F = np.empty((n_orb, mesh.n))
    for i in range(n_orb):
        psi = np.zeros(mesh.n)
        for _ in range(n_gauss):
            a = int(rng.integers(len(mesh.nuclei)))
            R = mesh.nuclei[a]
            e = np.exp(rng.uniform(np.log(expo[0]), np.log(expo[1])))
            s = rng.choice([-1.0, 1.0])
            r2 = (mesh.x - R[0]) ** 2 + (mesh.y - R[1]) ** 2 + (mesh.z - R[2]) ** 2
            psi += s * np.exp(-e * r2)
        F[i] = -2.0 * V * psi
    k = rng.uniform(k_range[0], k_range[1], n_orb)
    return F, k


def multi_orbital_system(seed=3, target_points=1_000_000, n_orb=32, order=7, max_depth=7):
    """Three nuclei (Z = 6, 7, 8), order-7 cells, n_orb orbitals with distinct k_i."""
    rng = np.random.default_rng(seed)
    nuclei = rng.uniform(-2.0, 2.0, (3, 3))
    mesh = mesh_with_points(nuclei, [6.0, 7.0, 8.0], order, max_depth, target_points)
    F, k = orbital_batch(mesh, n_orb, rng)
    mesh.meta.update(seed=seed)
    return mesh, F, k


UNEVEN_SIZES = (50_000, 120_000, 300_000, 600_000, 1_200_000, 2_500_000)
UNEVEN_ORBITALS = (4, 8, 8, 16, 32, 64)


def uneven_systems(seed=4, sizes=UNEVEN_SIZES, orbitals=UNEVEN_ORBITALS, max_depth=7):
    """Independent systems of different sizes: 1-8 nuclei, Z in {1,6,8}, order 5-7."""
    rng = np.random.default_rng(seed)
    out = []
    for npts, norb in zip(sizes, orbitals):
        natoms = int(rng.integers(1, 9))
        nuclei = rng.uniform(-3.0, 3.0, (natoms, 3))
        Z = rng.choice([1.0, 6.0, 8.0], natoms)
        order = int(rng.integers(5, 8))
        mesh = mesh_with_points(nuclei, Z, order, max_depth, npts)
        F, k = orbital_batch(mesh, norb, rng)
        out.append((mesh, F, k))
    return out


def ring_molecule():
    """Planar 12-atom ring: 6 Z=6 on a radius-2.6 hexagon, 6 Z=1 at radius 4.7."""
    ang = np.arange(6) * np.pi / 3.0
    C = np.stack([2.6 * np.cos(ang), 2.6 * np.sin(ang), np.zeros(6)], 1)
    H = np.stack([4.7 * np.cos(ang), 4.7 * np.sin(ang), np.zeros(6)], 1)
    return np.concatenate([C, H]), np.array([6.0] * 6 + [1.0] * 6)
