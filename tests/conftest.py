import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = "treecode-accelerated-green-iteration_gb300"
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module(PKG)


@pytest.fixture(scope="session")
def native(pkg):
    """The built C-ABI library (built here if missing; nvcc cross-compiles)."""
    nat = importlib.import_module(PKG + "._native")
    if not os.path.exists(nat.LIB_PATH):
        importlib.import_module(PKG + ".build").build()
    return nat


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def dev(native):
    return importlib.import_module(PKG + ".device")


@pytest.fixture(scope="session")
def BT(pkg):
    return pkg.BaryTreeInterface


@pytest.fixture(scope="session")
def syn(pkg):
    return pkg.synthetic


@pytest.fixture(scope="session")
def small_mesh(syn):
    """Single Z=4 atom, coarse refinement: 25,920 Chebyshev points (120 cells)."""
    mesh, f, rho = syn.single_atom(factor=1.0, max_depth=3)
    return mesh, f, rho


def point_sets():
    """Seeded point clouds that exercise the tree rules."""
    rng = np.random.default_rng(7)
    sets = {}
    sets["uniform"] = rng.uniform(-1, 1, (3000, 3))
    blobs = np.concatenate([rng.normal(c, s, (700, 3)) for c, s in
                            (((0, 0, 0), 0.05), ((1, 0.5, 0), 0.3), ((-2, 1, 1), 0.01))])
    sets["blobs"] = blobs
    d = rng.uniform(-1, 1, (500, 3))
    sets["duplicates"] = np.concatenate([d, d, d[:100]])
    plane = rng.uniform(-1, 1, (2000, 3))
    plane[:, 2] = 0.25
    sets["plane"] = plane
    sets["line"] = np.stack([np.linspace(0, 1, 1500), np.zeros(1500), np.zeros(1500)], 1)
    sets["tiny"] = rng.uniform(0, 1, (7, 3))
    sets["single"] = np.array([[0.3, -0.2, 0.1]])
    return sets


def to_cuda(*arrs):
    import torch
    return [torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda") for a in arrs]


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(np.asarray(b)), 1e-300))
