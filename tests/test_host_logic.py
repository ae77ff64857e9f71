"""Host-side logic of the reference-facing Python modules (no GPU)."""
import importlib
import os
import sys

import numpy as np
import pytest

from conftest import PKG, ROOT


def test_enum_values_match_reference(BT):
    # BaryTreeInterface.py:20-46
    assert [int(k) for k in BT.Kernel] == list(range(10))
    assert (BT.Kernel.COULOMB, BT.Kernel.YUKAWA) == (1, 2)
    assert (BT.Singularity.SKIPPING, BT.Singularity.SUBTRACTION) == (1, 2)
    assert (BT.Approximation.LAGRANGE, BT.Approximation.HERMITE) == (1, 2)
    assert (BT.ComputeType.PARTICLE_CLUSTER, BT.ComputeType.CLUSTER_CLUSTER) == (1, 3)
    with pytest.raises(TypeError):
        BT.Kernel.from_param(2)


def _args(BT, n=3):
    a = np.zeros(n)
    return [n, n, a, a, a, a, a, a, a, a, a, BT.Kernel.YUKAWA, 1, np.array([1.0]),
            BT.Singularity.SUBTRACTION, BT.Approximation.LAGRANGE, BT.ComputeType.PARTICLE_CLUSTER]


def test_missing_tree_parameters_assert_like_reference(BT):
    # BaryTreeInterface.py:106-112
    with pytest.raises(AssertionError, match="theta"):
        BT.callTreedriver(*_args(BT), True, 0, degree=7, sourceLeafSize=1, targetLeafSize=1)
    with pytest.raises(AssertionError, match="degree"):
        BT.callTreedriver(*_args(BT), True, 0, theta=0.7, sourceLeafSize=1, targetLeafSize=1)
    with pytest.raises(AssertionError, match="sourceLeafSize"):
        BT.callTreedriver(*_args(BT), True, 0, theta=0.7, degree=7, targetLeafSize=1)


def test_bad_gpupresent_exits_like_reference(BT, capsys):
    # BaryTreeInterface.py:153-155
    with pytest.raises(SystemExit):
        BT.callTreedriver(*_args(BT), "yes", 0, theta=0.7, degree=7, sourceLeafSize=1,
                          targetLeafSize=1)
    assert "GPUpresent" in capsys.readouterr().out


def test_non_float64_inputs_rejected(BT):
    args = _args(BT)
    args[2] = np.zeros(3, np.float32)
    with pytest.raises(TypeError):
        BT.callTreedriver(*args, True, 0, theta=0.7, degree=7, sourceLeafSize=1, targetLeafSize=1)


def test_modules_import_top_level_like_tagi():
    """TAGI does `import BaryTreeInterface as BT` with the utilities dir on sys.path."""
    d = os.path.join(ROOT, PKG)
    sys.path.insert(0, d)
    try:
        for name in ("BaryTreeInterface", "orthogonalization_wrapper", "interpolation_wrapper"):
            m = importlib.import_module(name)
            assert m.__file__.startswith(d)
    finally:
        sys.path.remove(d)


def test_synthetic_mesh_quadrature(syn):
    mesh, f, rho = syn.single_atom(factor=1.0, max_depth=5)
    assert mesh.n == 50112                       # 232 cells of 6^3 points
    assert abs(mesh.w.sum() - 40.0 ** 3) < 1e-8  # weights integrate the domain volume
    assert abs(np.sum(rho * mesh.w) - 2.0) < 1e-3
    lo, hi = syn.refine_cells([[0, 0, 0]], 20.0, 5, 4.0)
    assert len(lo) * 216 == 957312               # the literal refinement rule


def test_hartree_system_shape(syn):
    """The Coulomb Hartree workload: ~1.5M points, order-7 cells, density
    integrating to the nuclear charge (the mesh resolves the Gaussians)."""
    mesh, rho = syn.hartree_system()
    assert abs(mesh.n - 1_500_000) < 20_000 and mesh.order == 7 and len(mesh.nuclei) == 4
    ztot = mesh.charges.sum()
    assert abs(np.sum(rho * mesh.w) - ztot) / ztot < 1e-6
