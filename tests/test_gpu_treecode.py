"""Subsystems (b)-(d) on the GPU against the CPU oracle.

Tolerances (relative L2 over all targets):
  FP64 mode vs FP64 oracle treecode with identical lists   <= 1e-12
  mixed mode vs FP64 oracle treecode                       <= 1e-6
  treecode vs FP64 direct sum: the approximation error, stated per case.
"""
import numpy as np
import pytest

from conftest import rel_l2, to_cuda

pytestmark = pytest.mark.gpu

CASES = [  # kernel, param, singularity
    ("YUKAWA", 1.0, "SUBTRACTION"),
    ("YUKAWA", 2.3, "SKIPPING"),
    ("COULOMB", 1.0, "SUBTRACTION"),
    ("COULOMB", 0.0, "SKIPPING"),
]


@pytest.fixture(scope="module")
def mesh_plan(dev, oracle, small_mesh):
    mesh, f, rho = small_mesh
    g = dev.TreecodePlan.for_mesh(*to_cuda(mesh.x, mesh.y, mesh.z, mesh.w), theta=0.7, degree=7,
                                  source_leaf=300, target_leaf=300)
    c = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, 7, 300, 300, 1.0)
    assert g.info()["far_entries"] > 0
    return mesh, f, rho, g, c


@pytest.mark.parametrize("kname,kp,sname", CASES)
def test_fp64_and_mixed_match_oracle(BT, mesh_plan, kname, kp, sname):
    mesh, f, rho, g, c = mesh_plan
    kern, sing = BT.Kernel[kname], BT.Singularity[sname]
    q = f if kname == "YUKAWA" else rho
    ref = c.convolve(q, q, mesh.w, kern, [kp], sing)
    (qt,) = to_cuda(q)
    out64 = g.convolve(qt, qt, kern, [kp], sing, precision="fp64").cpu().numpy()
    assert rel_l2(out64, ref) <= 1e-12
    out32 = g.convolve(qt, qt, kern, [kp], sing, precision="mixed").cpu().numpy()
    assert rel_l2(out32, ref) <= 1e-6


def test_weight_and_modified_charges(BT, mesh_plan):
    mesh, f, rho, g, c = mesh_plan
    assert rel_l2(g.charges(0), c.weight_charges()) <= 1e-13
    (ft,) = to_cuda(f)
    g.convolve(ft, ft, BT.Kernel.YUKAWA, [1.0], BT.Singularity.SUBTRACTION, precision="fp64")
    assert rel_l2(g.charges(1)[0], c.modified_charges(f, mesh.w)) <= 1e-13
    g.convolve(ft, ft, BT.Kernel.YUKAWA, [1.0], BT.Singularity.SUBTRACTION, precision="mixed")
    assert rel_l2(g.charges(2)[0], c.modified_charges(f, mesh.w)) <= 1e-6


def test_treecode_error_against_direct_sum(BT, oracle, mesh_plan):
    mesh, f, rho, g, c = mesh_plan
    sub = np.arange(0, mesh.n, 7)
    (ft,) = to_cuda(f)
    out = g.convolve(ft, ft, BT.Kernel.YUKAWA, [1.0], BT.Singularity.SUBTRACTION,
                     precision="mixed").cpu().numpy()
    d = oracle.direct(mesh.x, mesh.y, mesh.z, f, mesh.x, mesh.y, mesh.z, f, mesh.w, 2, [1.0], 2,
                      subset=sub)
    assert rel_l2(out[sub], d) <= 1e-6


def test_batched_orbitals_equal_single_calls(BT, dev, mesh_plan):
    """FP64: a batch of orbitals gives exactly the single-orbital results.
    Mixed: batches of >= 4 Yukawa orbitals run the orbital-group kernels
    (shared pair geometry, per-orbital exponent), so they agree with the
    single-orbital kernels to the mixed-precision tolerance."""
    mesh, f, rho, g, c = mesh_plan
    rng = np.random.default_rng(5)
    F = np.stack([f * rng.uniform(0.5, 2) + rng.normal(0, 0.01, mesh.n) for _ in range(5)])
    ks = rng.uniform(0.4, 3.0, 5)
    (Ft,) = to_cuda(F)
    for prec in ("fp64", "mixed"):
        batch = g.convolve(Ft, Ft, BT.Kernel.YUKAWA, ks, BT.Singularity.SUBTRACTION,
                           precision=prec).cpu().numpy()
        for i in range(5):
            one = g.convolve(Ft[i].contiguous(), Ft[i].contiguous(), BT.Kernel.YUKAWA, [ks[i]],
                             BT.Singularity.SUBTRACTION, precision=prec).cpu().numpy()
            if prec == "fp64":
                assert np.array_equal(batch[i], one), i
            else:
                assert rel_l2(batch[i], one) <= 1e-6, i
    ref = c.convolve(F[3], F[3], mesh.w, BT.Kernel.YUKAWA, [ks[3]], BT.Singularity.SUBTRACTION)
    assert rel_l2(batch[3], ref) <= 1e-6


@pytest.mark.parametrize("sname", ["SUBTRACTION", "SKIPPING"])
def test_orbital_groups_of_eight_match_oracle(BT, mesh_plan, sname):
    """Nine orbitals: one full group of 8 and a partial group of 1."""
    mesh, f, rho, g, c = mesh_plan
    rng = np.random.default_rng(8)
    F = np.stack([f * rng.uniform(-2, 2) + rng.normal(0, 0.05, mesh.n) * np.abs(f) for _ in range(9)])
    ks = rng.uniform(0.4, 3.0, 9)
    (Ft,) = to_cuda(F)
    sing = BT.Singularity[sname]
    out = g.convolve(Ft, Ft, BT.Kernel.YUKAWA, ks, sing, precision="mixed").cpu().numpy()
    for i in (0, 5, 8):
        ref = c.convolve(F[i], F[i], mesh.w, BT.Kernel.YUKAWA, [ks[i]], sing)
        assert rel_l2(out[i], ref) <= 1e-6, i


def test_call_treedriver_dropin(BT, oracle, small_mesh):
    mesh, f, rho = small_mesh
    kp = np.array([1.0])
    out = BT.callTreedriver(mesh.n, mesh.n, np.copy(mesh.x), np.copy(mesh.y), np.copy(mesh.z),
                            np.copy(f), np.copy(mesh.x), np.copy(mesh.y), np.copy(mesh.z), np.copy(f),
                            np.copy(mesh.w), BT.Kernel.YUKAWA, 1, kp, BT.Singularity.SUBTRACTION,
                            BT.Approximation.LAGRANGE, BT.ComputeType.PARTICLE_CLUSTER, True, 0,
                            theta=0.7, degree=7, sourceLeafSize=300, targetLeafSize=300, sizeCheck=1.0)
    c = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, 7, 300, 300, 1.0)
    ref = c.convolve(f, f, mesh.w, 2, [1.0], 2)
    assert out.dtype == np.float64 and out.shape == (mesh.n,)
    assert rel_l2(out, ref) <= 1e-12
    mixed = BT.callTreedriver(mesh.n, mesh.n, mesh.x, mesh.y, mesh.z, f, mesh.x, mesh.y, mesh.z, f,
                              mesh.w, BT.Kernel.YUKAWA, 1, kp, BT.Singularity.SUBTRACTION,
                              BT.Approximation.LAGRANGE, BT.ComputeType.PARTICLE_CLUSTER, True, 0,
                              theta=0.7, degree=7, sourceLeafSize=300, targetLeafSize=300,
                              precision="mixed")
    assert rel_l2(mixed, ref) <= 1e-6
