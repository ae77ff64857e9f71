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


def test_exact_symbol_with_the_reference_binding(BT, native, oracle, small_mesh):
    """A TAGI user points ctypes at this library and binds BaryTreeInterface
    with the reference's own argtypes tuple (BaryTreeInterface.py:67-72: enum
    classes for kernel, singularity, approximation and compute type), then
    calls it the way callTreedriver does (:130-145).  The library default is
    FP64, so the result equals the oracle's FP64 treecode to 1e-12."""
    import ctypes

    mesh, f, rho = small_mesh
    lib = ctypes.CDLL(native.LIB_PATH)
    dp = ctypes.POINTER(ctypes.c_double)
    fn = lib.BaryTreeInterface
    fn.argtypes = (ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, BT.Kernel, ctypes.c_int, dp,
                   BT.Singularity, BT.Approximation, BT.ComputeType, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                   ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int)
    arrays = [np.copy(a) for a in (mesh.x, mesh.y, mesh.z, f, mesh.x, mesh.y, mesh.z, f, mesh.w)]
    kp = np.array([1.0])
    result = np.zeros(mesh.n)
    P = lambda a: a.ctypes.data_as(dp)
    fn(ctypes.c_int(mesh.n), ctypes.c_int(mesh.n), *[P(a) for a in arrays], P(result), BT.Kernel.YUKAWA,
       ctypes.c_int(1), P(kp), BT.Singularity.SUBTRACTION, BT.Approximation.LAGRANGE,
       BT.ComputeType.PARTICLE_CLUSTER, ctypes.c_double(0.7), ctypes.c_int(7), ctypes.c_int(300),
       ctypes.c_int(300), ctypes.c_double(1.0), ctypes.c_double(-1), ctypes.c_int(0))
    c = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, 7, 300, 300, 1.0)
    ref = c.convolve(f, f, mesh.w, BT.Kernel.YUKAWA, [1.0], BT.Singularity.SUBTRACTION)
    assert rel_l2(result, ref) <= 1e-12
    # the enum-typed parameters refuse plain integers, as the reference binding does
    with pytest.raises(ctypes.ArgumentError):
        fn(mesh.n, mesh.n, *[P(a) for a in arrays], P(result), 2, 1, P(kp), 2, 1, 1, 0.7, 7, 300, 300, 1.0, -1.0, 0)


def test_two_kernel_parameters_k_and_epsilon(BT, small_mesh):
    """The regularize=True call form (greenIterationFixedPoint.py:223-227,
    scfFixedPoint.py:246-250) passes Kernel.YUKAWA with
    numberOfKernelParameters=2 and [k, epsilon].  The YUKAWA and COULOMB
    kernels read the first parameter only, so that call gives exactly the
    one-parameter result (the reference itself warns when epsilon != 0)."""
    mesh, f, rho = small_mesh
    common = dict(theta=0.7, degree=7, sourceLeafSize=300, targetLeafSize=300)

    def call(nkp, kp):
        return BT.callTreedriver(mesh.n, mesh.n, np.copy(mesh.x), np.copy(mesh.y), np.copy(mesh.z), np.copy(f),
                                 np.copy(mesh.x), np.copy(mesh.y), np.copy(mesh.z), np.copy(f), np.copy(mesh.w),
                                 BT.Kernel.YUKAWA, nkp, kp, BT.Singularity.SUBTRACTION, BT.Approximation.LAGRANGE,
                                 BT.ComputeType.PARTICLE_CLUSTER, True, 0, **common)

    one = call(1, np.array([1.3]))
    two = call(2, np.array([1.3, 0.0]))
    assert np.array_equal(one, two)
    assert np.array_equal(one, call(2, np.array([1.3, 0.25])))
