"""Parity at the benchmark configurations' own sizes, and the FP64 direct-sum
kernel that every accuracy figure of the benchmark rests on.

* tagi_direct_dev (the exact FP64 direct sum the benchmark and the autotuner
  measure errors against) against the oracle's direct sum, <= 1e-12.
* Single Z = 4 atom, 50,112 points, leaves 500 (the CPU-runnable case): the
  whole convolution against the oracle treecode, Yukawa k = 1 on f = V psi and
  Coulomb alpha = 1 on rho = 2 psi^2; lists integer for integer; FP64 <= 1e-12,
  mixed <= 1e-6.
* Coulomb Hartree, 1,498,624 points, leaves 2000: lists integer for integer;
  FP64 <= 1e-12 and mixed <= 1e-6 on a stratified sample of whole target
  batches (the oracle convolves only those batches, with the full lists).
* 32 Yukawa orbitals on a 1M-point mesh in one batched launch: mixed <= 1e-6
  for orbitals at the edges of the orbital groups, on sampled batches; then
  FP64 Gram-Schmidt over the 32 results, each step against the oracle's step
  on the same input (1e-13 times the step's own cancellation factor).

Reference call sites: greenIterationFixedPoint.py:314-321 (Yukawa orbital
convolution), scfFixedPoint.py:297-303 (Coulomb Hartree convolution),
Orthogonalization.c:14-119 (Gram-Schmidt).
"""
import math

import numpy as np
import pytest
import torch

from conftest import rel_l2, to_cuda

pytestmark = pytest.mark.gpu

YUK, COUL = 2, 1
SKIP, SS = 1, 2


def batch_pairs(cplan):
    """Pair count of every target batch of an oracle plan."""
    L = cplan.lists()
    st, tt = cplan.tree(0), cplan.tree(1)
    bn = L["batch_node"]
    bsz = tt["end"][bn] - tt["begin"][bn]
    src_len = st["end"] - st["begin"]
    cs = np.concatenate([[0], np.cumsum(src_len[L["near_list"]])])
    near = cs[L["near_off"][1:]] - cs[L["near_off"][:-1]]
    return bsz * (near + np.diff(L["far_off"]) * cplan.P)


def stratified_batches(cplan, count):
    """`count` batches evenly spread over the batches sorted by pair count
    (lightest and heaviest included)."""
    pairs = batch_pairs(cplan)
    order = np.argsort(pairs, kind="stable")
    pick = np.unique(np.linspace(0, len(order) - 1, min(count, len(order))).round().astype(int))
    return np.sort(order[pick])


def batch_target_indices(cplan, sel):
    """Caller-order target indices of the selected batches."""
    L = cplan.lists()
    tt = cplan.tree(1)
    return np.concatenate([tt["perm"][tt["begin"][n]:tt["end"][n]] for n in L["batch_node"][sel]])


def assert_same_lists(gplan, cplan):
    gl, cl = gplan.lists(), cplan.lists()
    for k in cl:
        assert np.array_equal(gl[k], cl[k]), f"list {k} differs from the oracle"


# ---------------------------------------------------------------------------
# The FP64 direct sum
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("kernel,kp,sing", [(YUK, 1.0, SS), (YUK, 2.3, SKIP), (COUL, 1.0, SS), (COUL, 0.0, SKIP)])
def test_direct_kernel_matches_oracle(dev, oracle, small_mesh, kernel, kp, sing):
    mesh, f, rho = small_mesh
    q = f if kernel == YUK else rho
    rng = np.random.default_rng(11)
    sub = np.sort(rng.choice(mesh.n, 3000, replace=False)).astype(np.int32)
    x, y, z, w, qt = to_cuda(mesh.x, mesh.y, mesh.z, mesh.w, q)
    st = torch.as_tensor(sub, device="cuda")
    got = dev.direct(x, y, z, qt, x, y, z, qt, w, kernel, [kp], sing, subset=st).cpu().numpy()
    ref = oracle.direct(mesh.x, mesh.y, mesh.z, q, mesh.x, mesh.y, mesh.z, q, mesh.w, kernel, [kp], sing,
                        subset=sub)
    assert rel_l2(got, ref) <= 1e-12


def test_direct_kernel_distinct_targets_and_all_targets(dev, oracle, small_mesh):
    """Targets that are not sources (no coincident pairs), every target computed."""
    mesh, f, rho = small_mesh
    rng = np.random.default_rng(12)
    tx, ty, tz = (rng.uniform(-3, 3, 2000) for _ in range(3))
    tv = rng.normal(size=2000)
    args = to_cuda(tx, ty, tz, tv, mesh.x, mesh.y, mesh.z, f, mesh.w)
    for kernel, kp in ((YUK, 0.8), (COUL, 1.0)):
        got = dev.direct(*args, kernel, [kp], SS).cpu().numpy()
        ref = oracle.direct(tx, ty, tz, tv, mesh.x, mesh.y, mesh.z, f, mesh.w, kernel, [kp], SS)
        assert rel_l2(got, ref) <= 1e-12, kernel


# ---------------------------------------------------------------------------
# Single Z = 4 atom, 50,112 points, leaves 500: the whole convolution
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def atom50k(dev, oracle, syn):
    mesh, f, rho = syn.single_atom(factor=1.0, max_depth=5)
    assert mesh.n == 50_112
    g = dev.TreecodePlan.for_mesh(*to_cuda(mesh.x, mesh.y, mesh.z, mesh.w), theta=0.7, degree=7,
                                  source_leaf=500, target_leaf=500)
    c = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, 7, 500, 500, 1.0)
    yield mesh, f, rho, g, c
    g.close()


def test_single_atom_50k_lists(atom50k):
    mesh, f, rho, g, c = atom50k
    assert_same_lists(g, c)
    assert g.info()["far_entries"] > 0


@pytest.mark.parametrize("kernel,q_name", [(YUK, "f"), (COUL, "rho")])
def test_single_atom_50k_whole_convolution(atom50k, kernel, q_name):
    mesh, f, rho, g, c = atom50k
    q = f if q_name == "f" else rho
    ref = c.convolve(q, q, mesh.w, kernel, [1.0], SS)
    (qt,) = to_cuda(q)
    out64 = g.convolve(qt, qt, kernel, [1.0], SS, precision="fp64").cpu().numpy()
    assert rel_l2(out64, ref) <= 1e-12
    out32 = g.convolve(qt, qt, kernel, [1.0], SS, precision="mixed").cpu().numpy()
    assert rel_l2(out32, ref) <= 1e-6


# ---------------------------------------------------------------------------
# Coulomb Hartree, 1,498,624 points, leaves 2000
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def hartree15m(dev, oracle, syn):
    mesh, rho = syn.hartree_system(seed=2)
    assert mesh.n == 1_498_624
    x, y, z, w = to_cuda(mesh.x, mesh.y, mesh.z, mesh.w)
    g = dev.TreecodePlan.for_mesh(x, y, z, w, theta=0.7, degree=7, source_leaf=2000, target_leaf=2000)
    c = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, 7, 2000, 2000, 1.0)
    sel = stratified_batches(c, 48)
    ref, _, _ = oracle.convolve_batches(c, rho, rho, mesh.w, COUL, [1.0], SS, sel)
    idx = batch_target_indices(c, sel)
    yield mesh, rho, g, c, ref[idx], idx
    g.close()


def test_hartree_1_5m_lists(hartree15m):
    mesh, rho, g, c, ref, idx = hartree15m
    assert_same_lists(g, c)


def test_hartree_1_5m_fp64_and_mixed(hartree15m):
    mesh, rho, g, c, ref, idx = hartree15m
    assert len(idx) > 20_000
    (qt,) = to_cuda(rho)
    out64 = g.convolve(qt, qt, COUL, [1.0], SS, precision="fp64").cpu().numpy()
    assert rel_l2(out64[idx], ref) <= 1e-12
    out32 = g.convolve(qt, qt, COUL, [1.0], SS, precision="mixed").cpu().numpy()
    assert rel_l2(out32[idx], ref) <= 1e-6


# ---------------------------------------------------------------------------
# 32 Yukawa orbitals on 1M points, one batched launch, then Gram-Schmidt
# ---------------------------------------------------------------------------
def test_32_orbitals_1m_batched_then_gram_schmidt(dev, oracle, syn):
    mesh, F, k = syn.multi_orbital_system(seed=3, n_orb=32)
    assert F.shape == (32, mesh.n) and mesh.n > 900_000
    x, y, z, w, Ft = to_cuda(mesh.x, mesh.y, mesh.z, mesh.w, F)
    g = dev.TreecodePlan.for_mesh(x, y, z, w, theta=0.7, degree=7, source_leaf=2000, target_leaf=2000)
    out = g.convolve(Ft, Ft, YUK, k, SS, precision="mixed")
    torch.cuda.synchronize()
    c = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, 7, 2000, 2000, 1.0)
    assert_same_lists(g, c)
    sel = stratified_batches(c, 16)
    idx = batch_target_indices(c, sel)
    outh = out.cpu().numpy()
    for o in (0, 7, 8, 31):   # first/last of orbital groups of 8
        ref, _, _ = oracle.convolve_batches(c, F[o], F[o], mesh.w, YUK, [k[o]], SS, sel)
        assert rel_l2(outh[o][idx], ref[idx]) <= 1e-6, o
    # FP64 Gram-Schmidt of the 32 new orbitals psi' = conv / 4pi, in orbital
    # order.  Each step is compared with the oracle's step on the same input;
    # the tolerance scales with |U| / |U - projections| (the cancellation the
    # step itself amplifies, whatever the summation order).
    V = (out / (4.0 * math.pi)).contiguous()
    for j in range(32):
        Vh = V.cpu().numpy()
        U = Vh[j].copy()
        r = (Vh[:j] * (U * mesh.w)).sum(1)
        perp = U - r @ Vh[:j]
        amp = math.sqrt((U * U * mesh.w).sum() / (perp * perp * mesh.w).sum())
        dev.mgs(V, V[j].clone(), w, j)
        oracle.mgs(Vh, U, mesh.w, j)
        assert rel_l2(V[j].cpu().numpy(), Vh[j]) <= 1e-13 * max(1.0, amp), (j, amp)
    g.close()
