"""Yukawa orbital groups of 16 (orbitals packed in pairs per FP32 operation)
on the GPU.

The 16-orbital kernels sum each orbital's pairs in a different order than the
8-orbital ones (one lane per orbital instead of one lane per source), so the
two are compared at the mixed-precision tolerance, and both against the CPU
oracle's FP64 treecode on the same tree (relative L2 <= 1e-6).  Degrees 3, 5,
7 and 9 take the four far-field instantiations (proxy-grid edge <= 4, <= 8,
exactly 8, above 8); 20 orbitals leave 12 padded slots in the second group.
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2, to_cuda

pytestmark = pytest.mark.gpu

NORB = 20


@pytest.fixture(scope="module")
def system(syn):
    (mesh, F, k), = syn.uneven_systems(seed=21, sizes=(30000,), orbitals=(NORB,), max_depth=5)
    return mesh, F, k


@pytest.mark.parametrize("degree", [7, 9, 5, 3])
def test_group16_matches_group8_and_oracle(BT, dev, oracle, system, degree):
    mesh, F, k = system
    x, y, z, w, Ft = to_cuda(mesh.x, mesh.y, mesh.z, mesh.w, F)
    plan = dev.TreecodePlan.for_mesh(x, y, z, w, theta=0.7, degree=degree, source_leaf=300, target_leaf=300)
    assert plan.info()["far_entries"] > 0
    SS = BT.Singularity.SUBTRACTION
    a = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, k, SS, precision="mixed", orbitals_per_item=16)
    b = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, k, SS, precision="mixed", orbitals_per_item=8)
    plan.close()
    assert torch.isfinite(a).all()
    for o in range(NORB):
        assert rel_l2(a[o].cpu().numpy(), b[o].cpu().numpy()) <= 1e-6
    if degree in (7, 9):
        c = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, degree, 300, 300, 1.0)
        got = a.cpu().numpy()
        for o in (0, 15, 16, NORB - 1):
            ref = c.convolve(F[o], F[o], mesh.w, BT.Kernel.YUKAWA, [k[o]], SS)
            assert rel_l2(got[o], ref) <= 1e-6


def test_group16_skipping_matches_group8(BT, dev, system):
    mesh, F, k = system
    x, y, z, w, Ft = to_cuda(mesh.x, mesh.y, mesh.z, mesh.w, F)
    plan = dev.TreecodePlan.for_mesh(x, y, z, w, theta=0.7, degree=7, source_leaf=300, target_leaf=300)
    SK = BT.Singularity.SKIPPING
    a = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, k, SK, precision="mixed", orbitals_per_item=16)
    b = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, k, SK, precision="mixed", orbitals_per_item=8)
    plan.close()
    for o in range(NORB):
        assert rel_l2(a[o].cpu().numpy(), b[o].cpu().numpy()) <= 1e-6


def test_group16_systems_equal_single_calls(BT, dev, syn):
    out = syn.uneven_systems(seed=22, sizes=(8000, 20000), orbitals=(17, 32), max_depth=5)
    plans = [dev.TreecodePlan.for_mesh(*to_cuda(m.x, m.y, m.z, m.w), theta=0.7, degree=7, source_leaf=300,
                                       target_leaf=300) for m, _, _ in out]
    S = dev.Systems(plans, [F.shape[0] for _, F, _ in out], BT.Kernel.YUKAWA, precision="mixed",
                    orbitals_per_item=16)
    assert S.info()["orbitals_per_item"] == 16
    Fs = [to_cuda(F)[0] for _, F, _ in out]
    res = S.convolve(Fs, Fs, [k for _, _, k in out], BT.Singularity.SUBTRACTION)
    for (m, F, k), p, Ft, r in zip(out, plans, Fs, res):
        ref = p.convolve(Ft, Ft, BT.Kernel.YUKAWA, k, BT.Singularity.SUBTRACTION, precision="mixed",
                         orbitals_per_item=16)
        assert torch.equal(r, ref)
    S.close()
    for p in plans:
        p.close()


def test_group16_loop_ceilings_are_measured(native):
    import ctypes
    L = native.lib()
    v = ctypes.c_double()
    for variant in (4, 5):
        native.check(L.tagi_pair_peak(2, 2, variant, 1.0, ctypes.byref(v), None))
        assert v.value > 1e11
    assert L.tagi_pair_peak(2, 2, 6, 1.0, ctypes.byref(v), None) == native.TAGI_ERR_ARG
