"""Batched calls on the GPU: several systems in one persistent launch per field
pass, kernel parameters in device memory, CUDA-graph capture and replay.

Every system of a multi-system launch runs the same per-item arithmetic as
its own single-plan call with the same orbital grouping, so those results are
compared for EQUALITY; accuracy against the CPU oracle is re-checked for one
system at the mixed-precision tolerance (relative L2 <= 1e-6) and the FP64
tolerance (<= 1e-12).
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2, to_cuda

pytestmark = pytest.mark.gpu

SIZES = (6000, 15000, 30000)
ORBITALS = (3, 5, 9)


@pytest.fixture(scope="module")
def systems(dev, syn):
    out = []
    for mesh, F, k in syn.uneven_systems(seed=11, sizes=SIZES, orbitals=ORBITALS, max_depth=5):
        plan = dev.TreecodePlan.for_mesh(*to_cuda(mesh.x, mesh.y, mesh.z, mesh.w), theta=0.7, degree=7,
                                         source_leaf=300, target_leaf=300)
        out.append((mesh, F, k, plan))
    assert any(p.info()["far_entries"] > 0 for *_, p in out)
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_systems_equal_single_plan_calls(BT, dev, systems, precision):
    plans = [p for *_, p in systems]
    S = dev.Systems(plans, ORBITALS, BT.Kernel.YUKAWA, precision=precision)
    info = S.info()
    assert info["systems"] == 3
    assert info["near_items"] > 0 and info["far_items"] > 0
    og = info["orbitals_per_item"]
    assert og in ((4, 8, 16) if precision == "mixed" else (1,))
    Fs = [to_cuda(F)[0] for _, F, _, _ in systems]
    outs = S.convolve(Fs, Fs, [k for _, _, k, _ in systems], BT.Singularity.SUBTRACTION)
    for (mesh, F, k, plan), Ft, o in zip(systems, Fs, outs):
        ref = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, k, BT.Singularity.SUBTRACTION, precision=precision,
                            orbitals_per_item=og)
        assert torch.equal(o, ref)
    S.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_systems_match_oracle(BT, dev, oracle, systems, precision, tol):
    plans = [p for *_, p in systems]
    S = dev.Systems(plans, ORBITALS, BT.Kernel.YUKAWA, precision=precision)
    Fs = [to_cuda(F)[0] for _, F, _, _ in systems]
    outs = S.convolve(Fs, Fs, [k for _, _, k, _ in systems], BT.Singularity.SUBTRACTION)
    mesh, F, k, _ = systems[1]
    c = oracle.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, 0.7, 7, 300, 300, 1.0)
    got = outs[1].cpu().numpy()
    for o in (0, len(k) - 1):
        ref = c.convolve(F[o], F[o], mesh.w, BT.Kernel.YUKAWA, [k[o]], BT.Singularity.SUBTRACTION)
        assert rel_l2(got[o], ref) <= tol
    S.close()


def test_one_shot_batched_call_equals_systems_object(BT, dev, systems):
    meshes = [m for m, *_ in systems]
    off = np.concatenate([[0], np.cumsum([m.n for m in meshes])]).astype(np.int32)
    x, y, z, w = (np.concatenate([getattr(m, a) for m in meshes]) for a in "xyzw")
    vals = np.concatenate([F.reshape(-1) for _, F, _, _ in systems])
    ks = np.concatenate([k for _, _, k, _ in systems])
    xt, yt, zt, wt, vt = to_cuda(x, y, z, w, vals)
    got = dev.treecode_batched(off, ORBITALS, xt, yt, zt, wt, vt, BT.Kernel.YUKAWA, ks,
                               BT.Singularity.SUBTRACTION, theta=0.7, degree=7, source_leaf=300,
                               target_leaf=300, precision="mixed")
    S = dev.Systems([p for *_, p in systems], ORBITALS, BT.Kernel.YUKAWA, precision="mixed")
    Fs = [to_cuda(F)[0] for _, F, _, _ in systems]
    outs = S.convolve(Fs, Fs, [k for _, _, k, _ in systems], BT.Singularity.SUBTRACTION)
    assert torch.equal(got, torch.cat([o.reshape(-1) for o in outs]))
    S.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_kernel_parameters_equal_host(BT, systems, precision):
    mesh, F, k, plan = systems[1]
    (Ft,) = to_cuda(F)
    host = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, k, BT.Singularity.SUBTRACTION, precision=precision)
    devk = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, torch.as_tensor(k, device="cuda"),
                         BT.Singularity.SUBTRACTION, precision=precision)
    assert torch.equal(host, devk)
    assert not plan.check_parameters()


def test_unusable_device_parameter_is_flagged(BT, systems):
    mesh, F, k, plan = systems[0]
    (Ft,) = to_cuda(F[0])
    out = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, torch.tensor([-1.0], device="cuda", dtype=torch.float64),
                        BT.Singularity.SUBTRACTION)
    torch.cuda.synchronize()
    assert plan.check_parameters()
    assert torch.isnan(out).all()
    assert not plan.check_parameters()  # the check clears the flag


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_matches_eager_calls(BT, dev, systems, precision):
    """Capture one batched convolution with device-resident k_i, then change the
    charge vectors and k_i in place and replay: the graph computes exactly
    what an uncaptured call on the new data computes."""
    mesh, F, k, plan = systems[2]
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(2)
    with torch.cuda.stream(stream):
        Ft = torch.as_tensor(F, device="cuda").contiguous()
        kt = torch.as_tensor(k, device="cuda").contiguous()
        out = torch.empty_like(Ft)
        plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, kt, BT.Singularity.SUBTRACTION, precision=precision, out=out,
                      stream=stream)  # uncaptured first call: scratch and work lists
        with dev.Graph.capture(stream) as g:
            plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, kt, BT.Singularity.SUBTRACTION, precision=precision,
                          out=out, stream=stream)
        assert g.nodes() >= 6
        F2 = F * rng.uniform(0.5, 1.5, (F.shape[0], 1))
        k2 = rng.uniform(0.4, 3.0, len(k))
        Ft.copy_(torch.as_tensor(F2, device="cuda"))
        kt.copy_(torch.as_tensor(k2, device="cuda"))
        g.replay(stream)
        stream.synchronize()
        ref = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, k2, BT.Singularity.SUBTRACTION, precision=precision,
                            stream=stream)
        stream.synchronize()
    assert torch.equal(out, ref)
    g.close()


def test_capture_without_prior_call_is_refused(BT, dev, native, systems):
    mesh, F, k, _ = systems[0]
    fresh = dev.TreecodePlan.for_mesh(*to_cuda(mesh.x, mesh.y, mesh.z, mesh.w), source_leaf=300,
                                      target_leaf=300)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        Ft = torch.as_tensor(F, device="cuda").contiguous()
        kt = torch.as_tensor(k, device="cuda").contiguous()
        out = torch.empty_like(Ft)
        with pytest.raises(native.TagiError) as e:
            with dev.Graph.capture(stream):
                fresh.convolve(Ft, Ft, BT.Kernel.YUKAWA, kt, BT.Singularity.SUBTRACTION, out=out, stream=stream)
        assert e.value.code == native.TAGI_ERR_STATE
        # the stream is usable again and the same call now runs
        fresh.convolve(Ft, Ft, BT.Kernel.YUKAWA, kt, BT.Singularity.SUBTRACTION, out=out, stream=stream)
        stream.synchronize()
    assert torch.isfinite(out).all()
    fresh.close()


def test_targets_per_thread_does_not_change_results(BT, systems):
    mesh, F, k, plan = systems[2]
    (Ft,) = to_cuda(F[:2])
    a = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, k[:2], BT.Singularity.SUBTRACTION, orbitals_per_item=1,
                      targets_per_thread=1)
    b = plan.convolve(Ft, Ft, BT.Kernel.YUKAWA, k[:2], BT.Singularity.SUBTRACTION, orbitals_per_item=1,
                      targets_per_thread=2)
    assert torch.equal(a, b)


def test_autotune_picks_a_candidate_within_tolerance(BT, pkg, systems, tmp_path):
    import importlib
    tune = importlib.import_module(pkg.__name__ + ".autotune")
    mesh, F, k, _ = systems[2]
    x, y, z, w, Ft = to_cuda(mesh.x, mesh.y, mesh.z, mesh.w, F)
    cache = str(tmp_path / "tune.json")
    r = tune.tune(x, y, z, w, Ft, BT.Kernel.YUKAWA, k, BT.Singularity.SUBTRACTION,
                  leaves=((300, 300), (600, 300)), sample_orbitals=4, repeats=1, n_check=512, tol=1e-5,
                  cache_path=cache)
    assert r["met_tol"] and r["rel_err"] <= 1e-5 and not r["cached"]
    assert (r["source_leaf"], r["target_leaf"]) in ((300, 300), (600, 300))
    assert r["orbitals_per_item"] in (0, 1, 4) and r["targets_per_thread"] in (0, 1, 2)
    assert len(r["table"]) == 2 + 2 * 2  # two trees, then groups {1, 4} x targets per thread {1, 2}
    again = tune.tune(x, y, z, w, Ft, BT.Kernel.YUKAWA, k, BT.Singularity.SUBTRACTION,
                      leaves=((300, 300), (600, 300)), sample_orbitals=4, tol=1e-5, cache_path=cache)
    assert again["cached"] and again["source_leaf"] == r["source_leaf"]


def test_group_pair_ceiling_is_measured(native):
    import ctypes
    L = native.lib()
    v = ctypes.c_double()
    native.check(L.tagi_pair_peak(2, 2, 2, 1.0, ctypes.byref(v), None))
    assert v.value > 1e11
    assert L.tagi_pair_peak(1, 2, 2, 1.0, ctypes.byref(v), None) == native.TAGI_ERR_UNSUPPORTED
