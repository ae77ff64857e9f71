"""Launch-shape autotuner for the treecode convolution (project-written).

For one mesh and one convolution workload it times candidate shapes on the
GPU with CUDA events and keeps the fastest candidate that meets the accuracy
target.  The knobs:

  * source / target leaf sizes of the plan -- the tree shape sets the
    near/far balance and the target-batch sizes;
  * orbitals per work item (1, 4, 8 or 16; Yukawa in mixed precision shares each
    pair's geometry across a group of orbitals);
  * targets per thread in the single-orbital field kernels (1 or 2).

Accuracy gate: the first orbital's result at a seeded sample of targets is
compared with the exact FP64 direct sum there (tagi_direct_dev); a candidate
whose relative L2 error exceeds ``tol`` is rejected.  Cost of a candidate =
convolution time per orbital + plan build time / ``reuse`` (the number of
orbital convolutions one plan serves: orbitals x Green-iteration steps).

The reference fixes these by hand per run (theta, degree, leaf sizes passed
to callTreedriver, 3D-GreenIteration/src/utilities/BaryTreeInterface.py:88-93);
its callers use source and target leaves of equal size.

Results can be kept in a JSON cache keyed by GPU name, kernel, singularity,
precision, orbital count and point count, so a workload is tuned once.
"""
import json
import os
import time

import numpy as np
import torch

try:
    from . import device as _dev_mod
    from .BaryTreeInterface import Kernel
except ImportError:
    import device as _dev_mod
    from BaryTreeInterface import Kernel

DEFAULT_LEAVES = ((1000, 1000), (2000, 1000), (2000, 2000), (4000, 1000), (4000, 2000))


def _events():
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _key(kernel, singularity, precision, norb, n, theta, degree):
    return (f"{torch.cuda.get_device_name()}|k{int(kernel)}|s{int(singularity)}|{precision}|"
            f"o{int(norb)}|n{int(n)}|t{theta}|d{int(degree)}")


def _load(path):
    if not path or not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, cache):
    if not path:
        return
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _group_candidates(kernel, precision, norb):
    if int(kernel) != int(Kernel.YUKAWA) or precision != "mixed":
        return (1,)
    return tuple(g for g in (1, 4, 8, 16) if g == 1 or norb >= g)


def tune(x, y, z, w, values, kernel, kernel_params, singularity, precision="mixed", theta=0.7,
         degree=7, leaves=DEFAULT_LEAVES, reuse=10, tol=1e-6, n_check=1024, sample_orbitals=8,
         repeats=2, cache_path=None, seed=0, stream=None):
    """Tune one mesh (targets = sources = x, y, z with weights w).

    values: CUDA float64 [norb, n]; kernel_params: norb host values.  The first
    min(norb, sample_orbitals) orbitals are timed.  Returns a dict with the
    chosen source_leaf, target_leaf, orbitals_per_item, targets_per_thread,
    their ms per orbital, plan ms, relative error, and the table of all
    candidates tried."""
    n = int(x.numel())
    vals = values.reshape(-1, n)
    norb = vals.shape[0]
    ns = max(1, min(norb, sample_orbitals))
    vs = vals[:ns].contiguous()
    kp = np.asarray(kernel_params, dtype=np.float64).reshape(-1)[:ns]
    key = _key(kernel, singularity, precision, norb, n, theta, degree)
    cache = _load(cache_path)
    if key in cache:
        return dict(cache[key], cached=True)

    # exact reference at seeded sample targets, first orbital
    rng = np.random.default_rng(seed)
    sub_np = np.sort(rng.choice(n, min(n_check, n), replace=False)).astype(np.int32)
    sub = torch.as_tensor(sub_np, device=x.device)
    v0 = vs[0].contiguous()
    ref = _dev_mod.direct(x, y, z, v0, x, y, z, v0, w, kernel, [kp[0]], singularity, subset=sub,
                          stream=stream)
    refn = float(torch.linalg.norm(ref))
    out = torch.empty_like(vs)

    def run(plan, og, tpt):
        plan.convolve(vs, vs, kernel, kp, singularity, precision=precision, out=out, stream=stream,
                      orbitals_per_item=og, targets_per_thread=tpt)

    def measure(sl, tl, og, tpt, plan=None):
        built = plan is None
        a, b = _events()
        if built:
            a.record()
            plan = _dev_mod.TreecodePlan.for_mesh(x, y, z, w, theta=theta, degree=degree,
                                                  source_leaf=sl, target_leaf=tl, stream=stream)
            b.record()
            torch.cuda.synchronize()
            plan_ms = a.elapsed_time(b)
        else:
            plan_ms = None
        run(plan, og, tpt)  # warm-up: work lists, scratch
        torch.cuda.synchronize()
        err = float(torch.linalg.norm(out[0][sub.long()] - ref)) / max(refn, 1e-300)
        ts = []
        for _ in range(repeats):
            a, b = _events()
            a.record()
            run(plan, og, tpt)
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return plan, plan_ms, min(ts) / ns, err

    table = []
    best = None
    # stage 1: tree shape with automatic grouping
    plans = {}
    for sl, tl in leaves:
        plan, plan_ms, ms, err = measure(sl, tl, 0, 0)
        cost = ms + plan_ms / max(reuse, 1)
        row = dict(source_leaf=sl, target_leaf=tl, orbitals_per_item=0, targets_per_thread=0,
                   ms_per_orbital=ms, plan_ms=plan_ms, rel_err=err, cost=cost, ok=err <= tol)
        table.append(row)
        plans[(sl, tl)] = (plan, plan_ms)
        if row["ok"] and (best is None or cost < best["cost"]):
            best = row
    met = best is not None
    if not met:  # nothing meets the target: keep the most accurate tree, flagged
        best = min(table, key=lambda r: r["rel_err"])
    # stage 2: kernel shape on the chosen tree
    plan, plan_ms = plans[(best["source_leaf"], best["target_leaf"])]
    for og in _group_candidates(kernel, precision, ns):
        for tpt in (1, 2):
            _, _, ms, err = measure(best["source_leaf"], best["target_leaf"], og, tpt, plan=plan)
            cost = ms + plan_ms / max(reuse, 1)
            row = dict(source_leaf=best["source_leaf"], target_leaf=best["target_leaf"],
                       orbitals_per_item=og, targets_per_thread=tpt, ms_per_orbital=ms, plan_ms=plan_ms,
                       rel_err=err, cost=cost, ok=err <= tol)
            table.append(row)
            if (row["ok"] or not met) and cost < best["cost"] and err <= max(tol, best["rel_err"]):
                best = row
    for p, _ in plans.values():
        p.close()
    res = dict(best, met_tol=met, table=table, sample_orbitals=ns, reuse=reuse, tol=tol, key=key,
               tuned_at=time.strftime("%Y-%m-%dT%H:%M:%S"))
    cache[key] = res
    _store(cache_path, cache)
    return dict(res, cached=False)


def tune_systems(meshes, values, kernel_params, kernel, singularity, precision="mixed", theta=0.7,
                 degree=7, leaves=DEFAULT_LEAVES, reuse=10, tol=1e-6, sample_orbitals=8, cache_path=None,
                 stream=None):
    """Tune several systems for one joint launch: leaf sizes per system, then
    the launch-wide orbitals per item and targets per thread on the joint
    launch.  meshes: list of (x, y, z, w) CUDA tensors; values: list of
    [norb_s, n_s] CUDA tensors; kernel_params: list of host arrays.  Returns
    dict(leaves=[(sl, tl)...], orbitals_per_item, targets_per_thread, systems=[per-system
    results], joint=[rows])."""
    per = []
    for (x, y, z, w), v, k in zip(meshes, values, kernel_params):
        per.append(tune(x, y, z, w, v, kernel, k, singularity, precision=precision, theta=theta,
                        degree=degree, leaves=leaves, reuse=reuse, tol=tol,
                        sample_orbitals=sample_orbitals, cache_path=cache_path, stream=stream))
    plans = [_dev_mod.TreecodePlan.for_mesh(x, y, z, w, theta=theta, degree=degree,
                                            source_leaf=r["source_leaf"], target_leaf=r["target_leaf"],
                                            stream=stream)
             for (x, y, z, w), r in zip(meshes, per)]
    # the joint launch is timed on up to 16 orbitals per system, so every group size can be tried
    ns = [max(1, min(v.reshape(v.shape[0], -1).shape[0], max(sample_orbitals, 16))) for v in values]
    vs = [v.reshape(v.shape[0], -1)[:m].contiguous() for v, m in zip(values, ns)]
    ks = [np.asarray(k, dtype=np.float64).reshape(-1)[:m] for k, m in zip(kernel_params, ns)]
    outs = [torch.empty_like(v) for v in vs]
    joint = []
    best = None
    for og in _group_candidates(kernel, precision, max(ns)):
        for tpt in (1, 2):
            S = _dev_mod.Systems(plans, ns, kernel, precision=precision, orbitals_per_item=og,
                                 targets_per_thread=tpt, stream=stream)
            S.convolve(vs, vs, ks, singularity, outs=outs, stream=stream)
            torch.cuda.synchronize()
            a, b = _events()
            a.record()
            S.convolve(vs, vs, ks, singularity, outs=outs, stream=stream)
            b.record()
            torch.cuda.synchronize()
            ms = a.elapsed_time(b)
            S.close()
            row = dict(orbitals_per_item=og, targets_per_thread=tpt, ms=ms)
            joint.append(row)
            if best is None or ms < best["ms"]:
                best = row
    for p in plans:
        p.close()
    return dict(leaves=[(r["source_leaf"], r["target_leaf"]) for r in per],
                orbitals_per_item=best["orbitals_per_item"], targets_per_thread=best["targets_per_thread"],
                systems=per, joint=joint)
