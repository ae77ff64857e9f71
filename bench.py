#!/usr/bin/env python
"""Benchmark of the GB300 treecode convolution path.

Workload (default): the Coulomb Hartree convolution with singularity
subtraction on a seeded synthetic ~1.5M-point mesh (4 nuclei in a 6 Bohr box,
Z from {1,6,8}, order-7 cells, depth <= 7; density = 3 Gaussians per nucleus,
exponents log-uniform in [0.1, 10]), mixed precision, degree 7, theta 0.7.

One step = one full treecode convolution as one callTreedriver call does it:
tree + batches + lists + weight charges (the plan), modified charges, near
and far fields, epilogue -- inputs already resident in HBM.  ``value`` =
convolutions/s over all ranks.  ``e2e`` = the same through the C ABI
(tagi_BaryTreeInterface_ex) with pinned host buffers: host->device copies,
device allocation and the device->host result copy are inside the timing.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload hartree|orbitals|uneven|scf|mesh|twomesh]

``--workload uneven``: six independent synthetic systems (50k .. 2.5M points,
4/8/8/16/32/64 orbitals, Yukawa with subtraction, k_i ~ U[0.4, 3]) convolved
together, all orbitals of all systems in one persistent launch per field pass,
the launch sequence captured once as a CUDA graph and replayed; leaf sizes and
kernel shape chosen by the autotuner (untimed).  One step = one replay: one
Green-iteration sweep's convolutions (plans reused, as Green iteration reuses
them).  Compared with the plain path: one FP64 tagi_treecode_dev call per
orbital (tree + convolution each, reference parameters: leaves 500).

``--workload mesh``: the ring molecule's two-level mesh built on the device
(refinement + coarse and fine points); ``--workload twomesh``: the two-mesh
eigenvalue correction of 21 orbitals on that mesh.

``--impl reference`` times the CPU FP64 restatement of the same treecode (the
reference's BaryTree is not available) on the host cores, on a bounded sample
of target batches per step, extrapolated by pair count.
"""
import argparse
import ctypes
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = "treecode-accelerated-green-iteration_gb300"
sys.path.insert(0, ROOT)

METRIC = "orbital convs/s at 1e-6 rel err; wall time to 1e-5 Ha SCF: chosen vs plain"
UNIT = "convolutions/s"
THETA, DEGREE = 0.7, 7
LEAF = {"hartree": (2000, 2000), "orbitals": (2000, 2000)}
PAIR_FLOPS = {"coulomb_ss": 14, "yukawa_ss": 15}  # FP32 pipe operations counted per pair in the near-tile loop


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="hartree", choices=["hartree", "orbitals", "uneven", "scf", "mesh", "twomesh"])
    ap.add_argument("--scf-points", type=int, default=3_000_000, help="scf workload: mesh points")
    ap.add_argument("--scf-max-iter", type=int, default=60)
    ap.add_argument("--scf-orbitals", type=int, default=21, help="scf workload: orbitals (21 occupied)")
    ap.add_argument("--scf-mixing", type=float, default=0.3, help="scf workload: density mixing parameter")
    ap.add_argument("--scf-time-limit", type=float, default=1500.0, help="scf workload: seconds per run")
    ap.add_argument("--fp64-sample-systems", type=int, default=2,
                    help="uneven workload: systems whose plain FP64 one-call-per-orbital time is measured")
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="target CPU seconds of field work per CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def job_time_ms(local_ms, device=None):
    """Whole-job time: the slowest rank's timed region (MAX all-reduce; one rank: itself)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(local_ms)
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank_step, steps, world_size, total_ms):
    """Throughput of the whole job: units all ranks processed / the job time."""
    return units_per_rank_step * steps * world_size / (total_ms * 1e-3)


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------
def make_workload(name):
    pkg = importlib.import_module(PKG)
    syn = pkg.synthetic
    BT = pkg.BaryTreeInterface
    if name == "hartree":
        mesh, rho = syn.hartree_system(seed=2)
        return dict(mesh=mesh, values=rho[None, :], kparams=np.array([[1.0]]),
                    kernel=BT.Kernel.COULOMB, singularity=BT.Singularity.SUBTRACTION,
                    label="coulomb_ss", desc="coulomb_hartree_ss_1.5M")
    mesh, F, k = syn.multi_orbital_system(seed=3, n_orb=32)
    return dict(mesh=mesh, values=F, kparams=k[:, None], kernel=BT.Kernel.YUKAWA,
                singularity=BT.Singularity.SUBTRACTION, label="yukawa_ss",
                desc="yukawa_32_orbitals_1M")


# ---------------------------------------------------------------------------
# Clock sampling during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


# ---------------------------------------------------------------------------
# CPU baseline: the FP64 treecode restatement on the host cores
# ---------------------------------------------------------------------------
def cpu_treecode_sample(wl, target_seconds, threads, leaf=None):
    """Build the CPU plan (timed), convolve a sample of whole target batches
    sized to ~target_seconds of field work, extrapolate to one convolution by
    the pair counts of the full lists.  Returns (seconds per convolution, info)."""
    from oracle import oracle as O
    O.build()
    mesh = wl["mesh"]
    sl, tl = leaf or LEAF["hartree"]
    t0 = time.perf_counter()
    plan = O.Plan(mesh.x, mesh.y, mesh.z, mesh.x, mesh.y, mesh.z, mesh.w, THETA, DEGREE, sl, tl, 1.0)
    t_plan = time.perf_counter() - t0
    L = plan.lists()
    st, tt = plan.tree(0), plan.tree(1)
    nb = plan.n_batches
    bsz = tt["end"][L["batch_node"]] - tt["begin"][L["batch_node"]]
    ncnt = np.zeros(nb)
    src_len = st["end"] - st["begin"]
    for b in range(nb):
        ncnt[b] = src_len[L["near_list"][L["near_off"][b]:L["near_off"][b + 1]]].sum()
    pairs_b = bsz * (ncnt + np.diff(L["far_off"]) * plan.P)
    total_pairs = pairs_b.sum()
    rng = np.random.default_rng(17)
    order = rng.permutation(nb)
    q = wl["values"][0]
    kp = wl["kparams"][0]
    # calibration on a few batches, then a sample sized to the time target
    sel = np.sort(order[:4])
    _, (t_up, t_f), (pn, pf) = O.convolve_batches(plan, q, q, mesh.w, wl["kernel"], kp,
                                                  wl["singularity"], sel, threads)
    rate = (pn + pf) / max(t_f, 1e-9)
    want = rate * target_seconds
    csum = np.cumsum(pairs_b[order])
    nsel = int(np.clip(np.searchsorted(csum, want) + 1, 4, nb))
    sel = np.sort(order[:nsel])
    _, (t_up, t_f), (pn, pf) = O.convolve_batches(plan, q, q, mesh.w, wl["kernel"], kp,
                                                  wl["singularity"], sel, threads)
    frac = (pn + pf) / total_pairs
    seconds = t_plan + t_up + t_f / frac
    return seconds, dict(batches=int(nsel), of_batches=int(nb), pair_fraction=float(frac),
                         plan_s=t_plan, upward_s=t_up, sample_field_s=t_f,
                         pairs_per_s=(pn + pf) / t_f, total_pairs=float(total_pairs))


def reference_arm_mesh(args):
    """The oracle's restatement of the reference's mesh construction, whole mesh per step."""
    from oracle import mesh_oracle as MO
    pkg = importlib.import_module(PKG)
    c = MESH_CFG
    nuclei, _ = pkg.synthetic.ring_molecule()
    secs, n = [], 0
    for k in range(args.warmup + args.steps):
        a = time.perf_counter()
        base = MO.base_cells(c["XL"], c["XL"], c["XL"], c["max_side"])
        tab = MO.cell_table(MO.refine(base, nuclei, c["h"], c["H"], c["r"], c["level"]), c["order"])
        pts = MO.points(tab, c["order"])
        if k >= args.warmup:
            secs.append(time.perf_counter() - a)
        n = len(pts[0]) + len(pts[4])
    value = n / float(np.mean(secs))
    unit = "points/s"
    return {"metric": "mesh points/s (two-level first-kind mesh, refinement + points)", "value": value,
            "unit": unit, "ms_per_step": float(np.mean(secs)) * 1e3, "dtype": "f64",
            "config": {"workload": "ring_two_level_mesh", **c},
            "cpu_baseline": {"value": value, "unit": unit, "cores": 1, "kind": "port",
                             "sample": "whole mesh per step (Python recursion, numpy per cell)"},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def reference_arm_twomesh(args):
    """Oracle FP64 two-mesh correction cost per orbital on the h = 3 construction."""
    from oracle import mesh_oracle as MO
    pkg = importlib.import_module(PKG)
    c = MESH_CFG
    nuclei, _ = pkg.synthetic.ring_molecule()
    tab, pts = MO.build(c["XL"], c["max_side"], nuclei, c["order"], 3.0, c["H"], c["r"], c["level"])
    threads = os.cpu_count() or 1
    per_step = max(2.0, args.cpu_seconds / 4)
    secs = []
    for k in range(args.warmup + args.steps):
        s, info = cpu_two_mesh_sample(tab, pts, nuclei, per_step, threads)
        if k >= args.warmup:
            secs.append(s)
    value = 1.0 / float(np.mean(secs))
    unit = "orbitals/s"
    sample = (f"oracle FP64 correction of one orbital at h = 3 ({len(pts[0])} coarse / {len(pts[4])} fine "
              f"points): plan + upward in full, Yukawa field on {info['batches']} of {info['of_batches']} "
              "batches, extrapolated by pair count")
    return {"metric": "two-mesh eigenvalue corrections/s (orbitals)", "value": value, "unit": unit,
            "ms_per_step": float(np.mean(secs)) * 1e3, "dtype": "f64",
            "config": {"workload": "ring_two_mesh_correction_h3", "coarse_points": len(pts[0]),
                       "fine_points": len(pts[4]), "theta": THETA - 0.15, "degree": DEGREE + 2},
            "cpu_baseline": {"value": value, "unit": unit, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def reference_arm(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    if args.workload in ("mesh", "twomesh"):
        body = (reference_arm_mesh if args.workload == "mesh" else reference_arm_twomesh)(args)
        line = {"impl": "reference", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "data": "synthetic ring molecule (seeded)", **body}
        print(json.dumps(line), flush=True)
        return 0
    if args.workload == "scf":
        print(json.dumps({"impl": "reference", "unavailable": "the reference SCF needs its atomic data files "
                          "and BaryTree, neither of which is present"}), flush=True)
        return 0
    wl = make_workload(args.workload)
    threads = os.cpu_count() or 1
    per_step = max(2.0, args.cpu_seconds / 4)
    for _ in range(args.warmup):
        cpu_treecode_sample(wl, per_step, threads)
    secs, info = [], None
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s, info = cpu_treecode_sample(wl, per_step, threads)
        secs.append(s)
    wall = time.perf_counter() - t0
    mean_s = float(np.mean(secs))
    value = 1.0 / mean_s
    sample = (f"FP64 treecode restatement (oracle/tagi_oracle.c, OpenMP) on {info['batches']} of "
              f"{info['of_batches']} target batches per step ({info['pair_fraction']:.4f} of the "
              "pairs), plan + upward pass timed in full, fields extrapolated by pair count")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": wl["desc"], "points": int(wl["mesh"].n), "theta": THETA,
                       "degree": DEGREE, "leaf": list(LEAF["hartree"]), "precision": "fp64"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall, "cpu_pairs_per_s": info["pairs_per_s"]}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
def profile_traffic(kernel, label):
    """DRAM bytes per launch of a field kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_field_{label}_1.5M.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_launch"):
            try:
                return float(line.split("=")[1].split()[0])
            except (IndexError, ValueError):
                return None
    return None


def gb300_arm(args):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    pkg = importlib.import_module(PKG)
    dev = importlib.import_module(PKG + ".device")
    nat = pkg._native
    L = nat.lib()
    wl = make_workload(args.workload)
    mesh = wl["mesh"]
    cuda = torch.device("cuda", local)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    x, y, z, w = t(mesh.x), t(mesh.y), t(mesh.z), t(mesh.w)
    vals = t(wl["values"])
    norb = vals.shape[0]
    sl, tl = LEAF[args.workload]
    stream = torch.cuda.current_stream()

    def step():
        plan = dev.TreecodePlan.for_mesh(x, y, z, w, theta=THETA, degree=DEGREE, source_leaf=sl,
                                         target_leaf=tl)
        out = plan.convolve(vals, vals, wl["kernel"], wl["kparams"], wl["singularity"],
                            precision="mixed")
        info = plan.info()
        plan.close()
        return out, info

    for _ in range(args.warmup):
        out, info = step()
    torch.cuda.synchronize()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=cuda)  # 256 MB > L2
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    L.tagi_profile(1)
    prof_ms = np.zeros(7)
    prof_n = np.zeros(7, dtype=np.int64)
    prof_np = prof_n.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
    L.tagi_profile_read(nat.dptr(prof_ms), prof_np, 7)  # discard warm-up marks
    with ClockSampler(local) as clocks:
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()
        n0 = L.tagi_launch_count()
        for k in range(args.steps):
            flush.zero_()
            evs[k][0].record(stream)
            out, info = step()
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        if ws > 1:
            dist.barrier()
        launches = L.tagi_launch_count() - n0
    L.tagi_profile_read(nat.dptr(prof_ms), prof_np, 7)
    L.tagi_profile(0)
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = job_time_ms(float(sum(step_ms)), cuda)
    value = job_value(norb, args.steps, ws, total_ms)

    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return 0

    # accuracy of the timed result against the exact FP64 direct sum (GPU) on seeded targets
    rng = np.random.default_rng(99)
    sub = torch.as_tensor(np.sort(rng.choice(mesh.n, 4096, replace=False)).astype(np.int32),
                          device=cuda)
    o0 = out[0].contiguous()
    ref = dev.direct(x, y, z, vals[0].contiguous(), x, y, z, vals[0].contiguous(), w, wl["kernel"],
                     wl["kparams"][0], wl["singularity"], subset=sub)
    rel = float(torch.linalg.norm(o0[sub.long()] - ref) / torch.linalg.norm(ref))

    # roofline of the dominant field kernel
    # the ordinary near pass processes the near pairs outside close ranges
    pairs_near = (info["near_pairs"] - info["near_close_pairs"]) * norb
    pairs_far = info["far_pairs"] * norb
    near_ms = prof_ms[3] / max(prof_n[3], 1)
    far_ms = prof_ms[4] / max(prof_n[4], 1)
    dominant = "near" if near_ms >= far_ms else "far"
    k_ms = near_ms if dominant == "near" else far_ms
    k_pairs = pairs_near if dominant == "near" else pairs_far
    achieved = k_pairs / (k_ms * 1e-3)
    peak = ctypes.c_double()
    kp0 = float(wl["kparams"][0][0])
    nat.check(L.tagi_pair_peak(int(wl["kernel"]), int(wl["singularity"]),
                               0 if dominant == "near" else 1, kp0, ctypes.byref(peak),
                               ctypes.c_void_p(stream.cuda_stream)))
    traffic = profile_traffic(dominant, wl["label"])
    roofline = {"bound": "mufu", "achieved": achieved / 1e9, "peak": peak.value / 1e9,
                "unit": "Gpair/s", "frac": achieved / peak.value, "traffic": traffic,
                "kernel": f"{dominant}_mixed ({wl['label']})",
                "peak_source": "tagi_pair_peak: same pair arithmetic, operands in shared "
                               "memory/registers, measured live on this GPU",
                "kernel_ms_per_launch": k_ms, "pairs_per_launch": k_pairs,
                "fp32_tflops": achieved * PAIR_FLOPS[wl["label"]] / 1e12}

    # end to end through the C ABI with pinned host buffers
    pinned = [torch.empty(mesh.n, dtype=torch.float64, pin_memory=True) for _ in range(9)]
    for p_, a_ in zip(pinned, (mesh.x, mesh.y, mesh.z, wl["values"][0], mesh.x, mesh.y, mesh.z,
                               wl["values"][0], mesh.w)):
        p_.numpy()[:] = a_
    hout = torch.empty(mesh.n, dtype=torch.float64, pin_memory=True)
    hp = [nat.dptr(p_.numpy()) for p_ in pinned]
    kpar = np.ascontiguousarray(wl["kparams"][0], dtype=np.float64)

    def e2e_call():
        return L.tagi_BaryTreeInterface_ex(mesh.n, mesh.n, *hp, nat.dptr(hout.numpy()),
                                           int(wl["kernel"]), len(kpar), nat.dptr(kpar),
                                           int(wl["singularity"]), 1, 1, THETA, DEGREE, sl, tl,
                                           1.0, -1.0, 0, nat.PREC_MIXED)
    nat.check(e2e_call())
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        nat.check(e2e_call())
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": 1.0 / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 9 * 8 * mesh.n,
           "d2h_bytes_per_step": 8 * mesh.n, "path": "tagi_BaryTreeInterface_ex (C ABI, host buffers)",
           "note": "per step one single-charge-vector call"}

    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        threads = os.cpu_count() or 1
        secs, cinfo = cpu_treecode_sample(wl, args.cpu_seconds, threads)
        cpu = {"value": norb / secs if args.workload == "hartree" else 1.0 / secs, "unit": UNIT,
               "cores": threads, "kind": "port",
               "sample": (f"FP64 treecode restatement on {cinfo['batches']} of {cinfo['of_batches']} "
                          f"target batches ({cinfo['pair_fraction']:.4f} of the pairs), plan and "
                          "upward pass timed in full, fields extrapolated by pair count")}

    clk = clocks.summary()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded mesh and densities)",
        "config": {"workload": wl["desc"], "points": int(mesh.n), "orbitals": int(norb),
                   "theta": THETA, "degree": DEGREE, "leaf": [sl, tl], "precision": "mixed",
                   "step": "plan (tree, lists, weight charges) + convolution, inputs in HBM",
                   "l2": "256 MB buffer written between timed steps (untimed)",
                   "parallelism": f"replicas x{ws} (independent convolutions, no collective)",
                   "rel_l2_vs_fp64_direct": rel, "rel_l2_sample_targets": 4096,
                   "pairs_per_conv": info["near_pairs"] + info["far_pairs"],
                   "near_pairs": info["near_pairs"], "far_pairs": info["far_pairs"],
                   "near_close_pairs": info["near_close_pairs"]},
        "phase_ms_per_step": {k: float(v) / args.steps for k, v in zip(
            ("tree", "lists", "upward", "near", "far", "glue", "near_close"), prof_ms)},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
        "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# Uneven multi-system batch: one persistent launch per pass, CUDA graph
# ---------------------------------------------------------------------------
UNEVEN_LEAVES = ((1000, 1000), (2000, 1000), (2000, 2000), (4000, 2000))
PLAIN_LEAF = 500  # 500-point leaves, the tree parameters the reference's single-atom runs use


def uneven_arm(args):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    pkg = importlib.import_module(PKG)
    dev = importlib.import_module(PKG + ".device")
    tune = importlib.import_module(PKG + ".autotune")
    nat = pkg._native
    L = nat.lib()
    BT = pkg.BaryTreeInterface
    K, SS = BT.Kernel.YUKAWA, BT.Singularity.SUBTRACTION
    cuda = torch.device("cuda", local)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=cuda)
    systems = pkg.synthetic.uneven_systems(seed=4)
    meshes = [(t(m.x), t(m.y), t(m.z), t(m.w)) for m, _, _ in systems]
    vals = [t(F) for _, F, _ in systems]
    ks = [np.asarray(k, dtype=np.float64) for _, _, k in systems]
    norbs = [int(F.shape[0]) for _, F, _ in systems]
    npts = [int(m.n) for m, _, _ in systems]

    # autotuner (untimed): leaves per system, joint kernel shape
    t0 = time.perf_counter()
    tuned = tune.tune_systems(meshes, vals, ks, K, SS, precision="mixed", theta=THETA, degree=DEGREE,
                              leaves=UNEVEN_LEAVES, reuse=50, tol=1e-6, sample_orbitals=4)
    tune_s = time.perf_counter() - t0
    plans = [dev.TreecodePlan.for_mesh(*mesh, theta=THETA, degree=DEGREE, source_leaf=sl, target_leaf=tl)
             for mesh, (sl, tl) in zip(meshes, tuned["leaves"])]
    S = dev.Systems(plans, norbs, K, precision="mixed", orbitals_per_item=tuned["orbitals_per_item"],
                    targets_per_thread=tuned["targets_per_thread"])
    kdev = [t(k) for k in ks]
    outs = [torch.empty_like(v) for v in vals]
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        S.convolve(vals, vals, kdev, SS, outs=outs, stream=stream)  # uncaptured first call
        with dev.Graph.capture(stream) as graph:
            S.convolve(vals, vals, kdev, SS, outs=outs, stream=stream)
        for _ in range(args.warmup):
            graph.replay(stream)
        stream.synchronize()
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=cuda)  # 256 MB > L2
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with ClockSampler(local) as clocks:
            if ws > 1:
                dist.barrier()
            torch.cuda.synchronize()
            n0 = L.tagi_launch_count()
            for k in range(args.steps):
                flush.zero_()
                evs[k][0].record(stream)
                graph.replay(stream)
                evs[k][1].record(stream)
            torch.cuda.synchronize()
            if ws > 1:
                dist.barrier()
    n_nodes = graph.nodes()
    # launches inside the timed region: every replay runs the captured kernels
    launches_per_replay = None
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = job_time_ms(float(sum(step_ms)), cuda)
    orb_total = sum(norbs)
    value = job_value(orb_total, args.steps, ws, total_ms)
    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return 0

    # per-pass device times from one profiled uncaptured call
    L.tagi_profile(1)
    prof_ms = np.zeros(7)
    prof_n = np.zeros(7, dtype=np.int64)
    prof_np = prof_n.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
    L.tagi_profile_read(nat.dptr(prof_ms), prof_np, 7)
    c0 = L.tagi_launch_count()
    S.convolve(vals, vals, kdev, SS, outs=outs)
    torch.cuda.synchronize()
    launches_per_replay = int(L.tagi_launch_count() - c0)
    L.tagi_profile_read(nat.dptr(prof_ms), prof_np, 7)
    L.tagi_profile(0)

    # accuracy: first and last orbital of every system at 1024 seeded targets vs FP64 direct sum
    rng = np.random.default_rng(99)
    errs = []
    for (x, y, z, w), v, k, o, n in zip(meshes, vals, ks, outs, npts):
        sub = torch.as_tensor(np.sort(rng.choice(n, min(1024, n), replace=False)).astype(np.int32), device=cuda)
        for j in (0, v.shape[0] - 1):
            vj = v[j].contiguous()
            ref = dev.direct(x, y, z, vj, x, y, z, vj, w, K, [k[j]], SS, subset=sub)
            errs.append(float(torch.linalg.norm(o[j][sub.long()] - ref) / torch.linalg.norm(ref)))

    # pair counts and roofline of the dominant pass (near, orbital groups)
    infos = [p.info() for p in plans]
    pairs_near = sum((i["near_pairs"] - i["near_close_pairs"]) * no for i, no in zip(infos, norbs))
    pairs_far = sum(i["far_pairs"] * no for i, no in zip(infos, norbs))
    pairs_all = sum((i["near_pairs"] + i["far_pairs"]) * no for i, no in zip(infos, norbs))
    near_ms, far_ms = prof_ms[3], prof_ms[4]
    og = S.info()["orbitals_per_item"]
    peak = ctypes.c_double()
    nat.check(L.tagi_pair_peak(int(K), int(SS), 2 if og > 1 else 0, 1.0, ctypes.byref(peak),
                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    achieved = pairs_near / (near_ms * 1e-3)
    roofline = {"bound": "mufu", "achieved": achieved / 1e9, "peak": peak.value / 1e9, "unit": "Gpair/s",
                "frac": achieved / peak.value, "traffic": None,
                "kernel": f"near_group<OG={og}> over all systems" if og > 1 else "near_mixed over all systems",
                "peak_source": "tagi_pair_peak variant 2 (orbital-group near loop, 8 orbitals per pair "
                               "geometry), measured live on this GPU" if og > 1 else "tagi_pair_peak variant 0",
                "kernel_ms_per_launch": near_ms, "pairs_per_launch": pairs_near,
                "far_ms_per_launch": far_ms, "far_pairs_per_launch": pairs_far}

    # plain path: one FP64 tagi_treecode_dev call per orbital (tree + convolution), leaves 500
    plain = []
    for i in range(min(args.fp64_sample_systems, len(systems))):
        x, y, z, w = meshes[i]
        v0 = vals[i][0].contiguous()
        torch.cuda.synchronize()
        a = time.perf_counter()
        dev.treecode(x, y, z, v0, x, y, z, v0, w, K, [ks[i][0]], SS, THETA, DEGREE, PLAIN_LEAF, PLAIN_LEAF,
                     precision="fp64")
        torch.cuda.synchronize()
        plain.append(time.perf_counter() - a)
    # pair counts of the plain trees (plan only) to extend the measured FP64 rate to every system
    plain_pairs = []
    for mesh in meshes:
        p = dev.TreecodePlan.for_mesh(*mesh, theta=THETA, degree=DEGREE, source_leaf=PLAIN_LEAF,
                                      target_leaf=PLAIN_LEAF)
        inf = p.info()
        plain_pairs.append(inf["near_pairs"] + inf["far_pairs"])
        p.close()
    rate64 = sum(plain_pairs[:len(plain)]) / sum(plain)
    plain_s = sum(no * (plain[i] if i < len(plain) else plain_pairs[i] / rate64)
                  for i, no in enumerate(norbs))
    plain_value = orb_total / plain_s

    # end to end: host arrays -> tagi_treecode_batched (plans, tuned leaves per call) -> host
    off = np.concatenate([[0], np.cumsum(npts)]).astype(np.int32)
    hx, hy, hz, hw = (torch.as_tensor(np.concatenate([getattr(m, a) for m, _, _ in systems])).pin_memory()
                      for a in "xyzw")
    hv = torch.as_tensor(np.concatenate([F.reshape(-1) for _, F, _ in systems])).pin_memory()
    kall = np.concatenate(ks)
    hout = torch.empty_like(hv).pin_memory()
    sl_e, tl_e = tuned["leaves"][-1]  # the largest system's leaves (one leaf setting per one-shot call)
    torch.cuda.synchronize()
    a = time.perf_counter()
    dx, dy, dz, dw, dv = (h.to(cuda, non_blocking=True) for h in (hx, hy, hz, hw, hv))
    dout = dev.treecode_batched(off, norbs, dx, dy, dz, dw, dv, K, kall, SS, theta=THETA, degree=DEGREE,
                                source_leaf=sl_e, target_leaf=tl_e, precision="mixed")
    hout.copy_(dout, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - a
    e2e = {"value": orb_total / e2e_s, "unit": "orbital convolutions/s",
           "h2d_bytes_per_step": int(8 * (4 * off[-1] + hv.numel())), "d2h_bytes_per_step": int(8 * hout.numel()),
           "path": "tagi_treecode_batched (one-shot: plans built inside the call), pinned host buffers"}

    cpu = None
    if not args.no_cpu_baseline and ws == 1:
        threads = os.cpu_count() or 1
        i = 2  # 300k-point system: CPU FP64 pair rate on a sample of its batches
        m, F, k = systems[i]
        wl = dict(mesh=m, values=F, kparams=k[:, None], kernel=K, singularity=SS)
        secs, cinfo = cpu_treecode_sample(wl, args.cpu_seconds, threads, leaf=tuned["leaves"][i])
        rate = cinfo["pairs_per_s"]
        cpu_s = sum(no * (i_["near_pairs"] + i_["far_pairs"]) / rate for i_, no in zip(infos, norbs))
        cpu = {"value": orb_total / cpu_s, "unit": "orbital convolutions/s", "cores": threads, "kind": "port",
               "sample": (f"FP64 treecode restatement on {cinfo['batches']} of {cinfo['of_batches']} batches "
                          f"of the {m.n}-point system (one orbital); its pair rate "
                          f"{rate:.3g}/s applied to all {orb_total} orbital convolutions' pair counts")}

    clk = clocks.summary()
    line = {
        "metric": METRIC, "value": value, "unit": "orbital convolutions/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded meshes and orbitals)",
        "config": {"workload": "uneven_6_systems_yukawa_ss", "points": npts, "orbitals": norbs,
                   "theta": THETA, "degree": DEGREE, "precision": "mixed",
                   "step": "one CUDA-graph replay: all orbitals of all systems, one persistent launch per field "
                           "pass; plans reused",
                   "graph_nodes": n_nodes, "l2": "256 MB buffer written between timed steps (untimed)",
                   "autotune": {"leaves": tuned["leaves"], "orbitals_per_item": tuned["orbitals_per_item"],
                                "targets_per_thread": tuned["targets_per_thread"], "seconds": tune_s,
                                "joint": tuned["joint"]},
                   "rel_l2_vs_fp64_direct_max": max(errs), "rel_l2_checks": len(errs),
                   "pairs_per_step": pairs_all},
        "phase_ms_uncaptured_call": {k_: float(v_) for k_, v_ in zip(
            ("tree", "lists", "upward", "near", "far", "glue", "near_close"), prof_ms)},
        "plain_fp64_one_call_per_orbital": {
            "value": plain_value, "unit": "orbital convolutions/s",
            "measured_systems": len(plain), "seconds_per_orbital_measured": plain,
            "fp64_pairs_per_s": rate64, "speedup_of_batched": value / plain_value,
            "note": "systems beyond the measured ones extrapolated by their plain-tree pair counts"},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
        "gpu_launches": launches_per_replay * args.steps,
    }
    print(json.dumps(line), flush=True)
    S.close()
    for p in plans:
        p.close()
    if ws > 1:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# Ring-molecule SCF: plain Green iteration vs the learned extrapolation
# ---------------------------------------------------------------------------
def ring_guess(mesh, nuclei, charges, norb=24):
    """Atom-centred start: carbon 1s, carbon 2s, hydrogen 1s, carbon 2p_z, carbon 2p_x;
    eigenvalue guesses.  24 orbitals for 21 doubly occupied levels: the three unoccupied
    buffer orbitals keep one wayward orbital from corrupting the density."""
    funcs, eps = [], []
    for kind in ("c1s", "c2s", "h1s", "c2pz", "c2px"):
        for R, z in zip(nuclei, charges):
            dx, dy, dz = mesh.x - R[0], mesh.y - R[1], mesh.z - R[2]
            r = np.sqrt(dx * dx + dy * dy + dz * dz)
            if kind == "c1s" and z > 1:
                funcs.append(np.exp(-5.7 * r))
                eps.append(-10.0)
            elif kind == "c2s" and z > 1:
                funcs.append((1 - 0.8 * r) * np.exp(-1.6 * r))
                eps.append(-0.7)
            elif kind == "h1s" and z == 1:
                funcs.append(np.exp(-r))
                eps.append(-0.5)
            elif kind == "c2pz" and z > 1:
                funcs.append(dz * np.exp(-1.6 * r))
                eps.append(-0.4)
            elif kind == "c2px" and z > 1:
                funcs.append(dx * np.exp(-1.6 * r))
                eps.append(-0.3)
    return np.stack(funcs[:norb]), np.array(eps[:norb])


def scf_arm(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if rank != 0:
        return 0
    pkg = importlib.import_module(PKG)
    scf_mod = importlib.import_module(PKG + ".scf")
    learned = importlib.import_module(PKG + ".learned")
    L = pkg._native.lib()
    nuclei, charges = pkg.synthetic.ring_molecule()
    t0 = time.perf_counter()
    mesh = pkg.synthetic.mesh_with_points(nuclei, charges, 7, 8, args.scf_points)
    mesh_s = time.perf_counter() - t0
    psi0, eps0 = ring_guess(mesh, nuclei, charges, args.scf_orbitals)
    gauge = -0.5
    runs = {}
    for name in ("plain", "learned"):
        ex = learned.LearnedExtrapolator(512, rollout=8) if name == "learned" else None
        torch.cuda.synchronize()
        n0 = L.tagi_launch_count()
        with ClockSampler(local) as clocks:
            a = time.perf_counter()
            s = scf_mod.SCF(mesh.x, mesh.y, mesh.z, mesh.w, nuclei, charges, psi0, eps0 + gauge, 42.0,
                            gauge_shift=gauge, mixing=args.scf_mixing, source_leaf=2000, target_leaf=2000,
                            extrapolator=ex)
            out = s.run(tol=1e-5, max_scf=args.scf_max_iter, time_limit=args.scf_time_limit)
            wall = time.perf_counter() - a
        runs[name] = dict(converged=out["converged"], seconds=wall, scf_iterations=out["iterations"],
                          sweeps=(ex.stats["sweeps"] if ex else out["sweeps"]), Etotal=out["Etotal"],
                          eigenvalues=out["eigenvalues"], launches=int(L.tagi_launch_count() - n0),
                          last_eigenvalue_change=s.history[-1]["eigenvalue_change"],
                          learned_stats=(dict(ex.stats, disabled=ex.disabled) if ex else None),
                          clocks=clocks.summary())
        s.close()
        del s
        torch.cuda.empty_cache()
    pl, le = runs["plain"], runs["learned"]
    line = {
        "metric": METRIC, "value": le["seconds"], "unit": "s to 1e-5 Ha eigenvalue change (learned)",
        "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": le["seconds"] * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic ring molecule (6 C at r=2.6, 6 H at r=4.7 Bohr), seeded mesh",
        "config": {"workload": "ring_scf_21_occupied_orbitals", "points": int(mesh.n), "orbitals": int(len(eps0)),
                   "occupied": 21, "electrons": 42,
                   "theta": THETA, "degree": DEGREE, "leaf": [2000, 2000], "precision": "mixed",
                   "exchange": "Slater (LDA, no correlation)", "orbital_mixing": "Anderson, history 5",
                   "density_mixing": f"Anderson, history 10, beta {args.scf_mixing}", "mesh_build_s": mesh_s,
                   "step": "one full SCF run from the atom-centred guess"},
        "plain": pl, "learned": le, "speedup_learned_vs_plain": pl["seconds"] / le["seconds"],
        "clocks": le["clocks"], "gpu_launches": le["launches"],
    }
    print(json.dumps(line), flush=True)
    return 0


# Two-level mesh of the ring molecule by the reference's coarsenedUniformTwoLevel
# rule: domain [-20, 20]^3, base cells of side 5, order 7, near spacing h = 1,
# far spacing H = 5, ball radius r = 2, level -2 (8 fine children per cell
# within 1.5 r of a nucleus): 5,104 cells, 2.61M coarse + 14.3M fine points.
MESH_CFG = dict(XL=20.0, max_side=5.0, order=7, h=1.0, H=5.0, r=2.0, level=-2.0)


def mesh_arm(args):
    """Device mesh generation (tagi_mesh_refine + tagi_mesh_points).  value =
    mesh points (coarse + fine) generated per second with the base cells and
    nuclei already on the device; e2e = the same through mesh.build_mesh from
    host parameters with every mesh array read back to the host."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    pkg = importlib.import_module(PKG)
    M = importlib.import_module(PKG + ".mesh")
    L = pkg._native.lib()
    c = MESH_CFG
    nuclei, _ = pkg.synthetic.ring_molecule()
    order = c["order"]
    base = M.base_cells(c["XL"], c["XL"], c["XL"], c["max_side"])
    tables = M.unit_tables(order)
    base_d = torch.as_tensor(base, device="cuda")
    atoms_d = torch.as_tensor(np.ascontiguousarray(nuclei, np.float64), device="cuda")
    stream = torch.cuda.Stream()

    def step():
        cells, ppc_c, ppc_f, nfine = M.refine_cells(base_d, atoms_d, order, c["h"], c["H"], c["r"], c["level"],
                                                    stream=stream)
        C, F = M.mesh_points(cells, ppc_f, order, nfine, tables, stream=stream)
        return cells, ppc_f, C, F

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            out = step()
        ncell, nc, nf = out[0][0].numel(), out[2][0].numel(), out[3][0].numel()
        # the points pass alone (coarse + fine kernels), CUDA events on its stream
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        pts_ms = []
        for _ in range(5):
            ev[0].record(stream)
            M.mesh_points(out[0], out[1], order, nf, tables, stream=stream)
            ev[1].record(stream)
            stream.synchronize()
            pts_ms.append(ev[0].elapsed_time(ev[1]))
        del out
        torch.cuda.synchronize()
        n0 = L.tagi_launch_count()
        with ClockSampler(local) as clocks:
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(args.steps):
                out = step()
                del out
            t1.record(stream)
            stream.synchronize()
        total_ms = t0.elapsed_time(t1)
        launches = int(L.tagi_launch_count() - n0)
    pts = nc + nf
    ms = total_ms / args.steps
    # e2e: host parameters in, every mesh array back on the host
    e2e_ms = []
    d2h = 0
    for _ in range(args.steps):
        a = time.perf_counter()
        m = M.build_mesh(c["XL"], c["max_side"], nuclei, order, c["h"], c["H"], c["r"], c["level"],
                         tables=tables)
        host = [t.cpu() for t in (m.X, m.Y, m.Z, m.W, m.Xf, m.Yf, m.Zf, m.Wf, m.cellX, m.cellY, m.cellZ,
                                  m.cellDX, m.cellDY, m.cellDZ, m.PtsPerCellCoarse, m.PtsPerCellFine)]
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - a) * 1e3)
        d2h = sum(h.numel() * h.element_size() for h in host)
        del m, host
    pts_med = statistics.median(pts_ms)
    alg_bytes = 32 * pts + 56 * ncell
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs") or 6800.0
    achieved = alg_bytes / (pts_med * 1e-3) / 1e9
    line = {"metric": "mesh points/s (two-level first-kind mesh, refinement + points)",
            "value": pts / (ms * 1e-3), "unit": "points/s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic ring molecule (12 nuclei), seeded",
            "config": {"workload": "ring_two_level_mesh", **c, "cells": int(ncell), "coarse_points": int(nc),
                       "fine_points": int(nf), "l2": "outputs (541 MB) larger than L2"},
            "roofline": {"bound": "hbm", "kernel": "points pass (mesh_coarse_points + mesh_fine_points)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "bytes_per_launch": alg_bytes, "ms": pts_med,
                         "peak_source": "measured" if "hbm_gbs" in peaks else "fallback"},
            "e2e": {"value": pts / (statistics.median(e2e_ms) * 1e-3), "unit": "points/s",
                    "h2d_bytes_per_step": int(base.nbytes + nuclei.nbytes), "d2h_bytes_per_step": int(d2h)},
            "clocks": clocks.summary(), "gpu_launches": launches}
    if not args.no_cpu_baseline:
        from oracle import mesh_oracle as MO
        a = time.perf_counter()
        lv = MO.refine(base, nuclei, c["h"], c["H"], c["r"], c["level"])
        tab = MO.cell_table(lv, order)
        MO.points(tab, order, *tables)
        secs = time.perf_counter() - a
        line["cpu_baseline"] = {"value": pts / secs, "unit": "points/s", "cores": 1, "kind": "port",
                                "sample": "the whole mesh by the oracle's restatement (Python recursion, "
                                          "numpy per cell)"}
    print(json.dumps(line), flush=True)
    return 0


def cpu_two_mesh_sample(tab, pts, nuclei, target_seconds, threads):
    """Oracle cost of one orbital's two-mesh correction on a mesh: the FP64
    plan (coarse targets, fine sources, theta 0.55, degree 9) and upward pass
    timed in full, the Yukawa field on a sample of target batches sized to
    ~target_seconds, extrapolated by pair count.  Returns (seconds, info)."""
    from oracle import oracle as O
    O.build()
    X, Y, Z, W, Xf, Yf, Zf, Wf = pts
    t0 = time.perf_counter()
    plan = O.Plan(X, Y, Z, Xf, Yf, Zf, Wf, THETA - 0.15, DEGREE + 2, 2000, 2000, 1.0)
    t_plan = time.perf_counter() - t0
    L_ = plan.lists()
    st, tt = plan.tree(0), plan.tree(1)
    nb = plan.n_batches
    bsz = tt["end"][L_["batch_node"]] - tt["begin"][L_["batch_node"]]
    src_len = st["end"] - st["begin"]
    ncnt = np.array([src_len[L_["near_list"][L_["near_off"][b]:L_["near_off"][b + 1]]].sum() for b in range(nb)])
    pairs_b = bsz * (ncnt + np.diff(L_["far_off"]) * plan.P)
    R = nuclei[0]
    fc = np.exp(-np.sqrt((X - R[0]) ** 2 + (Y - R[1]) ** 2 + (Z - R[2]) ** 2))
    ff = np.exp(-np.sqrt((Xf - R[0]) ** 2 + (Yf - R[1]) ** 2 + (Zf - R[2]) ** 2))
    order = np.random.default_rng(17).permutation(nb)
    sel = np.sort(order[:4])
    _, (t_up, t_f), (pn, pf) = O.convolve_batches(plan, fc, ff, Wf, 2, [1.0], 2, sel, threads)
    want = (pn + pf) / max(t_f, 1e-9) * target_seconds
    nsel = int(np.clip(np.searchsorted(np.cumsum(pairs_b[order]), want) + 1, 4, nb))
    sel = np.sort(order[:nsel])
    _, (t_up, t_f), (pn, pf) = O.convolve_batches(plan, fc, ff, Wf, 2, [1.0], 2, sel, threads)
    frac = (pn + pf) / pairs_b.sum()
    return t_plan + t_up + t_f / frac, dict(plan_s=t_plan, upward_s=t_up, batches=nsel, of_batches=nb,
                                            pair_fraction=float(frac), pairs_per_s=(pn + pf) / t_f)


def twomesh_arm(args):
    """Two-mesh eigenvalue correction (twomesh.TwoMeshCorrection) of the ring
    molecule's 21 atom-centred orbitals on its device-built two-level mesh
    (MESH_CFG: 2.61M coarse, 14.3M fine points).  One step = one whole
    correction: interpolations, the Hartree convolution and the 21 Yukawa
    convolutions (one batched launch per field pass) with coarse targets and
    fine sources at theta 0.55, degree 9, exchange, Harrison update; the plan
    is built once (untimed), as the reference's correction reuses one tree
    per call.  value = orbitals corrected per second."""
    import torch
    from types import SimpleNamespace
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    pkg = importlib.import_module(PKG)
    M = importlib.import_module(PKG + ".mesh")
    T = importlib.import_module(PKG + ".twomesh")
    nat = pkg._native
    L = nat.lib()
    c = MESH_CFG
    nuclei, charges = pkg.synthetic.ring_molecule()

    def setup(h):
        m = M.build_mesh(c["XL"], c["max_side"], nuclei, c["order"], h, c["H"], c["r"], c["level"])
        hx = SimpleNamespace(x=m.X.cpu().numpy(), y=m.Y.cpu().numpy(), z=m.Z.cpu().numpy())
        psi, eps = ring_guess(hx, nuclei, charges, 21)
        w = m.W.cpu().numpy()
        psi /= np.sqrt((psi * psi * w).sum(1))[:, None]
        rho = 2.0 * (psi * psi).sum(0)
        corr = T.TwoMeshCorrection(m.X, m.Y, m.Z, m.W, m.Xf, m.Yf, m.Zf, m.Wf, m.PtsPerCellCoarse,
                                   m.PtsPerCellFine, c["order"], nuclei, charges, theta=THETA, degree=DEGREE,
                                   source_leaf=2000, target_leaf=2000, precision="mixed")
        return m, corr, psi, eps, rho

    m, corr, psi, eps, rho = setup(c["h"])
    psi_d = torch.as_tensor(psi, device="cuda")
    rho_d = torch.as_tensor(rho, device="cuda")
    for _ in range(max(args.warmup, 1)):
        out = corr.correct(psi_d, eps, rho_d, n_electrons=42.0)
    corr.stream.synchronize()
    prof_ms = np.zeros(7)
    prof_n = np.zeros(7, dtype=np.int64)
    prof_np = prof_n.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
    L.tagi_profile(1)
    L.tagi_profile_read(nat.dptr(prof_ms), prof_np, 7)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    n0 = L.tagi_launch_count()
    with ClockSampler(local) as clocks:
        ev[0].record(corr.stream)
        for _ in range(args.steps):
            out = corr.correct(psi_d, eps, rho_d, n_electrons=42.0)
        ev[1].record(corr.stream)
        corr.stream.synchronize()
    launches = int(L.tagi_launch_count() - n0)
    L.tagi_profile_read(nat.dptr(prof_ms), prof_np, 7)
    L.tagi_profile(0)
    ms = ev[0].elapsed_time(ev[1]) / args.steps
    info = corr.plan.info()
    # dominant kernel: the near field (1 Hartree + 21 Yukawa orbitals per step)
    near_pairs = (info["near_pairs"] - info["near_close_pairs"]) * 22 * args.steps
    far_pairs = info["far_pairs"] * 22 * args.steps
    dominant = "near" if prof_ms[3] >= prof_ms[4] else "far"
    k_ms = prof_ms[3] if dominant == "near" else prof_ms[4]
    k_pairs = near_pairs if dominant == "near" else far_pairs
    peak = ctypes.c_double()
    # 21 of the 22 orbital-convolutions per step run in one orbital-group
    # launch (several orbitals per pair geometry): its near-loop peak is variant 2
    nat.check(L.tagi_pair_peak(2, 2, 2 if dominant == "near" else 1, 1.0, ctypes.byref(peak),
                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    achieved = k_pairs / (k_ms * 1e-3)
    # e2e: host orbitals and density in, corrected eigenvalues out
    e2e_ms = []
    for _ in range(args.steps):
        a = time.perf_counter()
        o = corr.correct(psi, eps, rho, n_electrons=42.0)
        e2e_ms.append((time.perf_counter() - a) * 1e3)
    line = {"metric": "two-mesh eigenvalue corrections/s (orbitals)", "value": 21 / (ms * 1e-3),
            "unit": "orbitals/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 1),
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic ring molecule (12 nuclei), atom-centred guess orbitals",
            "config": {"workload": "ring_two_mesh_correction_21_orbitals", "coarse_points": int(m.n),
                       "fine_points": int(m.Xf.numel()), "theta": THETA - 0.15, "degree": DEGREE + 2,
                       "leaf": [2000, 2000], "precision": "mixed",
                       "l2": "inputs (2.6M x 21 orbitals, 14.3M-point fine mesh) larger than L2",
                       "eigenvalue_corrections": [float(v) for v in out["deltaE"]]},
            "phase_ms_per_step": {k: float(prof_ms[i]) / args.steps for i, k in
                                  enumerate(("tree", "lists", "upward", "near", "far", "glue", "near_close"))},
            "roofline": {"bound": "mufu", "kernel": f"{dominant}_mixed (yukawa/coulomb ss)",
                         "achieved": achieved / 1e9, "peak": peak.value / 1e9, "unit": "Gpair/s",
                         "frac": achieved / peak.value, "traffic": None,
                         "peak_source": ("tagi_pair_peak variant 2 (orbital-group near loop, Yukawa SS), "
                                         "measured live" if dominant == "near" else
                                         "tagi_pair_peak variant 1 (far loop), measured live")},
            "e2e": {"value": 21 / (statistics.median(e2e_ms) * 1e-3), "unit": "orbitals/s",
                    "h2d_bytes_per_step": int(psi.nbytes + rho.nbytes), "d2h_bytes_per_step": 8 * 21},
            "clocks": clocks.summary(), "gpu_launches": launches}
    corr.close()
    del corr, psi_d, rho_d, out, m
    torch.cuda.empty_cache()
    if not args.no_cpu_baseline:
        # same construction at h = 3 (320k coarse / 721k fine points): GPU and oracle side by side
        hs = 3.0
        ms_small, corr_s, psi_s, eps_s, rho_s = setup(hs)
        corr_s.correct(psi_s, eps_s, rho_s)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(corr_s.stream)
        corr_s.correct(psi_s, eps_s, rho_s)
        b.record(corr_s.stream)
        corr_s.stream.synchronize()
        gpu_small = 21 / (a.elapsed_time(b) * 1e-3)
        from oracle import mesh_oracle as MO
        tab, pts = MO.build(c["XL"], c["max_side"], nuclei, c["order"], hs, c["H"], c["r"], c["level"])
        threads = os.cpu_count() or 1
        secs, inf = cpu_two_mesh_sample(tab, pts, nuclei, args.cpu_seconds, threads)
        line["cpu_baseline"] = {
            "value": 1.0 / secs, "unit": "orbitals/s", "cores": threads, "kind": "port",
            "sample": (f"oracle FP64 correction of one orbital on the same construction at h = {hs} "
                       f"({len(pts[0])} coarse / {len(pts[4])} fine points): plan + upward timed in full, "
                       f"Yukawa field on {inf['batches']} of {inf['of_batches']} batches "
                       f"({inf['pair_fraction']:.3f} of the pairs), extrapolated by pair count"),
            "gpu_same_mesh_orbitals_per_s": gpu_small}
        corr_s.close()
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "mesh":
        return mesh_arm(args)
    if args.workload == "twomesh":
        return twomesh_arm(args)
    if args.workload == "uneven":
        return uneven_arm(args)
    if args.workload == "scf":
        return scf_arm(args)
    return gb300_arm(args)


if __name__ == "__main__":
    sys.exit(main())
