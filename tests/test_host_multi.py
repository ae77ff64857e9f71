"""Host-side logic that needs no GPU: the replica timing of bench.py across two
gloo ranks, Fermi occupations, the BF16 rounding the network oracle uses, the
autotuner's cache, the Anderson restatement."""
import importlib
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import PKG, ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    local = [120.0, 95.0][rank]  # the ranks' own timed regions
    total = bench.job_time_ms(local, None)
    value = bench.job_value(3, 5, world, total)
    q.put((rank, total, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total, value in out:
        assert total == 120.0  # MAX over ranks
        assert value == pytest.approx(3 * 5 * 2 / 0.120)


def test_single_process_job_time_is_local():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_time_ms(42.0) == 42.0
    assert bench.job_value(1, 4, 1, 500.0) == pytest.approx(8.0)


def test_fermi_occupations():
    scf = importlib.import_module(PKG + ".scf")
    eps = np.array([-10.0, -1.0, -0.5, -0.3, 0.2])
    occ, ef = scf.fermi_occupations(eps, 6.0)
    assert occ.sum() == pytest.approx(6.0, abs=1e-9)
    assert np.all(np.diff(occ) <= 0) and occ[0] == pytest.approx(2.0)
    assert -0.5 < ef < -0.3  # three doubly occupied levels at 300 K
    with pytest.raises(ValueError):
        scf.fermi_occupations(eps[:2], 6.0)


def test_nuclear_repulsion():
    scf = importlib.import_module(PKG + ".scf")
    assert scf.nuclear_repulsion([[0, 0, 0], [0, 0, 2.0]], [1.0, 3.0]) == pytest.approx(1.5)


def test_bf16_rounding_matches_torch(oracle):
    from oracle import mlp_oracle
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(10000).astype(np.float32) * 10.0 ** rng.integers(-20, 20, 10000),
                        np.array([1.0, -2.5, 1e-30, 3.0e38], np.float32)]).astype(np.float32)
    ref = torch.as_tensor(x).to(torch.bfloat16).float().numpy()
    assert np.array_equal(mlp_oracle.bf16(x), ref)


def test_autotune_cache_round_trip(tmp_path):
    at = importlib.import_module(PKG + ".autotune")
    path = str(tmp_path / "sub" / "cache.json")
    assert at._load(path) == {}
    at._store(path, {"k": {"source_leaf": 2000}})
    assert at._load(path) == {"k": {"source_leaf": 2000}}
    with open(path, "w") as f:
        f.write("not json")
    assert at._load(path) == {}


def test_anderson_restatement_two_rows(oracle):
    """With two rows the Anderson weight minimizes |F_1 + c (F_0 - F_1)|_W."""
    from oracle import gi_oracle
    rng = np.random.default_rng(3)
    n = 50
    w = rng.uniform(0.5, 1.5, n)
    rin = [rng.standard_normal(n), rng.standard_normal(n)]
    rout = [rng.standard_normal(n), rng.standard_normal(n)]
    F0, F1 = rout[0] - rin[0], rout[1] - rin[1]
    d = F1 - F0
    c = np.sum(d * F1 * w) / np.sum(d * d * w)
    expect_in = rin[1] + c * (rin[0] - rin[1])
    expect_out = rout[1] + c * (rout[0] - rout[1])
    got = gi_oracle.anderson(rin, rout, w, 0.5)
    assert np.allclose(got, 0.5 * expect_out + 0.5 * expect_in)
