"""Host-side arithmetic of bench.py (no GPU): the pipe roofline, the operation
counts per unit, the stratified CPU sample and the fitted per-pair costs."""
import importlib
import os
import sys

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def bench():
    sys.argv = ["bench.py"]
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    return importlib.import_module("bench")


RATES = dict(ffma=3.86e13, ffma2=3.72e13, ex2=1.0e13, rsqrt=5.0e12, lg2=5.0e12, sms=152)


def test_pipe_roofline_picks_the_binding_pipe(bench):
    # Coulomb near: 9 FP32 lane ops, 1 ex2, 1 rsqrt per pair -> MUFU-bound
    r = bench.pipe_roofline(1e12, 500.0, (9.0, 1.0, 1.0, 0.0), RATES, 2070.0)
    t_mufu = 1 / 1.0e13 + 1 / 5.0e12
    assert r["bound"] == "mufu"
    assert abs(r["peak"] - 1 / t_mufu) / r["peak"] < 1e-12
    assert abs(r["frac"] - 2e12 * t_mufu) < 1e-12
    assert abs(r["pipe_frac"]["fp32"] - 2e12 * 9 / 3.86e13) < 1e-12
    # the orbital-group loop: ex2 per pair-orbital, rsqrt and lg2 per pair on MUFU
    ops = bench.field_ops("near_group", "yukawa_ss", 8, 8)
    g = bench.pipe_roofline(1e12, 500.0, ops, RATES, None)
    t_m = 1 / 1.0e13 + 0.125 / 5.0e12 + 0.125 / 5.0e12
    t_f = 4.0 / 3.86e13
    assert g["bound"] == ("mufu" if t_m > t_f else "fp32") and g["pipe_rates_per_sm_clk"] is None
    assert abs(g["peak"] - 1 / max(t_m, t_f)) / g["peak"] < 1e-12
    assert abs(g["frac"] - g["achieved"] / g["peak"]) < 1e-12


def test_field_ops_counts(bench):
    assert bench.field_ops("near_mixed", "coulomb_ss") == (9.0, 1.0, 1.0, 0.0)
    assert bench.field_ops("near_mixed", "yukawa_ss") == (10.0, 1.0, 1.0, 0.0)
    assert bench.field_ops("near_group", "yukawa_ss", 8) == (4.0, 1.0, 0.125, 0.125)
    assert bench.field_ops("far_group", "yukawa_ss", 8, 8) == (3.40625, 1.0, 0.125, 0.125)
    with pytest.raises(ValueError):
        bench.field_ops("nothing", "yukawa_ss")


def test_stratified_sample_spans_the_pair_counts(bench):
    rng = np.random.default_rng(1)
    pairs = rng.lognormal(0, 2, 500)
    sel = bench.stratified_batches(pairs, 48)
    assert len(sel) == 48 and np.all(np.diff(sel) > 0)
    assert pairs.argmax() in sel and pairs.argmin() in sel
    assert np.array_equal(sel, bench.stratified_batches(pairs, 48))   # deterministic
    assert len(bench.stratified_batches(pairs[:10], 48)) == 10


def test_cost_model_recovers_near_and_far_costs(bench):
    rng = np.random.default_rng(2)
    near, far = rng.uniform(1e6, 1e8, 40), rng.uniform(1e6, 1e8, 40)
    secs = 3e-9 * near + 1e-9 * far
    a, c = bench.cost_model(near, far, secs)
    assert abs(a - 3e-9) < 1e-15 and abs(c - 1e-9) < 1e-15
    # a fit with a negative rate falls back to one shared rate: total seconds / total pairs
    secs2 = 5e-9 * near - 1e-9 * far
    a2, c2 = bench.cost_model(near, far, secs2)
    assert a2 == c2 == pytest.approx(secs2.sum() / (near + far).sum())


def test_loop_variant_follows_the_group_size(bench):
    assert bench.loop_variant("near_mixed", 1) == 0 and bench.loop_variant("far_mixed", 1) == 1
    assert bench.loop_variant("near_group", 8) == 2 and bench.loop_variant("far_group", 8) == 3
    assert bench.loop_variant("near_group", 16) == 4 and bench.loop_variant("far_group", 16) == 5
    assert bench.loop_variant("near_group", 4) == 2
