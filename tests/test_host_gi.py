"""Host-side logic of the Green-iteration driver (no GPU): which Gram-Schmidt
entry point runs for how many orbitals, and the capture refusal above the
allocation-free limit."""
import contextlib
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG


class _FakeLib:
    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def f(*args):
            self.calls.append((name, args[3]))
            return 0
        return f


class _FakeStream:
    cuda_stream = 0
    device = "cuda:0"


@pytest.fixture()
def gi_mod(monkeypatch):
    gi = importlib.import_module(PKG + ".gi")
    fake = _FakeLib()
    monkeypatch.setattr(gi._native, "lib", lambda: fake)
    monkeypatch.setattr(gi, "_capturing", lambda s: False)
    monkeypatch.setattr(gi, "mgs_turn", lambda s: contextlib.nullcontext())
    gi._fake = fake
    return gi


@pytest.mark.parametrize("m", [1, 129, 130, 200])
def test_orthonormalize_picks_the_entry_point(gi_mod, m):
    psi = torch.zeros((m, 8), dtype=torch.float64)
    w = torch.ones(8, dtype=torch.float64)
    gi_mod.orthonormalize(psi, w, _FakeStream())
    names = {c[0] for c in gi_mod._fake.calls}
    want = "tagi_mgs_dev_noalloc" if m <= gi_mod.NOALLOC_MAX_ORBITALS else "tagi_mgs_dev"
    assert names == {want}
    assert [c[1] for c in gi_mod._fake.calls] == list(range(m))   # rows in orbital order


def test_capture_refused_above_the_limit(gi_mod):
    g = object.__new__(gi_mod.GreenIteration)
    g.norb = gi_mod.NOALLOC_MAX_ORBITALS + 1
    g._eager_sweeps = 1
    g._graph = None
    with pytest.raises(RuntimeError, match="not capturable"):
        g.capture()


def test_limit_matches_the_library(native):
    """128 earlier rows is the largest target the allocation-free entry point takes."""
    gi = importlib.import_module(PKG + ".gi")
    L = native.lib()
    assert L.tagi_mgs_dev_noalloc(None, None, None, gi.NOALLOC_MAX_ORBITALS, 10, 200, None) == native.TAGI_ERR_ARG
    L.tagi_clear_error()
