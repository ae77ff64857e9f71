"""The learned extrapolator's kernels against the CPU restatement
(oracle/mlp_oracle.py).

GEMM: BF16 operands, FP32 accumulation vs FP64 accumulation of the same BF16
values: relative L2 <= 1e-5.  Forward and backward of the whole network:
intermediates are BF16 on both sides (a rare one-ulp flip near a rounding tie
can differ), gradients relative L2 <= 2e-3.
"""
import ctypes
import importlib

import numpy as np
import pytest
import torch

from conftest import PKG, rel_l2

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


@pytest.fixture(scope="module")
def L(native):
    return native.lib()


@pytest.fixture(scope="module")
def mo():
    from oracle import mlp_oracle
    return mlp_oracle


def _bf(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32)).to(torch.bfloat16).cuda()


@pytest.mark.parametrize("M,N,K,ta,tb", [(70, 45, 100, False, False), (129, 64, 33, True, False),
                                         (64, 130, 257, False, True), (300, 17, 64, True, True)])
def test_gemm_matches_numpy(L, native, mo, M, N, K, ta, tb):
    rng = np.random.default_rng(M + N + K)
    A = mo.bf16(rng.standard_normal((M, K)).astype(np.float32))
    B = mo.bf16(rng.standard_normal((K, N)).astype(np.float32))
    At = _bf(A.T if ta else A)
    Bt = _bf(B.T if tb else B)
    sAm, sAk = (1, M) if ta else (K, 1)
    sBk, sBn = (1, K) if tb else (N, 1)
    C = torch.zeros(M, N, dtype=torch.float32, device="cuda")
    native.check(L.tagi_mlp_gemm(_p(At), sAm, sAk, _p(Bt), sBk, sBn, M, N, K, 0, _p(C), None, N, None, None, None))
    ref = A.astype(np.float64) @ B.astype(np.float64)
    assert rel_l2(C.cpu().numpy(), ref) <= 1e-5
    part = torch.zeros(8 * M * N, dtype=torch.float32, device="cuda")
    C2 = torch.zeros_like(C)
    native.check(L.tagi_mlp_gemm_splitk(_p(At), sAm, sAk, _p(Bt), sBk, sBn, M, N, K, 4, _p(part), _p(C2), None))
    assert rel_l2(C2.cpu().numpy(), ref) <= 1e-5
    # epilogues: bias + relu to bf16, mask to bf16, bias to f32
    bias = torch.as_tensor(rng.standard_normal(N).astype(np.float32), device="cuda")
    H = torch.zeros(M, N, dtype=torch.bfloat16, device="cuda")
    native.check(L.tagi_mlp_gemm(_p(At), sAm, sAk, _p(Bt), sBk, sBn, M, N, K, 1, None, _p(H), N, _p(bias), None,
                                 None))
    refh = mo.bf16(np.maximum(ref + bias.cpu().numpy(), 0).astype(np.float32))
    assert rel_l2(H.float().cpu().numpy(), refh) <= 1e-2
    Mk = torch.zeros(M, N, dtype=torch.bfloat16, device="cuda")
    native.check(L.tagi_mlp_gemm(_p(At), sAm, sAk, _p(Bt), sBk, sBn, M, N, K, 2, None, _p(Mk), N, None, _p(H), None))
    refm = mo.bf16((ref * (refh > 0)).astype(np.float32))
    assert rel_l2(Mk.float().cpu().numpy(), refm) <= 1e-2


def test_forward_backward_match_oracle(pkg, mo):
    learned = importlib.import_module(PKG + ".learned")
    P, rows = 64, 300
    net = learned.MLP(P, hidden=96, seed=3)
    rng = np.random.default_rng(1)
    X = mo.bf16(rng.standard_normal((rows, net.ldx)).astype(np.float32))
    X[:, net.din:] = 0
    Xt = _bf(X)
    dn = rng.standard_normal((rows, P)).astype(np.float32)
    T = (0.7 * dn + 0.1 * rng.standard_normal((rows, P))).astype(np.float32)
    # non-trivial biases so every ReLU region is exercised
    for k in ("b1", "b2", "b3"):
        net.params[k].copy_(torch.as_tensor(0.1 * rng.standard_normal(net.params[k].numel()).astype(np.float32)))
    loss = float(net.loss_and_grads(Xt, torch.as_tensor(dn).cuda(), torch.as_tensor(T).cuda(), rows))
    torch.cuda.synchronize()
    W = {k: net.half[k].float().cpu().numpy() for k in ("W1", "W2", "W3")}
    b = {k: net.params[k].cpu().numpy() for k in ("b1", "b2", "b3")}
    Y, H1, H2 = mo.forward(X, W["W1"], b["b1"], W["W2"], b["b2"], W["W3"], b["b3"])
    assert rel_l2(net.Y[:rows].cpu().numpy(), Y) <= 2e-3
    alpha = float(net.params["alpha"].item())
    l_ref, dY, dalpha = mo.mse_grad(Y, dn, T, alpha)
    assert abs(loss - l_ref) <= 2e-3 * abs(l_ref)
    assert abs(float(net.grads["alpha"].item()) - dalpha) <= 2e-3 * abs(dalpha) + 1e-9
    g = mo.backward(X, H1, H2, W["W2"], W["W3"], dY)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
        assert rel_l2(net.grads[k].cpu().numpy(), g[k]) <= 2e-3, k


def test_patch_features_match_oracle(pkg, mo):
    learned = importlib.import_module(PKG + ".learned")
    L = pkg._native.lib()
    P, ncell, norb = 27, 40, 3
    n = P * ncell
    rng = np.random.default_rng(2)
    psi = rng.standard_normal((norb, n))
    d = 1e-3 * rng.standard_normal((norb, n))
    d[1, :P] = 0.0  # a patch without an update: the floor sets its scale
    eps = np.array([-2.0, -1.0, -0.5])
    dfloor = np.array([1e-6, 2e-6, 3e-6])
    ldx = ((2 * P + 1 + 31) // 32) * 32
    X = torch.zeros(norb * ncell, ldx, dtype=torch.bfloat16, device="cuda")
    sc = torch.zeros(norb * ncell, dtype=torch.float32, device="cuda")
    dn = torch.zeros(norb * ncell, P, dtype=torch.float32, device="cuda")
    # keep the device copies referenced until the kernel has run
    psi_t, d_t, eps_t, fl_t = (torch.as_tensor(a).cuda() for a in (psi, d, eps, dfloor))
    pkg._native.check(L.tagi_mlp_patch_features(_p(psi_t), _p(d_t), _p(eps_t), _p(fl_t), norb, ncell, P, n,
                                                ldx, _p(X), _p(sc), _p(dn), None))
    torch.cuda.synchronize()
    Xr, scr, dnr = mo.patch_features(psi, d, eps, dfloor, P, ldx)
    assert rel_l2(sc.cpu().numpy(), scr) <= 1e-6
    assert rel_l2(dn.cpu().numpy(), dnr) <= 1e-6
    assert rel_l2(X.float().cpu().numpy(), Xr) <= 1e-2
    assert learned.MLP(P).ldx == ldx


def test_training_learns_a_linear_update_map(pkg):
    """Updates that shrink by a fixed factor per step: the loss falls by orders of magnitude."""
    learned = importlib.import_module(PKG + ".learned")
    P, rows = 64, 512
    net = learned.MLP(P, lr=3e-3, seed=0)
    rng = np.random.default_rng(4)
    dn = rng.standard_normal((rows, P)).astype(np.float32)
    X = np.zeros((rows, net.ldx), np.float32)
    X[:, :P] = rng.standard_normal((rows, P))
    X[:, P:2 * P] = dn
    X[:, 2 * P] = -1.0
    T = 0.8 * dn
    Xt, dnt, Tt = _bf(X), torch.as_tensor(dn).cuda(), torch.as_tensor(T).cuda()
    first = float(net.loss_and_grads(Xt, dnt, Tt, rows))
    net.adam_step()
    for _ in range(200):
        last = float(net.loss_and_grads(Xt, dnt, Tt, rows))
        net.adam_step()
    assert last < 1e-2 * first
    # the prediction alpha dn + MLP(x) reproduces the 0.8 contraction
    Y = net.forward(Xt, rows)
    pred = float(net.params["alpha"].item()) * dnt + Y
    assert float(torch.linalg.norm(pred - Tt) / torch.linalg.norm(Tt)) < 0.1
