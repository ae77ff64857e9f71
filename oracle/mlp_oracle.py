"""CPU restatement of the learned extrapolator's network (TEST INFRASTRUCTURE
ONLY: the checker of csrc/mlp.cu's forward and backward kernels).

The device rounds every GEMM operand to BF16 (round to nearest even) and
accumulates in FP32; this restatement rounds the same operands the same way
and accumulates in FP64, so the two agree to FP32 accumulation error (plus a
rare one-ulp BF16 flip of an intermediate near a rounding tie).
"""
import numpy as np


def bf16(a):
    """Round float32 values to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def forward(X, W1, b1, W2, b2, W3, b3):
    """X, W* already BF16-valued.  Returns (Y f32, H1 bf16, H2 bf16)."""
    f = np.float64
    H1 = bf16(np.maximum(X.astype(f) @ W1.T.astype(f) + b1, 0.0).astype(np.float32))
    H2 = bf16(np.maximum(H1.astype(f) @ W2.T.astype(f) + b2, 0.0).astype(np.float32))
    Y = (H2.astype(f) @ W3.T.astype(f) + b3).astype(np.float32)
    return Y, H1, H2


def mse_grad(Y, dn, T, alpha):
    rows, P = Y.shape
    r = alpha * dn.astype(np.float64) + Y - T
    g = (2.0 * r / (rows * P)).astype(np.float32)
    return float(np.sum(r * r)), g, float(np.sum(g.astype(np.float64) * dn))


def backward(X, H1, H2, W2, W3, dY):
    """Gradients of the weights and biases from dY (f32); intermediates as the device keeps them."""
    f = np.float64
    dY16 = bf16(dY)
    gW3 = dY16.T.astype(f) @ H2.astype(f)
    gb3 = dY.astype(f).sum(0)
    dH2 = bf16(((dY16.astype(f) @ W3.astype(f)) * (H2 > 0)).astype(np.float32))
    gW2 = dH2.T.astype(f) @ H1.astype(f)
    gb2 = dH2.astype(f).sum(0)
    dH1 = bf16(((dH2.astype(f) @ W2.astype(f)) * (H1 > 0)).astype(np.float32))
    gW1 = dH1.T.astype(f) @ X.astype(f)
    gb1 = dH1.astype(f).sum(0)
    return dict(W1=gW1, b1=gb1, W2=gW2, b2=gb2, W3=gW3, b3=gb3)


def patch_features(psi, d, eps, dfloor, P, ldx):
    """Rows (orbital, cell): [psi/s_psi, d/s_d, eps, 0...] with the device's scales (FP32)."""
    norb, n = psi.shape
    ncell = n // P
    rows = norb * ncell
    X = np.zeros((rows, ldx), np.float32)
    scale = np.zeros(rows, np.float32)
    dn = np.zeros((rows, P), np.float32)
    for m in range(norb):
        for c in range(ncell):
            r = m * ncell + c
            pp = psi[m, c * P:(c + 1) * P].astype(np.float32)
            dd = d[m, c * P:(c + 1) * P].astype(np.float32)
            rp = np.sqrt(np.sum(pp.astype(np.float64) ** 2) / P) + 1e-30
            rd = max(np.sqrt(np.sum(dd.astype(np.float64) ** 2) / P), float(dfloor[m])) + 1e-30
            X[r, :P] = pp / np.float32(rp)
            X[r, P:2 * P] = dd / np.float32(rd)
            X[r, 2 * P] = eps[m]
            dn[r] = dd / np.float32(rd)
            scale[r] = rd
    return bf16(X), scale, dn
