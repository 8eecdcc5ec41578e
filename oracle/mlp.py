"""CPU restatement of the learned estimator's network (TEST INFRASTRUCTURE).

Forward pass and gradients of the 32768 -> 512 -> 512 -> 1 ReLU MLP of
rayspace3d_gb300/csrc/rs_mlp.cu in float64, with BF16 rounding exactly where the GPU
rounds (inputs, W1, W2, W3 and the hidden activations before they enter a GEMM, the
backpropagated activations before the weight-gradient GEMMs).  Only tests/ use it, to
check the tensor-core kernels' outputs and gradients; it has no reference counterpart
(the reference has no learned estimator).

Also the feature pooling of rs_mlp_features.
"""
from __future__ import annotations

import numpy as np

IN, HID = 32768, 512
O_W1, O_B1 = 0, IN * HID
O_W2 = O_B1 + HID
O_B2 = O_W2 + HID * HID
O_W3 = O_B2 + HID
O_B3 = O_W3 + HID
N_PARAMS = O_B3 + 1


def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return (r.astype(np.uint32) << 16).view(np.float32)


def unpack(p: np.ndarray):
    return (p[O_W1:O_B1].reshape(HID, IN), p[O_B1:O_W2], p[O_W2:O_B2].reshape(HID, HID), p[O_B2:O_W3],
            p[O_W3:O_B3], p[O_B3:O_B3 + 1])


def forward(p: np.ndarray, X: np.ndarray):
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, np.float32))
    xh = bf16(X).astype(np.float64)
    h1 = np.maximum(xh @ bf16(W1).astype(np.float64).T + b1, 0.0)
    h1h = bf16(h1.astype(np.float32)).astype(np.float64)
    h2 = np.maximum(h1h @ bf16(W2).astype(np.float64).T + b2, 0.0)
    h2h = bf16(h2.astype(np.float32)).astype(np.float64)
    w3h = bf16(W3).astype(np.float64)
    y = h2h @ w3h + b3[0]
    return y, (xh, h1, h1h, h2, h2h, w3h)


def gradients(p: np.ndarray, X: np.ndarray, t: np.ndarray):
    """(loss, gradient vector in the parameter layout)."""
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, np.float32))
    y, (xh, h1, h1h, h2, h2h, w3h) = forward(p, X)
    B = len(t)
    dy = 2.0 * (y - t) / B
    loss = float(np.mean((y - t) ** 2))
    g = np.zeros(N_PARAMS, np.float64)
    g[O_W3:O_B3] = dy @ h2h
    g[O_B3] = dy.sum()
    d2 = np.outer(dy, w3h) * (h2 > 0)
    d2h = bf16(d2.astype(np.float32)).astype(np.float64)
    g[O_W2:O_B2] = (d2h.T @ h1h).reshape(-1)
    g[O_B2:O_W3] = d2.sum(axis=0)
    d1 = (d2h @ bf16(W2).astype(np.float64)) * (h1 > 0)
    d1h = bf16(d1.astype(np.float32)).astype(np.float64)
    g[O_W1:O_B1] = (d1h.T @ xh).reshape(-1)
    g[O_B1:O_W2] = d1.sum(axis=0)
    return loss, g


def pool(cells: np.ndarray, R: int) -> np.ndarray:
    """rs_mlp_features of one grid: 16^3 blocks x 4 channels, channel-major."""
    c = np.asarray(cells)
    cc = c["CenterCount"].astype(np.float64).reshape(R, R, R)
    tc = c["TouchCount"].astype(np.float64).reshape(R, R, R)
    sa = tc * c["AvgSizeMean"].astype(np.float64).reshape(R, R, R)
    sr = tc * c["VolRatio"].astype(np.float64).reshape(R, R, R)
    edges = [(b * R + 15) // 16 for b in range(17)]
    out = np.zeros((4, 16, 16, 16), np.float32)
    for bz in range(16):
        for by in range(16):
            for bx in range(16):
                sl = (slice(edges[bz], edges[bz + 1]), slice(edges[by], edges[by + 1]), slice(edges[bx], edges[bx + 1]))
                a, t, s1, s2 = cc[sl].sum(), tc[sl].sum(), sa[sl].sum(), sr[sl].sum()
                out[0, bz, by, bx] = np.log1p(a)
                out[1, bz, by, bx] = np.log1p(t)
                out[2, bz, by, bx] = np.log1p(s1 / t) if t > 0 else 0.0
                out[3, bz, by, bx] = s2 / t if t > 0 else 0.0
    return out.reshape(-1)
