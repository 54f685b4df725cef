"""CPU restatement of the surrogate MLP's forward and backward pass
(test infrastructure: the oracle for the GPU gradients).

float64 arithmetic with the same BF16 roundings the GPU applies: inputs,
SiLU activations, the output gradient and the hidden-layer gradients are
rounded to BF16 (round to nearest even) before they enter a product;
weights are the BF16 copies of the FP32 master parameters.  Parameter
layout as photic_gb300/csrc/photic_kernels.h (W1 [128][16], b1, W2, b2,
W3, b3, W4 [16][128], b4)."""
from __future__ import annotations

import numpy as np

IN, H, OUT = 16, 128, 16
OFF = {}
_o = 0
for name, size in [("W1", H * IN), ("b1", H), ("W2", H * H), ("b2", H), ("W3", H * H),
                   ("b3", H), ("W4", OUT * H), ("b4", OUT)]:
    OFF[name] = (_o, size)
    _o += size
N_PARAMS = _o

IN_MEAN = np.array([0.011, 0.012, 0.010, 0.0035, 35.0, 0.0], dtype=np.float32)
IN_STD = np.array([0.006, 0.007, 0.007, 0.004, 10.0, 10.0], dtype=np.float32)
OUT_MEAN = np.array([-3.80, -3.45, -4.95, 0.275, 12.75], dtype=np.float32)
OUT_STD = np.array([0.865, 1.065, 1.129, 0.130, 7.07], dtype=np.float32)


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    out = {}
    for k, (o, n) in OFF.items():
        v = p[o:o + n]
        out[k] = v.reshape(H, IN) if k == "W1" else v.reshape(H, H) if k in ("W2", "W3") \
            else v.reshape(OUT, H) if k == "W4" else v
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x):
    w = unpack(p)
    R = x.shape[0]
    x0 = np.zeros((R, IN))
    x0[:, :6] = ((x.astype(np.float32) - IN_MEAN) / IN_STD)
    x0 = bf16(x0)
    zs, acts = [], [x0]
    a = x0
    for l in (1, 2, 3):
        z = a @ bf16(w[f"W{l}"]).T + w[f"b{l}"]
        zs.append(z)
        a = bf16(silu(z))
        acts.append(a)
    y = a @ bf16(w["W4"]).T + w["b4"]
    return y, zs, acts


def grads(p, x, t):
    """Gradient of mean((Y - t_std)^2) over the 5 outputs and R rows."""
    w = unpack(p)
    R = x.shape[0]
    y, zs, acts = forward(p, x)
    tn = (t.astype(np.float32) - OUT_MEAN) / OUT_STD
    d = np.zeros((R, OUT))
    d[:, :5] = y[:, :5] - tn
    loss = float(np.mean(d[:, :5] ** 2))
    dY = bf16((2.0 * d / (R * 5)).astype(np.float32))
    g = np.zeros(N_PARAMS)
    gw = {}
    gw["W4"] = dY.T @ acts[3]
    gw["b4"] = dY.sum(0)
    dZ = bf16((dY @ bf16(w["W4"])) * dsilu(zs[2]))
    for l in (3, 2, 1):
        gw[f"W{l}"] = dZ.T @ acts[l - 1]
        gw[f"b{l}"] = dZ.sum(0)
        if l > 1:
            dZ = bf16((dZ @ bf16(w[f"W{l}"])) * dsilu(zs[l - 2]))
    for k, (o, n) in OFF.items():
        g[o:o + n] = gw[k].reshape(-1)
    return g, loss
