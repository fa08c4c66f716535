"""TEST INFRASTRUCTURE ONLY: host restatement of the learned-lambda network (float64 numpy).

The network (8 -> 64 -> 64 -> 64 -> 1, SiLU) has no counterpart in the reference; this module
states its mathematics independently of the CUDA kernels so the tensor-core forward pass and
gradient can be checked.  With `emulate=True` it rounds to BF16 exactly where the kernels do
(normalised inputs, hidden activations a1 and a2, the back-propagated dz of every layer, the
weights W1..W3) and computes everything else in float64; with `emulate=False` it is the plain
float64 network, whose analytic gradient is checked against finite differences.

Parameter layout (flat float32[8961]): W1[64][8], b1[64], W2[64][64], b2[64], W3[64][64], b3[64],
w4[64], b4.  Normalisation (float32[18]): mean[8], inv_std[8], output scale, blend (the blend
only mixes the output with an input feature when a step uses it; `forward` returns the estimate).
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID = 8, 64
SIZES = [("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
         ("W3", (N_HID, N_HID)), ("b3", (N_HID,)), ("w4", (N_HID,)), ("b4", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)
N_NORM = 2 * N_IN + 2


def bf16(x) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), through float32, returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params) -> dict:
    p = np.asarray(params, dtype=np.float64)
    assert p.size == N_PARAMS
    out, o = {}, 0
    for name, shape in SIZES:
        k = int(np.prod(shape))
        out[name] = p[o:o + k].reshape(shape)
        o += k
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SIZES])


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sigmoid(z)


def dsilu(z):
    s = sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


def forward(params, norm, feat, emulate=True):
    """Returns (output in lambda units [n], cache for the backward pass)."""
    P = unpack(params)
    norm = np.asarray(norm, dtype=np.float64)
    mean, inv_std, scale = norm[:N_IN], norm[N_IN:2 * N_IN], norm[2 * N_IN]
    r = bf16 if emulate else (lambda v: np.asarray(v, dtype=np.float64))
    x = np.asarray(feat, dtype=np.float64)
    x = r((x - mean) * inv_std)
    W1, W2, W3 = r(P["W1"]), r(P["W2"]), r(P["W3"])
    z1 = x @ W1.T + P["b1"]
    a1 = r(silu(z1))
    z2 = a1 @ W2.T + P["b2"]
    a2 = r(silu(z2))
    z3 = a2 @ W3.T + P["b3"]
    a3 = silu(z3)
    y = a3 @ P["w4"] + P["b4"][0]
    cache = dict(x=x, z1=z1, a1=a1, z2=z2, a2=a2, z3=z3, a3=a3, y=y, W2=W2, W3=W3, P=P,
                 scale=scale, r=r)
    return y * scale, cache


def gradient(params, norm, feat, target, emulate=True):
    """(dL/dparams [N_PARAMS], L) for L = (1/n) sum (y - target/scale)^2, y the pre-scale output."""
    _, c = forward(params, norm, feat, emulate)
    r, P = c["r"], c["P"]
    n = len(c["y"])
    t = np.asarray(target, dtype=np.float64) / c["scale"]
    e = c["y"] - t
    loss = float(np.sum(e * e) / n)
    dy = 2.0 * e / n
    g = {"w4": c["a3"].T @ dy, "b4": np.array([dy.sum()])}
    dz3 = r(dy[:, None] * P["w4"][None, :] * dsilu(c["z3"]))
    g["W3"] = dz3.T @ c["a2"]
    g["b3"] = dz3.sum(0)
    dz2 = r((dz3 @ c["W3"]) * dsilu(c["z2"]))
    g["W2"] = dz2.T @ c["a1"]
    g["b2"] = dz2.sum(0)
    dz1 = r((dz2 @ c["W2"]) * dsilu(c["z1"]))
    g["W1"] = dz1.T @ c["x"]
    g["b1"] = dz1.sum(0)
    return pack(g), loss


def loss(params, norm, feat, target, emulate=False):
    y, c = forward(params, norm, feat, emulate)
    t = np.asarray(target, dtype=np.float64) / c["scale"]
    return float(np.mean((c["y"] - t) ** 2))
