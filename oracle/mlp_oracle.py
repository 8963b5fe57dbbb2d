"""CPU restatement (numpy) of the learned relocation proposal's MLP, test
infrastructure only: the forward pass and the MSE backward pass of
msplat_gb300/csrc/mlp.cu (22 -> 64 -> 64 -> 2, SiLU), with the same BF16
roundings where the kernels round (layer inputs, weights, and the dL/dy and
dL/dz2 operands of the tensor-core backward products) when `bf16=True`, and
exact float64 arithmetic otherwise (for finite-difference checks).

Parameter layout (flat FP32, kMlp* in kernels.h): W1 [32][64], b1 [64],
W2 [64][64], b2 [64], W3 [64][16], b3 [16]."""
from __future__ import annotations

import numpy as np

N_IN = 22
OFF = dict(W1=(0, (32, 64)), b1=(2048, (64,)), W2=(2112, (64, 64)), b2=(6208, (64,)), W3=(6272, (64, 16)),
           b3=(7296, (16,)))
N_PARAMS = 7312


def unpack(P):
    P = np.asarray(P)
    return {k: P[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in OFF.items()}


def pack(d):
    P = np.zeros(N_PARAMS, np.float32)
    for k, (o, s) in OFF.items():
        P[o:o + int(np.prod(s))] = np.asarray(d[k], np.float32).ravel()
    return P


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float32."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(np.shape(x))


def bf16_bits(x):
    return (np.ascontiguousarray(bf16(x), np.float32).view(np.uint32) >> 16).astype(np.uint16)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init_params(seed=0):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases; unused rows/columns zero."""
    rng = np.random.default_rng(seed)
    d = {k: np.zeros(s, np.float32) for k, (o, s) in OFF.items()}
    d["W1"][:N_IN] = rng.uniform(-1, 1, (N_IN, 64)) / np.sqrt(N_IN)
    d["W2"][:] = rng.uniform(-1, 1, (64, 64)) / 8.0
    d["W3"][:, :2] = rng.uniform(-1, 1, (64, 2)) / 8.0
    return pack(d)


def forward(X, P, rounding=True):
    """X [n, 32] (float); returns (y [n, 2], cache)."""
    f = np.float32 if rounding else np.float64
    p = {k: v.astype(f) for k, v in unpack(P).items()}
    r = bf16 if rounding else (lambda a: a)
    X = r(np.asarray(X, f))
    W1, W2, W3 = r(p["W1"]), r(p["W2"]), r(p["W3"])
    Z1 = (X.astype(np.float64) @ W1.astype(np.float64)).astype(f) + p["b1"]
    H1 = r(silu(Z1))
    Z2 = (H1.astype(np.float64) @ W2.astype(np.float64)).astype(f) + p["b2"]
    H2 = r(silu(Z2))
    Y = (H2.astype(np.float64) @ W3.astype(np.float64)).astype(f) + p["b3"]
    return Y[:, :2], dict(X=X, Z1=Z1, H1=H1, Z2=Z2, H2=H2, Y=Y, W2=W2, W3=W3)


def loss_and_grad(X, T, P, rounding=True):
    """Mean over samples of the summed squared error of the 2 outputs, and its
    gradient with respect to the flat parameters."""
    n = len(X)
    y, c = forward(X, P, rounding)
    r = bf16 if rounding else (lambda a: a)
    e = y - np.asarray(T, y.dtype)
    loss = float(np.sum(e * e) / n)
    dY = np.zeros_like(c["Y"])
    dY[:, :2] = 2.0 * e / n
    g = {}
    g["W3"] = c["H2"].T.astype(np.float64) @ dY
    g["b3"] = dY.sum(0)
    dH2 = r(dY) @ c["W3"].T
    dZ2 = dH2 * silu_grad(c["Z2"])
    g["W2"] = c["H1"].T.astype(np.float64) @ dZ2
    g["b2"] = dZ2.sum(0)
    dH1 = r(dZ2) @ c["W2"].T
    dZ1 = dH1 * silu_grad(c["Z1"])
    g["W1"] = c["X"].T.astype(np.float64) @ dZ1
    g["W1"][N_IN:] = 0.0
    g["b1"] = dZ1.sum(0)
    return loss, pack(g) if rounding else _pack64(g)


def _pack64(d):
    P = np.zeros(N_PARAMS, np.float64)
    for k, (o, s) in OFF.items():
        P[o:o + int(np.prod(s))] = np.asarray(d[k], np.float64).ravel()
    return P
