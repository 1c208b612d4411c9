"""numpy restatement of the learned-guess network (per-element MLP).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA forward/backward/Adam
kernels (neko-top_gb300/csrc/mlp.cu).  The network and loss:

    H1 = relu(X W1 + b1),  H2 = relu(H1 W2 + b2),  Y = H2 W3 + b3,
    loss = mean((Y - T)^2)

Parameters are one flat float32 array [W1 | b1 | W2 | b2 | W3 | b3] with W
row-major [in x out].  With ``emulate_bf16`` the function rounds exactly the
operands the GPU rounds to BF16 (X, the weights, H1, H2 and the GEMM copies
of dY and dZ) and accumulates in float64, so the only remaining difference to
the GPU is FP32 accumulation order.
"""
from __future__ import annotations

import numpy as np


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    out = ((u + r) & 0xFFFF0000).astype(np.uint32)
    return out.view(np.float32)


def bf16_bits(a):
    """BF16 bit patterns (uint16) of float32 values (round to nearest even)."""
    return (bf16(a).view(np.uint32) >> 16).astype(np.uint16)


def layout(F, H, O):
    oW1 = 0
    ob1 = F * H
    oW2 = ob1 + H
    ob2 = oW2 + H * H
    oW3 = ob2 + H
    ob3 = oW3 + H * O
    return dict(W1=(oW1, (F, H)), b1=(ob1, (H,)), W2=(oW2, (H, H)), b2=(ob2, (H,)), W3=(oW3, (H, O)),
                b3=(ob3, (O,))), ob3 + O


def unpack(p, F, H, O):
    lay, n = layout(F, H, O)
    assert p.size == n
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in lay.items()}


def pack(d, F, H, O):
    lay, n = layout(F, H, O)
    p = np.zeros(n, dtype=np.float64)
    for k, (o, s) in lay.items():
        p[o:o + int(np.prod(s))] = np.asarray(d[k]).ravel()
    return p


def forward(p, X, F, H, O, emulate_bf16=True):
    P = unpack(np.asarray(p, dtype=np.float64), F, H, O)
    rb = (lambda a: bf16(a).astype(np.float64)) if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Xb = rb(X)
    W1, W2, W3 = rb(P["W1"]), rb(P["W2"]), rb(P["W3"])
    Z1 = Xb @ W1 + P["b1"]
    H1 = rb(np.maximum(Z1, 0.0))
    Z2 = H1 @ W2 + P["b2"]
    H2 = rb(np.maximum(Z2, 0.0))
    Y = H2 @ W3 + P["b3"]
    return Y, dict(Xb=Xb, W1=W1, W2=W2, W3=W3, H1=H1, H2=H2)


def loss_and_grad(p, X, T, F, H, O, emulate_bf16=True):
    Y, c = forward(p, X, F, H, O, emulate_bf16)
    rb = (lambda a: bf16(a).astype(np.float64)) if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    D = Y - T
    loss = float(np.mean(D * D))
    dY = (2.0 / D.size) * D
    if emulate_bf16:
        dY = dY.astype(np.float32).astype(np.float64)
    dYb = rb(dY)
    g = {}
    g["W3"] = c["H2"].T @ dYb
    g["b3"] = dY.sum(0)
    dH2 = dYb @ c["W3"].T
    dZ2 = np.where(c["H2"] > 0, dH2, 0.0)
    if emulate_bf16:
        dZ2 = dZ2.astype(np.float32).astype(np.float64)
    dZ2b = rb(dZ2)
    g["W2"] = c["H1"].T @ dZ2b
    g["b2"] = dZ2.sum(0)
    dH1 = dZ2b @ c["W2"].T
    dZ1 = np.where(c["H1"] > 0, dH1, 0.0)
    if emulate_bf16:
        dZ1 = dZ1.astype(np.float32).astype(np.float64)
    dZ1b = rb(dZ1)
    g["W1"] = c["Xb"].T @ dZ1b
    g["b1"] = dZ1.sum(0)
    return loss, pack(g, F, H, O)


def init_params(F, H, O, rng):
    d = {"W1": rng.uniform(-1, 1, (F, H)) * np.sqrt(6.0 / F), "b1": rng.uniform(-0.1, 0.1, H),
         "W2": rng.uniform(-1, 1, (H, H)) * np.sqrt(6.0 / H), "b2": rng.uniform(-0.1, 0.1, H),
         "W3": rng.uniform(-1, 1, (H, O)) * np.sqrt(6.0 / H), "b3": rng.uniform(-0.1, 0.1, O)}
    return pack(d, F, H, O)
