"""TEST INFRASTRUCTURE: NumPy restatement of the solid-angle surrogate network
(xmimsim_gb300/csrc/mlp.cu) used as the checker of the tensor-core kernels.

Same parameter layout and the same rounding points as the GPU kernels: BF16
weights, inputs and hidden activations (round to nearest even), FP32
accumulation (evaluated here in FP64 and rounded to FP32), SiLU, FP32 output
layer.  Gradients follow the same graph (straight-through through the BF16
roundings) for the checks of the backward kernels."""
from __future__ import annotations

import numpy as np

H, NIN = 128, 3
NPARAM = H * NIN + H + 3 * (H * H + H) + H + 1


ROUND_BF16 = True  # False: exact arithmetic (for checking the backward formulas)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    if not ROUND_BF16:
        return np.asarray(x, dtype=np.float64)
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & np.uint32(1)) + np.uint32(0x7FFF)
    return ((u + r) & np.uint32(0xFFFF0000)).view(np.float32)


def unpack(theta: np.ndarray):
    t = np.asarray(theta, dtype=np.float32 if ROUND_BF16 else np.float64)
    o = 0
    W0 = t[o:o + H * NIN].reshape(H, NIN); o += H * NIN
    b0 = t[o:o + H]; o += H
    Ws, bs = [W0], [b0]
    for _ in range(3):
        Ws.append(t[o:o + H * H].reshape(H, H)); o += H * H
        bs.append(t[o:o + H]); o += H
    wo = t[o:o + H]; o += H
    bo = t[o]
    return Ws, bs, wo, bo


def silu(z):
    return z / (1.0 + np.exp(-z))


def forward(theta: np.ndarray, x: np.ndarray, keep: bool = False):
    """Layer 0 in FP32 with unrounded inputs and W0 (the GPU computes it on
    the CUDA cores); layers 1-3 with BF16 activations and weights.  acts[0]
    is the BF16 input the backward pass's dW0 GEMM uses."""
    Ws, bs, wo, bo = unpack(theta)
    ft = np.float32 if ROUND_BF16 else np.float64
    xin = np.asarray(x, dtype=ft)
    acts, zs = [bf16(xin)], []
    h = None
    a = xin
    for l in range(4):
        W = Ws[l].astype(np.float64) if l == 0 else bf16(Ws[l]).astype(np.float64)
        z = (a.astype(np.float64) @ W.T + bs[l].astype(np.float64)).astype(ft)
        h = silu(z.astype(np.float64)).astype(ft)
        zs.append(z)
        a = bf16(h) if l < 3 else h
        acts.append(a)
    y = (h.astype(np.float64) @ wo.astype(np.float64)).astype(np.float32 if ROUND_BF16 else np.float64) + bo
    return (y, acts, zs) if keep else y


def init_params(seed: int) -> np.ndarray:
    """He-style initialisation of the parameter vector."""
    rng = np.random.default_rng(seed)
    parts = [rng.normal(0, np.sqrt(2.0 / NIN), H * NIN), np.zeros(H)]
    for _ in range(3):
        parts += [rng.normal(0, np.sqrt(2.0 / H), H * H), np.zeros(H)]
    parts += [rng.normal(0, np.sqrt(1.0 / H), H), np.zeros(1)]
    return np.concatenate(parts).astype(np.float32)


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def grad(theta: np.ndarray, x: np.ndarray, t: np.ndarray):
    """Gradient of mean((y - t)^2) with the GPU kernels' rounding points: the
    backward GEMMs take BF16 dZ, BF16 activations and BF16 weights; bias,
    output-layer and dZ values stay FP32."""
    Ws, bs, wo, bo = unpack(theta)
    y, acts, zs = forward(theta, x, keep=True)
    n = len(y)
    dy = (2.0 * (y.astype(np.float64) - t) / n)
    g = {}
    h3 = acts[4].astype(np.float64)
    g["wo"] = dy @ h3
    g["bo"] = dy.sum()
    ft = np.float32 if ROUND_BF16 else np.float64
    dz = (dy[:, None] * wo[None, :].astype(np.float64) * dsilu(zs[3].astype(np.float64))).astype(ft)
    for l in range(3, -1, -1):
        g[f"b{l}"] = dz.astype(np.float64).sum(axis=0)
        dzb = bf16(dz).astype(np.float64)
        g[f"W{l}"] = dzb.T @ acts[l].astype(np.float64)
        if l > 0:
            dh = dzb @ bf16(Ws[l]).astype(np.float64)
            dz = (dh * dsilu(zs[l - 1].astype(np.float64))).astype(ft)
    parts = [g["W0"].ravel(), g["b0"]]
    for l in range(1, 4):
        parts += [g[f"W{l}"].ravel(), g[f"b{l}"]]
    parts += [g["wo"], np.array([g["bo"]])]
    return np.concatenate(parts), float(np.mean((y.astype(np.float64) - t) ** 2))
