"""CPU reference of the surrogate network (test infrastructure, numpy).

Restates, layer by layer, the network that poe2d_gb300/csrc/sg_net.cpp runs
on the tensor cores, so its forward pass, loss and parameter gradients can be
checked on the host.  ``bf16=True`` rounds to bfloat16 (nearest-even) at the
points where the GPU path stores bf16: the inputs, the weights, every layer's
activation, the loss gradient, the ReLU-masked gradients and the im2col
gradients; sums are float64.  ``bf16=False`` is the plain float64 network,
used for finite-difference checks of the backward pass itself.

Parameters use the compact layout of poe_sg_get_params: per layer the weights
[Cout][K] (K = taps x Cin, tap-major) then the biases [Cout].
"""
from __future__ import annotations

import numpy as np

# (kind, Cin, Cout, H or T, up, relu)
LAYERS = [
    ("conv2d", 2, 64, 64, 1, True),
    ("conv2d", 64, 128, 32, 1, True),
    ("conv2d", 128, 128, 16, 1, True),
    ("conv2d", 128, 256, 8, 1, True),
    ("fc", 4096 + 3, 256, 0, 1, True),
    ("fc", 256, 2048, 0, 1, True),
    ("conv1d", 128, 128, 16, 2, True),
    ("conv1d", 128, 128, 32, 2, True),
    ("conv1d", 128, 128, 64, 2, True),
    ("conv1d", 128, 64, 128, 2, True),
    ("conv1d", 64, 64, 256, 2, True),
    ("conv1d", 64, 64, 512, 2, True),
    ("conv1d", 64, 384, 1024, 1, False),
]


def _k(kind, cin):
    return 9 * cin if kind == "conv2d" else (3 * cin if kind == "conv1d" else cin)


def param_count():
    return sum(c * _k(kind, ci) + c for kind, ci, c, *_ in LAYERS)


def split(params):
    """Compact parameter vector -> list of (W [Cout, K], b [Cout]) float64."""
    out, q = [], 0
    for kind, ci, co, *_ in LAYERS:
        k = _k(kind, ci)
        W = np.asarray(params[q:q + co * k], np.float64).reshape(co, k)
        q += co * k
        b = np.asarray(params[q:q + co], np.float64)
        q += co
        out.append((W, b))
    return out


def join(parts):
    return np.concatenate([np.concatenate([W.ravel(), b.ravel()]) for W, b in parts])


def to_bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _im2col2d(x):
    """x [B, H, W, C] -> col [B*H/2*W/2, 9C], columns (ky*3 + kx)*C + c (3x3, stride 2, pad 1)."""
    B, H, W, C = x.shape
    Ho, Wo = H // 2, W // 2
    xp = np.zeros((B, H + 2, W + 2, C), x.dtype)
    xp[:, 1:H + 1, 1:W + 1] = x
    cols = []
    for ky in range(3):
        for kx in range(3):
            cols.append(xp[:, ky:ky + 2 * Ho:2, kx:kx + 2 * Wo:2, :])
    return np.concatenate(cols, axis=3).reshape(B * Ho * Wo, 9 * C)


def _col2im2d(dcol, B, H, W, C):
    Ho, Wo = H // 2, W // 2
    d = dcol.reshape(B, Ho, Wo, 9, C)
    dxp = np.zeros((B, H + 2, W + 2, C))
    for ky in range(3):
        for kx in range(3):
            dxp[:, ky:ky + 2 * Ho:2, kx:kx + 2 * Wo:2, :] += d[:, :, :, ky * 3 + kx, :]
    return dxp[:, 1:H + 1, 1:W + 1]


def _im2col1d(x, up):
    """x [B, T, C] repeated `up` times -> col [B*T*up, 3C], columns tap*C + c (k=3, pad 1)."""
    u = np.repeat(x, up, axis=1)
    B, To, C = u.shape
    up_ = np.zeros((B, To + 2, C), x.dtype)
    up_[:, 1:To + 1] = u
    return np.concatenate([up_[:, t:t + To] for t in range(3)], axis=2).reshape(B * To, 3 * C)


def _col2im1d(dcol, B, T, C, up):
    To = T * up
    d = dcol.reshape(B, To, 3, C)
    du = np.zeros((B, To + 2, C))
    for t in range(3):
        du[:, t:t + To] += d[:, :, t, :]
    du = du[:, 1:To + 1]
    return du.reshape(B, T, up, C).sum(axis=2)


def forward(params, maps, scalars, bf16=True, keep=False):
    """maps [B, 64, 64, 2], scalars [B, 3] -> out [B, 1024, 384] (float64).
    keep=True also returns the per-layer (A operand, output) list for backward."""
    rb = to_bf16 if bf16 else (lambda v: np.asarray(v, np.float64))
    P = split(params)
    B = maps.shape[0]
    x = rb(maps)
    cache = []
    for i, ((kind, ci, co, hw, up, relu), (W, b)) in enumerate(zip(LAYERS, P)):
        Wq = rb(W)
        if kind == "conv2d":
            A = _im2col2d(x.reshape(B, hw, hw, ci))
        elif kind == "conv1d":
            A = _im2col1d(x.reshape(B, hw, ci), up)
        elif i == 4:
            A = np.concatenate([x.reshape(B, 4096), rb(scalars)], axis=1)
        else:
            A = x.reshape(B, ci)
        z = A @ Wq.T + b
        y = np.maximum(z, 0.0) if relu else z
        if i + 1 < len(LAYERS):
            y = rb(y)
        cache.append((A, y))
        x = y
    out = x.reshape(B, 1024, 384)
    return (out, cache) if keep else out


def loss_and_grads(params, maps, scalars, targets, bf16=True):
    """Mean squared error against targets [B, 1024, 384] and its gradient in
    the compact parameter layout, by explicit backpropagation."""
    rb = to_bf16 if bf16 else (lambda v: np.asarray(v, np.float64))
    P = split(params)
    B = maps.shape[0]
    out, cache = forward(params, maps, scalars, bf16=bf16, keep=True)
    t = np.asarray(targets, np.float64)
    n = out.size
    diff = out - t
    loss = float(np.sum(diff * diff) / n)
    dy = rb((2.0 / n) * diff).reshape(B * 1024, 384)
    grads = [None] * len(LAYERS)
    for i in range(len(LAYERS) - 1, -1, -1):
        kind, ci, co, hw, up, relu = LAYERS[i]
        A, y = cache[i]
        W, _ = P[i]
        if i == 3:
            dy = dy.reshape(B, -1)[:, :4096]
        dz = dy.reshape(-1, co) * (y.reshape(-1, co) > 0) if relu else dy.reshape(-1, co)
        gW = dz.T @ A
        gb = dz.sum(axis=0)
        grads[i] = (gW, gb)
        if i == 0:
            break
        dcol = rb(dz @ rb(W))
        if kind == "conv2d":
            dy = rb(_col2im2d(dcol, B, hw, hw, ci))
        elif kind == "conv1d":
            dy = rb(_col2im1d(dcol, B, hw, ci, up))
        else:
            dy = dcol
    return loss, join(grads)


# Adam's constants as the network's optimiser holds them: float32 values,
# with 1 - beta computed in float32 (poe_sg_adam, sg_ops.cu k_adam)
ADAM_B1 = np.float32(0.9)
ADAM_B2 = np.float32(0.999)
ADAM_EPS = 1e-8


def adam_step(w, g, m, v, t, lr, b1=ADAM_B1, b2=ADAM_B2, eps=ADAM_EPS):
    """One Adam step (Kingma & Ba 2015, Algorithm 1) in float64: step t
    (1-based) from parameters w, gradient g and moments m, v; returns the new
    (w, m, v).  m_hat = m / (1 - b1^t), v_hat = v / (1 - b2^t),
    w -= lr m_hat / (sqrt(v_hat) + eps)."""
    w, g, m, v = (np.asarray(a, np.float64) for a in (w, g, m, v))
    one_b1 = float(np.float32(1.0) - np.float32(b1))
    one_b2 = float(np.float32(1.0) - np.float32(b2))
    m = float(b1) * m + one_b1 * g
    v = float(b2) * v + one_b2 * g * g
    m_hat = m / (1.0 - float(b1) ** t)
    v_hat = v / (1.0 - float(b2) ** t)
    return w - lr * m_hat / (np.sqrt(v_hat) + eps), m, v


def bf16_bits(x):
    """float32 -> bfloat16 by round-to-nearest-even, returned as float32 bits
    with the low 16 bits clear (finite inputs)."""
    b = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32)
