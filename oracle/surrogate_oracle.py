"""CPU oracle for the surrogate network -- TEST INFRASTRUCTURE ONLY.

NumPy forward and backward of the library's 3D U-Net (gliomauq_gb300/csrc/
surrogate.cu): float64 arithmetic with the activations, weights and
gradients rounded to bf16 at the points where the GPU stores them, so that
the GPU's loss and parameter gradient can be checked against it. Layout
[batch, z, y, x, channel]; weights [cout, 27, cin], tap = dx+1 + 3(dy+1) + 9(dz+1).
"""
from __future__ import annotations

import numpy as np

LAYERS = [(16, 16, True), (16, 16, True), (16, 32, True), (32, 32, True), (32, 32, True),
          (64, 16, True), (32, 16, True), (16, 16, False)]


def offsets():
    out, p = [], 0
    for ci, co, _ in LAYERS:
        w = p
        p += co * 27 * ci
        out.append((w, p))
        p += co
    return out, p


def bf16(x):
    """Round float64 values to bf16 (round to nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def conv(x, w, b):
    """x [B,D,H,W,Ci], w [Co,27,Ci] -> [B,D,H,W,Co], zero padding."""
    B, D, H, W, Ci = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((B, D, H, W, w.shape[0]))
    for tap in range(27):
        dx, dy, dz = tap % 3 - 1, (tap // 3) % 3 - 1, tap // 9 - 1
        sl = xp[:, 1 + dz:1 + dz + D, 1 + dy:1 + dy + H, 1 + dx:1 + dx + W, :]
        out += sl @ w[:, tap, :].T
    if b is not None:
        out += b
    return out


def conv_wgrad(x, dy):
    """dw[co, tap, ci] = sum_v dy[v, co] x[v + tap, ci]."""
    B, D, H, W, Ci = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    Co = dy.shape[-1]
    dw = np.zeros((Co, 27, Ci))
    d2 = dy.reshape(-1, Co)
    for tap in range(27):
        dx, dyy, dz = tap % 3 - 1, (tap // 3) % 3 - 1, tap // 9 - 1
        sl = xp[:, 1 + dz:1 + dz + D, 1 + dyy:1 + dyy + H, 1 + dx:1 + dx + W, :].reshape(-1, Ci)
        dw[:, tap, :] = d2.T @ sl
    return dw


def conv_dgrad(dy, w):
    """dx = conv(dy, flipped/transposed w)."""
    wt = w[:, ::-1, :].transpose(2, 1, 0)  # [ci, 27, co] with the tap flipped
    return conv(dy, wt, None)


def pool(x):
    B, D, H, W, C = x.shape
    return x.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4, 6))


def pool_bwd(d):
    return 0.125 * d.repeat(2, 1).repeat(2, 2).repeat(2, 3)


def up(x):
    return x.repeat(2, 1).repeat(2, 2).repeat(2, 3)


def up_bwd(d):
    B, D, H, W, C = d.shape
    return d.reshape(B, D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4, 6))


def loss_and_grad(params, feats, targets, rounding=True):
    """params: flat float32 vector; feats [B,m,m,m,16]; targets [B,m,m,m].
    Returns (loss, flat gradient) with the GPU's bf16 rounding points, or in
    plain float64 with rounding=False (for finite-difference checks)."""
    bf16 = globals()["bf16"] if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    offs, P = offsets()
    W, Bs = [], []
    for (ci, co, _), (wo, bo) in zip(LAYERS, offs):
        W.append(bf16(params[wo:wo + co * 27 * ci].reshape(co, 27, ci)))
        Bs.append(np.asarray(params[bo:bo + co], dtype=np.float64))
    relu = lambda v: np.maximum(v, 0.0)
    x0 = bf16(feats)
    t0 = bf16(relu(conv(x0, W[0], Bs[0])))
    c0b = bf16(relu(conv(t0, W[1], Bs[1])))          # c0[16:32]
    p1 = bf16(pool(c0b))
    t1 = bf16(relu(conv(p1, W[2], Bs[2])))
    c1b = bf16(relu(conv(t1, W[3], Bs[3])))          # c1[32:64]
    p2 = bf16(pool(c1b))
    q2 = bf16(relu(conv(p2, W[4], Bs[4])))
    c1 = np.concatenate([up(q2), c1b], axis=-1)
    u1 = bf16(relu(conv(c1, W[5], Bs[5])))
    c0 = np.concatenate([up(u1), c0b], axis=-1)
    u0 = bf16(relu(conv(c0, W[6], Bs[6])))
    logits = conv(u0, W[7], Bs[7])
    if rounding:
        logits = logits.astype(np.float32).astype(np.float64)
    l0 = logits[..., 0]
    s = 1.0 / (1.0 + np.exp(-l0))
    nv = l0.size
    d = s - targets
    loss = np.sum(d * d) / nv
    dl = np.zeros_like(logits)
    dl[..., 0] = bf16(2.0 * d * s * (1.0 - s) / nv)
    g = np.zeros(P)

    def put(i, dw, db):
        wo, bo = offs[i]
        g[wo:wo + dw.size] = dw.ravel()
        g[bo:bo + db.size] = db

    def sumv(dy):
        return dy.reshape(-1, dy.shape[-1]).sum(axis=0)

    put(7, conv_wgrad(u0, dl), sumv(dl))
    du0 = bf16(conv_dgrad(dl, W[7])) * (u0 > 0)
    put(6, conv_wgrad(c0, du0), sumv(du0))
    dc0 = bf16(conv_dgrad(du0, W[6]))
    du1 = bf16(up_bwd(dc0[..., :16])) * (u1 > 0)
    put(5, conv_wgrad(c1, du1), sumv(du1))
    dc1 = bf16(conv_dgrad(du1, W[5]))
    dq2 = bf16(up_bwd(dc1[..., :32])) * (q2 > 0)
    put(4, conv_wgrad(p2, dq2), sumv(dq2))
    dp2 = bf16(conv_dgrad(dq2, W[4]))
    dc1b = bf16(dc1[..., 32:] + bf16(pool_bwd(dp2))) * (c1b > 0)
    put(3, conv_wgrad(t1, dc1b), sumv(dc1b))
    dt1 = bf16(conv_dgrad(dc1b, W[3])) * (t1 > 0)
    put(2, conv_wgrad(p1, dt1), sumv(dt1))
    dp1 = bf16(conv_dgrad(dt1, W[2]))
    dc0b = bf16(dc0[..., 16:] + bf16(pool_bwd(dp1))) * (c0b > 0)
    put(1, conv_wgrad(t0, dc0b), sumv(dc0b))
    dt0 = bf16(conv_dgrad(dc0b, W[1])) * (t0 > 0)
    put(0, conv_wgrad(x0, dt0), sumv(dt0))
    return loss, g
