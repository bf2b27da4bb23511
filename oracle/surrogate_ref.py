"""CPU float64 reference of the learned surrogate's network — TEST
INFRASTRUCTURE ONLY (the checker of the tcgen05 convolution kernels and of the
training gradients).  Same architecture and latent layout as
formura_gb300.surrogate, written with torch's CPU conv2d in float64 and
circular padding, differentiated by autograd.
"""
from __future__ import annotations

import math

import torch
import torch.nn.functional as Fn

OUT_SCALE = 0.05


def conv(x, w, b=None):
    """x [B][n][n][64] (channels last), w [co][9][ci] (tap = (dy+1)*3 + dx+1);
    periodic 3x3 correlation, float64."""
    xc = x.permute(0, 3, 1, 2)
    xc = Fn.pad(xc, (1, 1, 1, 1), mode="circular")
    k = w.reshape(w.shape[0], 3, 3, w.shape[2]).permute(0, 3, 1, 2)
    y = Fn.conv2d(xc, k)
    y = y.permute(0, 2, 3, 1)
    if b is not None:
        y = y + b
    return y


def gelu(x):
    return 0.5 * x * (1.0 + torch.erf(x / math.sqrt(2.0)))


def pack(U, V, F, K):
    """(U, V) [B][N][N] float64, F, K [B] -> latent [B][N/4][N/4][64]."""
    B, N = U.shape[0], U.shape[1]
    n = N // 4

    def fold(a):
        return a.reshape(B, n, 4, n, 4).permute(0, 1, 3, 2, 4).reshape(B, n, n, 16)

    Fp = ((F - 0.04) * 50.0)[:, None, None, None].expand(B, n, n, 16)
    Kp = ((K - 0.06) * 100.0)[:, None, None, None].expand(B, n, n, 16)
    return torch.cat([fold(U), fold(V), Fp, Kp], dim=3)


def unfold_out(y, N):
    B, n = y.shape[0], y.shape[1]
    dU = y[..., :16].reshape(B, n, n, 4, 4).permute(0, 1, 3, 2, 4).reshape(B, N, N)
    dV = y[..., 16:32].reshape(B, n, n, 4, 4).permute(0, 1, 3, 2, 4).reshape(B, N, N)
    return dU, dV


def forward(x, ws, bs, n_blocks=6):
    h = gelu(conv(x, ws[0], bs[0]))
    for k in range(n_blocks):
        a1 = gelu(conv(h, ws[1 + 2 * k], bs[1 + 2 * k]))
        h = h + conv(a1, ws[2 + 2 * k], bs[2 + 2 * k])
    return conv(h, ws[-1], bs[-1])


def loss_and_grads(U0, V0, F, K, U1, V1, ws, bs):
    """Mean squared error of the latent increments (channels 0..31) and its
    gradients with respect to every weight and bias (float64)."""
    ws = [w.clone().double().requires_grad_(True) for w in ws]
    bs = [b.clone().double().requires_grad_(True) for b in bs]
    x = pack(U0, V0, F, K)
    y = forward(x, ws, bs)
    N = U0.shape[1]
    tU, tV = (U1 - U0) / OUT_SCALE, (V1 - V0) / OUT_SCALE
    B, n = y.shape[0], y.shape[1]
    t = torch.cat([tU.reshape(B, n, 4, n, 4).permute(0, 1, 3, 2, 4).reshape(B, n, n, 16),
                   tV.reshape(B, n, 4, n, 4).permute(0, 1, 3, 2, 4).reshape(B, n, n, 16)], dim=3)
    loss = ((y[..., :32] - t) ** 2).mean()
    loss.backward()
    return loss.item(), [w.grad for w in ws], [b.grad for b in bs]
