"""Learned 16-step surrogate of the 2D Gray-Scott program (pearson-2d form).

A convolutional neural operator that maps (U, V, F, k) at step t to (U, V) at
step t+16, run with BF16 weights and activations and FP32 accumulation on the
tcgen05 tensor cores (``fm_conv3x3_*`` in libformura_gb300.so):

* the periodic N x N state is folded 4 x 4 into a 64-channel latent grid of
  (N/4) x (N/4) (space-to-depth; ``fm_sur_pack``);
* lift: 3x3 conv 64 -> 64 + GELU;
* 6 residual blocks: h <- h + conv(GELU(conv(h)));
* projection: 3x3 conv 64 -> 32 (stored as 64 with the last 32 output
  channels pinned to zero) -> the increments dU, dV (``fm_sur_unpack``).
All convolutions are periodic (the latent tensors carry a one-pixel periodic
halo).  14 convolutions of 36,864 weights: 0.52 M parameters.

Training (``Surrogate.train_step``): MSE on the 16-step increment, data and
weight gradients on the tensor cores (the data gradient is the forward
convolution with flipped, transposed weights; the weight gradient a split-K
GEMM over pixels), Adam on FP32 master weights.

The plain stencil remains the fallback and the reference for its error: see
:func:`formura_gb300.surrogate_run.run_with_surrogate`.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import List, Optional

import numpy as np
import torch

from ._lib import check, lib

C = 64
N_BLOCKS = 6
JUMP = 16
OUT_SCALE = 0.05  # latent output unit: increments of 0.05 in U or V


def _p(t: Optional[torch.Tensor]):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass
class _Layer:
    w: torch.Tensor     # fp32 master [64][9][64]
    b: torch.Tensor     # fp32 [64]
    wb: torch.Tensor    # bf16 copy
    wf: torch.Tensor    # bf16 flipped/transposed (data gradient)
    mw: torch.Tensor
    vw: torch.Tensor
    mb: torch.Tensor
    vb: torch.Tensor
    gw: torch.Tensor    # fp32 dW transposed [9][64][64]
    gb: torch.Tensor    # fp32 [64]
    mask_co: int        # -1: none


class Surrogate:
    def __init__(self, seed: int = 0, device: str = "cuda", n_blocks: int = N_BLOCKS):
        g = torch.Generator().manual_seed(seed)
        self.dev = torch.device(device)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.layers: List[_Layer] = []
        self.n_blocks = int(n_blocks)
        std = math.sqrt(2.0 / (9 * C))
        n_layers = 2 + 2 * self.n_blocks
        for i in range(n_layers):
            w = torch.randn(C, 9, C, generator=g) * std
            mask = -1
            if i >= 1 and i < n_layers - 1 and (i - 1) % 2 == 1:
                w *= 0.1          # second conv of each residual block starts small
            if i == n_layers - 1:
                w *= 0.1
                mask = 32
                w[32:] = 0.0
            self.layers.append(self._make_layer(w, mask))
        self.step_count = 0
        self._bufs = {}

    def _make_layer(self, w: torch.Tensor, mask: int) -> _Layer:
        d = self.dev
        w = w.to(d).contiguous()
        L = _Layer(w=w, b=torch.zeros(C, device=d), wb=w.to(torch.bfloat16).contiguous(),
                   wf=torch.empty(C, 9, C, dtype=torch.bfloat16, device=d),
                   mw=torch.zeros_like(w), vw=torch.zeros_like(w),
                   mb=torch.zeros(C, device=d), vb=torch.zeros(C, device=d),
                   gw=torch.zeros(9, C, C, device=d), gb=torch.zeros(C, device=d), mask_co=mask)
        return L

    # ---- parameters ----------------------------------------------------------
    def n_params(self) -> int:
        n = 0
        for i, L in enumerate(self.layers):
            co = L.mask_co if L.mask_co > 0 else C
            n += co * 9 * C + co
        return n

    def state_dict(self):
        return {"w": [L.w.cpu() for L in self.layers], "b": [L.b.cpu() for L in self.layers],
                "step": self.step_count}

    def save_npz(self, path) -> None:
        """Weights and biases as float32 arrays (w0..w13 [64][9][64], b0..b13)."""
        arrs = {}
        for i, L in enumerate(self.layers):
            arrs["w%d" % i] = L.w.cpu().numpy()
            arrs["b%d" % i] = L.b.cpu().numpy()
        arrs["step"] = np.array(self.step_count)
        arrs["n_blocks"] = np.array(self.n_blocks)
        np.savez_compressed(path, **arrs)

    def load_npz(self, path) -> None:
        with np.load(path) as z:
            nb = int(z["n_blocks"]) if "n_blocks" in z else N_BLOCKS
            if nb != self.n_blocks:
                raise ValueError("%s holds %d residual blocks, this network has %d"
                                 % (path, nb, self.n_blocks))
            for i, L in enumerate(self.layers):
                L.w.copy_(torch.from_numpy(z["w%d" % i]).to(self.dev))
                L.b.copy_(torch.from_numpy(z["b%d" % i]).to(self.dev))
                L.wb.copy_(L.w.to(torch.bfloat16))
            self.step_count = int(z["step"])

    def load_state_dict(self, sd):
        for L, w, b in zip(self.layers, sd["w"], sd["b"]):
            L.w.copy_(w.to(self.dev))
            L.b.copy_(b.to(self.dev))
            L.wb.copy_(L.w.to(torch.bfloat16))
        self.step_count = int(sd.get("step", 0))

    # ---- buffers ---------------------------------------------------------------
    def _buf(self, name: str, B: int, n: int, dtype=torch.bfloat16, ch: int = C) -> torch.Tensor:
        key = (name, B, n, dtype, ch)
        t = self._bufs.get(key)
        if t is None:
            if dtype == torch.float32 and name.startswith("yf"):
                t = torch.empty(B, n, n, ch, dtype=dtype, device=self.dev)
            else:
                t = torch.empty(B, n + 2, n + 2, ch, dtype=dtype, device=self.dev)
            self._bufs[key] = t
        return t

    def _conv(self, B, n, x, L: _Layer, *, weights=None, bias=True, gate=None, resid=None,
              act=0, z_out=None, y_out=None, y_f32=None):
        w = L.wb if weights is None else weights
        st = lib().fm_conv3x3_fwd_bf16(B, n, n, C, _p(x), _p(w), _p(L.b) if bias else None,
                                       _p(gate), _p(resid), act, _p(z_out), _p(y_out),
                                       _p(y_f32), _p(self.err), _stream())
        check(st, "fm_conv3x3_fwd_bf16")

    # ---- forward -----------------------------------------------------------------
    def forward_latent(self, xpad: torch.Tensor, B: int, n: int, keep: bool = False):
        """Latent prediction y (fp32 [B][n][n][64]) from the packed input."""
        Ls = self.layers
        h = self._buf("h0", B, n)
        z0 = self._buf("z0", B, n) if keep else None
        self._conv(B, n, xpad, Ls[0], act=1, z_out=z0, y_out=h)
        acts = [h]
        for k in range(self.n_blocks):
            c1, c2 = Ls[1 + 2 * k], Ls[2 + 2 * k]
            a1 = self._buf("a1_%d" % k if keep else "a1", B, n)
            z1 = self._buf("z1_%d" % k, B, n) if keep else None
            self._conv(B, n, h, c1, act=1, z_out=z1, y_out=a1)
            h_next = self._buf("h%d" % (k + 1) if keep else ("hA" if k % 2 == 0 else "hB"), B, n)
            self._conv(B, n, a1, c2, resid=h, y_out=h_next)
            h = h_next
            acts.append(h)
        y = self._buf("yf", B, n, torch.float32)
        self._conv(B, n, h, Ls[-1], y_f32=y)
        return y

    def predict(self, U: torch.Tensor, V: torch.Tensor, F: torch.Tensor, K: torch.Tensor):
        """In place: (U, V) <- the network's state 16 steps later.  U, V are
        float32 [B][N][N] CUDA tensors, F, K float32 [B]."""
        B, N = U.shape[0], U.shape[1]
        n = N // 4
        xpad = self._buf("x", B, n)
        check(lib().fm_sur_pack(B, N, _p(U), _p(V), _p(F), _p(K), _p(xpad), _stream()),
              "fm_sur_pack")
        y = self.forward_latent(xpad, B, n)
        check(lib().fm_sur_unpack(B, N, _p(y), _p(U), _p(V), OUT_SCALE, _stream()),
              "fm_sur_unpack")

    # ---- training ------------------------------------------------------------------
    def loss_and_grads(self, U0, V0, F, K, U1, V1) -> torch.Tensor:
        """Forward + backward of the MSE between the predicted and the true
        16-step increments; gradients land in each layer's gw/gb.  Returns the
        loss (a 0-d CUDA tensor, mean over latent outputs)."""
        B, N = U0.shape[0], U0.shape[1]
        n = N // 4
        Ls = self.layers
        xpad = self._buf("x", B, n)
        check(lib().fm_sur_pack(B, N, _p(U0), _p(V0), _p(F), _p(K), _p(xpad), _stream()),
              "fm_sur_pack")
        y = self.forward_latent(xpad, B, n, keep=True)
        count = B * n * n * 32
        loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        dy = self._buf("dy", B, n)
        check(lib().fm_sur_loss_grad(B, N, _p(y), _p(U0), _p(V0), _p(U1), _p(V1), _p(dy),
                                     _p(loss), OUT_SCALE, 1.0 / count, _stream()),
              "fm_sur_loss_grad")
        for L in Ls:
            L.gw.zero_()
            L.gb.zero_()
            check(lib().fm_sur_flip(_p(L.wb), _p(L.wf), _stream()), "fm_sur_flip")
        hs = [self._buf("h%d" % k, B, n) for k in range(self.n_blocks + 1)]
        # projection
        self._wgrad(B, n, hs[-1], dy, Ls[-1])
        dh = self._buf("dhA", B, n)
        self._conv(B, n, dy, Ls[-1], weights=Ls[-1].wf, bias=False, y_out=dh)
        # residual blocks, last to first
        for k in reversed(range(self.n_blocks)):
            c1, c2 = Ls[1 + 2 * k], Ls[2 + 2 * k]
            a1, z1 = self._buf("a1_%d" % k, B, n), self._buf("z1_%d" % k, B, n)
            self._wgrad(B, n, a1, dh, c2)
            dz1 = self._buf("dz1", B, n)
            self._conv(B, n, dh, c2, weights=c2.wf, bias=False, gate=z1, y_out=dz1)
            self._wgrad(B, n, hs[k], dz1, c1)
            dh_prev = self._buf("dhB" if k % 2 == 0 else "dhA2", B, n)
            self._conv(B, n, dz1, c1, weights=c1.wf, bias=False, resid=dh, y_out=dh_prev)
            dh = dh_prev
        # lift: dz0 = dh * gelu'(z0)
        z0 = self._buf("z0", B, n)
        dz0 = self._buf("dz0", B, n)
        check(lib().fm_sur_gelu_bwd(dz0.numel(), _p(dh), _p(z0), _p(dz0), _stream()),
              "fm_sur_gelu_bwd")
        self._wgrad(B, n, xpad, dz0, Ls[0])
        return loss / count

    def _wgrad(self, B, n, x, dy, L: _Layer):
        check(lib().fm_conv3x3_wgrad_bf16(B, n, n, C, _p(x), _p(dy), _p(L.gw), _p(self.err),
                                          _stream()), "fm_conv3x3_wgrad_bf16")
        check(lib().fm_sur_bias_grad(B, n, _p(dy), _p(L.gb), _stream()), "fm_sur_bias_grad")

    def adam_step(self, lr: float = 1e-3, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
        self.step_count += 1
        for L in self.layers:
            check(lib().fm_sur_adam(_p(L.w), _p(L.gw), _p(L.mw), _p(L.vw), _p(L.wb), _p(L.b),
                                    _p(L.gb), _p(L.mb), _p(L.vb), lr, b1, b2, eps,
                                    self.step_count, L.mask_co, _stream()), "fm_sur_adam")

    def train_step(self, U0, V0, F, K, U1, V1, lr: float = 1e-3) -> torch.Tensor:
        loss = self.loss_and_grads(U0, V0, F, K, U1, V1)
        self.adam_step(lr)
        return loss

    def check_errors(self):
        if int(self.err.item()) != 0:
            raise RuntimeError("a tensor-core wait gave up in a surrogate kernel")
