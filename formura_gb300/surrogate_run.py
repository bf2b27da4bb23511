"""Training data, training loop and the surrogate-accelerated run with the
plain stencil as fallback and as the reference for its error.

Training pairs come from the batched solver (the uneven-ensemble kernel of
fm_gs2d.cu): a pool of periodic 2D Gray-Scott instances with F ~ U[0.02, 0.06],
k ~ U[0.05, 0.07] and seeded random-square starts is advanced on the GPU;
every iteration takes the pool's current state and its state 16 steps later
as one batch of (input, target) pairs, and the pool is re-seeded with new
parameters and burn-in lengths every `reseed` iterations.

:func:`run_with_surrogate` advances a batch of instances `steps` steps.  Each
`anchor`-step segment runs `anchor/16 - 1` network jumps and then re-anchors
with 16 plain FP32 stencil steps; the network's own jump from the same state
is compared with those stencil steps, and an instance whose per-segment error
estimate (16 x the jump discrepancy) exceeds `tol` falls back to the plain
stencil — its segment is recomputed by the stencil from the segment's start
and it stays on the stencil.
"""
from __future__ import annotations

import time
from typing import Dict, Optional

import numpy as np
import torch

from . import inits, kernels
from .surrogate import JUMP, Surrogate

DU, DV, DT, DX = 2e-5, 1e-5, 1.0, 0.01


class PairStream:
    """Pairs (S_t, S_t+16) from a pool of `n_inst` N x N instances."""

    def __init__(self, n_inst: int = 64, N: int = 128, seed: int = 1, reseed: int = 100,
                 burn_in=(0, 2000)):
        self.n_inst, self.N, self.seed, self.reseed = n_inst, N, seed, reseed
        self.burn_in = burn_in
        self.it = 0
        self.generation = 0
        self._new_pool()

    def _new_pool(self):
        s = self.seed * 7919 + self.generation
        sizes, F, K = inits.gs2d_ensemble(self.n_inst, seed=s, sizes=(self.N,))
        self.F = torch.tensor(F, dtype=torch.float32, device="cuda")
        self.K = torch.tensor(K, dtype=torch.float32, device="cuda")
        self.ens = kernels.Ensemble(sizes, F, K, DU, DV, DT, DX)
        U, V = inits.gs2d_ensemble_state(sizes, seed=s)
        self.U = torch.from_numpy(U).cuda()
        self.V = torch.from_numpy(V).cuda()
        self.wU, self.wV = torch.empty_like(self.U), torch.empty_like(self.V)
        r = inits.uniform(s, 1)[0]
        b = int(self.burn_in[0] + r * (self.burn_in[1] - self.burn_in[0]))
        self.ens.forward(self.U, self.V, self.wU, self.wV, b, use_graph=False)
        self.generation += 1

    def next(self):
        if self.it and self.it % self.reseed == 0:
            self.ens.close()
            self._new_pool()
        self.it += 1
        B, N = self.n_inst, self.N
        U0 = self.U.clone().view(B, N, N)
        V0 = self.V.clone().view(B, N, N)
        self.ens.forward(self.U, self.V, self.wU, self.wV, JUMP, use_graph=True)
        return U0, V0, self.F, self.K, self.U.view(B, N, N), self.V.view(B, N, N)


def train(net: Surrogate, iters: int, n_inst: int = 64, N: int = 128, lr: float = 3e-4,
          seed: int = 1, time_budget: Optional[float] = None, log_every: int = 100,
          warmup: int = 300, burn_in=(0, 2000)) -> Dict:
    """Adam with linear warm-up and cosine decay; returns the loss history.
    Pairs come from `n_inst` N x N instances whose pool is re-seeded with a
    burn-in drawn from `burn_in` steps."""
    stream = PairStream(n_inst, N, seed=seed, burn_in=burn_in)
    hist = []
    t0 = time.time()
    done = 0
    for i in range(iters):
        lr_i = lr * min(1.0, (i + 1) / warmup) * 0.5 * (1.0 + np.cos(np.pi * i / max(1, iters)))
        U0, V0, F, K, U1, V1 = stream.next()
        loss = net.train_step(U0, V0, F, K, U1, V1, lr=max(lr_i, lr * 0.02))
        done += 1
        if i % log_every == 0 or i == iters - 1:
            hist.append((i, float(loss.item())))
        if time_budget is not None and time.time() - t0 > time_budget:
            break
    torch.cuda.synchronize()
    net.check_errors()
    return {"iters": done, "pairs": done * n_inst, "seconds": time.time() - t0, "loss": hist}


def jump_error(net: Surrogate, n_inst: int = 16, N: int = 128, seed: int = 99) -> Dict:
    """Relative L2 error of one network jump against 16 stencil steps, and the
    same for the no-model baseline (persistence: S_t+16 ~ S_t), on held-out
    pairs."""
    s = PairStream(n_inst, N, seed=seed, reseed=10 ** 9)
    U0, V0, F, K, U1, V1 = s.next()
    Up, Vp = U0.clone(), V0.clone()
    net.predict(Up, Vp, F, K)
    torch.cuda.synchronize()

    def rel(a, b, c, d):
        num = torch.linalg.vector_norm(a - b) ** 2 + torch.linalg.vector_norm(c - d) ** 2
        den = torch.linalg.vector_norm(b) ** 2 + torch.linalg.vector_norm(d) ** 2
        return float(torch.sqrt(num / den).item())

    return {
        "state_rel_l2": rel(Up, U1, Vp, V1),
        "state_rel_l2_persistence": rel(U0, U1, V0, V1),
        "increment_rel_l2": rel(Up - U0, U1 - U0, Vp - V0, V1 - V0),
    }


def run_plain(U, V, F, K, steps: int, ens: Optional[kernels.Ensemble] = None):
    """The plain FP32 stencil on a batch of equal-size instances (one
    persistent launch); U, V float32 [B][N][N] advanced in place."""
    B, N = U.shape[0], U.shape[1]
    own = ens is None
    if own:
        ens = kernels.Ensemble([N] * B, F.tolist(), K.tolist(), DU, DV, DT, DX)
    fu, fv = U.view(-1), V.view(-1)
    ens.forward(fu, fv, torch.empty_like(fu), torch.empty_like(fv), steps, use_graph=False)
    if own:
        ens.close()


def run_with_surrogate(net: Surrogate, U, V, F, K, steps: int = 4096, anchor: int = 256,
                       tol: float = 1e-2) -> Dict:
    """Advance U, V (float32 [B][N][N], in place) by `steps` with the
    surrogate, re-anchoring and falling back as described in the module doc."""
    assert steps % anchor == 0 and anchor % JUMP == 0
    B, N = U.shape[0], U.shape[1]
    Fl, Kl = F.tolist(), K.tolist()
    ens_all = kernels.Ensemble([N] * B, Fl, Kl, DU, DV, DT, DX)
    fallback = torch.zeros(B, dtype=torch.bool, device=U.device)
    jumps = anchor // JUMP - 1
    est = []
    for seg in range(steps // anchor):
        U0, V0 = U.clone(), V.clone()
        for _ in range(jumps):
            net.predict(U, V, F, K)
        # network's last jump vs the plain stencil from the same state
        Us, Vs = U.clone(), V.clone()
        net.predict(Us, Vs, F, K)
        run_plain(U, V, F, K, JUMP, ens_all)
        num = torch.linalg.vector_norm((Us - U).view(B, -1), dim=1) + \
            torch.linalg.vector_norm((Vs - V).view(B, -1), dim=1)
        den = torch.linalg.vector_norm(U.view(B, -1), dim=1) + \
            torch.linalg.vector_norm(V.view(B, -1), dim=1)
        e = (num / den) * (anchor // JUMP)
        est.append(e.max().item())
        bad = (e > tol) | fallback
        if bool(bad.any()):
            # fall back: recompute the whole segment of those instances with the stencil
            idx = torch.nonzero(bad).flatten()
            Ub, Vb = U0[idx].contiguous(), V0[idx].contiguous()
            run_plain(Ub, Vb, F[idx], K[idx], anchor)
            U[idx] = Ub
            V[idx] = Vb
            fallback |= bad
    ens_all.close()
    net.check_errors()
    return {"fallback": fallback.cpu().numpy().tolist(), "max_segment_error_estimate": est}
