"""The surrogate's tcgen05 convolution kernels and training gradients against
the CPU float64 reference (oracle/surrogate_ref.py).

Inputs and weights are rounded to bf16 before both paths see them, so the
single-convolution checks isolate accumulation order (fp32 on the tensor
cores): tolerance 1e-4 of the magnitude scale.  Whole-network gradients also
differ by the bf16 rounding of every intermediate activation on the GPU:
checked by relative norm error < 5e-2 and cosine similarity > 0.995 per layer.
"""
import ctypes

import numpy as np
import pytest
import torch

from formura_gb300 import _lib, inits
from formura_gb300.surrogate import C, Surrogate
from oracle import surrogate_ref as ref

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def pad_periodic(x):
    """[B][n][n][C] -> [B][n+2][n+2][C] with the periodic halo."""
    rows = torch.cat([x[:, -1:], x, x[:, :1]], 1)
    return torch.cat([rows[:, :, -1:], rows, rows[:, :, :1]], 2)


def bf16r(t):
    return t.to(torch.bfloat16).to(torch.float64)


@pytest.fixture(params=[2, 1, 0], ids=["tma", "resident", "gather"])
def conv_kernel(request):
    """The forward-convolution kernels: the weight-resident shifted-descriptor
    kernel with TMA staging and mbarrier-chained steps, the same with cp.async
    staging and a barrier per tile, and the per-tap gather kernel."""
    L = _lib.lib()
    L.fm_tune_set(b"conv.kernel", request.param)
    yield request.param
    L.fm_tune_clear()


@pytest.mark.parametrize("B,n", [(2, 16), (1, 32), (4, 8), (3, 40)])
def test_conv_fwd_matches_cpu(cuda_device, conv_kernel, B, n):
    if conv_kernel == 0 and (B * n * n) % 128:
        pytest.skip("the gather kernel needs B*H*W % 128 == 0")
    g = torch.Generator().manual_seed(B * 100 + n)
    x = bf16r(torch.randn(B, n, n, C, generator=g, dtype=torch.float64))
    w = bf16r(torch.randn(C, 9, C, generator=g, dtype=torch.float64) * 0.05)
    b = torch.randn(C, generator=g, dtype=torch.float64) * 0.1
    want = ref.conv(x, w, b)
    xg = pad_periodic(x).to(torch.bfloat16).cuda().contiguous()
    wg = w.to(torch.bfloat16).cuda().contiguous()
    bg = b.float().cuda()
    y = torch.empty(B, n, n, C, device="cuda")
    ypad = torch.zeros(B, n + 2, n + 2, C, dtype=torch.bfloat16, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = _lib.lib().fm_conv3x3_fwd_bf16(B, n, n, C, _p(xg), _p(wg), _p(bg), None, None, 0, None,
                                        _p(ypad), _p(y), _p(err),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, "fm_conv3x3_fwd_bf16")
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    scale = ref.conv(x.abs(), w.abs()).abs() + 1e-3
    assert ((y.double().cpu() - want).abs() <= 1e-4 * scale).all()
    # the padded bf16 output carries the periodic halo
    assert torch.equal(ypad.cpu(), pad_periodic(y.cpu().to(torch.bfloat16).double()).to(torch.bfloat16))


def test_conv_kernels_agree_bitwise(cuda_device):
    """The three forward kernels issue the same MMA sequence: identical outputs
    (the TMA kernel staging the residual too)."""
    B, n = 2, 64
    g = torch.Generator().manual_seed(5)
    x = pad_periodic(torch.randn(B, n, n, C, generator=g)).to(torch.bfloat16).cuda().contiguous()
    w = (torch.randn(C, 9, C, generator=g) * 0.05).to(torch.bfloat16).cuda().contiguous()
    b = (torch.randn(C, generator=g) * 0.1).cuda()
    res = torch.randn(B, n + 2, n + 2, C, generator=g).to(torch.bfloat16).cuda()
    L = _lib.lib()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = []
    try:
        for k in (0, 1, 2):
            L.fm_tune_set(b"conv.kernel", k)
            y = torch.zeros(B, n + 2, n + 2, C, dtype=torch.bfloat16, device="cuda")
            z = torch.zeros_like(y)
            yf = torch.zeros(B, n, n, C, device="cuda")
            _lib.check(L.fm_conv3x3_fwd_bf16(B, n, n, C, _p(x), _p(w), _p(b), _p(res), _p(res), 1,
                                             _p(z), _p(y), _p(yf), _p(err), s), "conv")
            outs.append((y, z, yf))
    finally:
        L.fm_tune_clear()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    for a, c in zip(outs[0], outs[1]):
        assert torch.equal(a, c)


def test_conv_wgrad_and_dgrad_match_autograd(cuda_device):
    B, n = 2, 16
    g = torch.Generator().manual_seed(7)
    x = bf16r(torch.randn(B, n, n, C, generator=g, dtype=torch.float64))
    w = bf16r(torch.randn(C, 9, C, generator=g, dtype=torch.float64) * 0.05)
    dy = bf16r(torch.randn(B, n, n, C, generator=g, dtype=torch.float64))
    xr, wr = x.clone().requires_grad_(True), w.clone().requires_grad_(True)
    ref.conv(xr, wr).backward(dy)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    xg = pad_periodic(x).to(torch.bfloat16).cuda().contiguous()
    dyg = pad_periodic(dy).to(torch.bfloat16).cuda().contiguous()
    dwt = torch.zeros(9, C, C, device="cuda")
    L = _lib.lib()
    _lib.check(L.fm_conv3x3_wgrad_bf16(B, n, n, C, _p(xg), _p(dyg), _p(dwt), _p(err), s), "wgrad")
    wb = w.to(torch.bfloat16).cuda().contiguous()
    wf = torch.empty_like(wb)
    _lib.check(L.fm_sur_flip(_p(wb), _p(wf), s), "flip")
    dx = torch.empty(B, n, n, C, device="cuda")
    _lib.check(L.fm_conv3x3_fwd_bf16(B, n, n, C, _p(dyg), _p(wf), None, None, None, 0, None, None,
                                     _p(dx), _p(err), s), "dgrad")
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    gw = dwt.double().cpu().permute(2, 0, 1)          # [t][ci][co] -> [co][t][ci]
    assert torch.allclose(gw, wr.grad, rtol=1e-4, atol=1e-4 * wr.grad.abs().max().item())
    assert torch.allclose(dx.double().cpu(), xr.grad, rtol=1e-4,
                          atol=1e-4 * xr.grad.abs().max().item())


def test_network_gradients_match_cpu_oracle(cuda_device):
    B, N = 2, 32
    sizes = [N] * B
    U0, V0 = inits.gs2d_ensemble_state(sizes, seed=4)
    U0 = U0.reshape(B, N, N)
    V0 = V0.reshape(B, N, N)
    rng = np.random.default_rng(0)
    U1 = U0 + 0.01 * rng.standard_normal(U0.shape).astype(np.float32)
    V1 = V0 + 0.01 * rng.standard_normal(V0.shape).astype(np.float32)
    F = np.array([0.03, 0.05], np.float32)
    K = np.array([0.055, 0.065], np.float32)
    net = Surrogate(seed=3)
    for L in net.layers:   # non-trivial biases
        L.b.copy_(torch.randn(C, generator=torch.Generator().manual_seed(1)).cuda() * 0.05)
        if L.mask_co > 0:
            L.b[L.mask_co:] = 0
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    loss = net.loss_and_grads(t(U0), t(V0), t(F), t(K), t(U1), t(V1))
    torch.cuda.synchronize()
    net.check_errors()
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).double()  # noqa: E731
    ws = [L.wb.double().cpu() for L in net.layers]
    bs = [L.b.double().cpu() for L in net.layers]
    lref, gws, gbs = ref.loss_and_grads(bf16r(d(U0)), bf16r(d(V0)), d(F), d(K), d(U1), d(V1), ws,
                                         bs)
    assert abs(loss.item() - lref) < 2e-2 * lref
    for i, (L, gw, gb) in enumerate(zip(net.layers, gws, gbs)):
        got = L.gw.double().cpu().permute(2, 0, 1)
        rel = ((got - gw).norm() / gw.norm()).item()
        cos = (torch.dot(got.flatten(), gw.flatten()) / (got.norm() * gw.norm())).item()
        assert rel < 5e-2 and cos > 0.995, (i, rel, cos)
        relb = ((L.gb.double().cpu() - gb).norm() / (gb.norm() + 1e-30)).item()
        assert relb < 5e-2, (i, relb)


def test_training_reduces_loss(cuda_device):
    """A few Adam steps on a fixed batch of true 16-step pairs reduce the loss."""
    from formura_gb300 import kernels

    B, N = 8, 64
    sizes, F, K = inits.gs2d_ensemble(B, seed=11, sizes=(N,))
    e = kernels.Ensemble(sizes, F, K)
    U, V = inits.gs2d_ensemble_state(sizes, seed=2)
    U, V = torch.from_numpy(U).cuda(), torch.from_numpy(V).cuda()
    wU, wV = torch.empty_like(U), torch.empty_like(V)
    e.forward(U, V, wU, wV, 200, use_graph=False)  # develop some structure
    U0, V0 = U.clone().view(B, N, N), V.clone().view(B, N, N)
    e.forward(U, V, wU, wV, 16, use_graph=False)
    U1, V1 = U.view(B, N, N), V.view(B, N, N)
    Ft = torch.tensor(F, dtype=torch.float32, device="cuda")
    Kt = torch.tensor(K, dtype=torch.float32, device="cuda")
    net = Surrogate(seed=0)
    first = net.train_step(U0, V0, Ft, Kt, U1, V1, lr=1e-3).item()
    for _ in range(60):
        last = net.train_step(U0, V0, Ft, Kt, U1, V1, lr=1e-3).item()
    net.check_errors()
    assert last < 0.2 * first, (first, last)


WEIGHTS = __import__("pathlib").Path(__file__).resolve().parents[1] / "formura_gb300" / \
    "weights" / "gs2d_surrogate.npz"


def test_trained_network_beats_the_method_without_it(cuda_device):
    """What the trained network gains: on held-out pairs its 16-step prediction
    is far closer to the stencil's than persistence (the no-model guess
    S(t+16) = S(t)) and than the untrained network."""
    from formura_gb300 import surrogate_run as sr

    net = Surrogate(seed=0)
    untrained = sr.jump_error(net, n_inst=8, N=128, seed=4242)
    net.load_npz(WEIGHTS)
    trained = sr.jump_error(net, n_inst=8, N=128, seed=4242)
    assert trained["state_rel_l2"] < trained["state_rel_l2_persistence"] / 5, trained
    assert trained["state_rel_l2"] < untrained["state_rel_l2"] / 5, (trained, untrained)


def test_fallback_reproduces_the_plain_stencil(cuda_device):
    """With the anchor criterion unmet the run falls back, and the result is the
    plain FP32 stencil's bit for bit; with the criterion disabled it is not."""
    from formura_gb300 import surrogate_run as sr

    B, N = 2, 128
    sizes, F, K = inits.gs2d_ensemble(B, seed=77, sizes=(N,))
    U0, V0 = inits.gs2d_ensemble_state(sizes, seed=77)
    Ft = torch.tensor(F, dtype=torch.float32, device="cuda")
    Kt = torch.tensor(K, dtype=torch.float32, device="cuda")
    net = Surrogate(seed=0)
    net.load_npz(WEIGHTS)

    def fresh():
        return (torch.from_numpy(U0).cuda().view(B, N, N).clone(),
                torch.from_numpy(V0).cuda().view(B, N, N).clone())

    Up, Vp = fresh()
    sr.run_plain(Up, Vp, Ft, Kt, 512)
    Us, Vs = fresh()
    info = sr.run_with_surrogate(net, Us, Vs, Ft, Kt, 512, 256, tol=1e-12)
    assert all(info["fallback"])
    assert torch.equal(Us, Up) and torch.equal(Vs, Vp)
    Un, Vn = fresh()
    info = sr.run_with_surrogate(net, Un, Vn, Ft, Kt, 512, 256, tol=1e30)
    assert not any(info["fallback"])
    assert not torch.equal(Un, Up)
    # the unchecked surrogate run still tracks the stencil to a few percent
    rel = torch.sqrt(((Un - Up) ** 2).sum() + ((Vn - Vp) ** 2).sum()) / \
        torch.sqrt((Up ** 2).sum() + (Vp ** 2).sum())
    assert rel.item() < 0.1, rel.item()
