"""The autotuner (formura_gb300/autotune.py): its pick is one of the
candidates, runs bit-exact against the oracle as the tuned default, and a
second call is answered from the cache without timing anything."""
import numpy as np
import pytest
import torch

from formura_gb300 import _lib, autotune, inits, kernels
from oracle import oracle
from tests.bits import same_bits

pytestmark = pytest.mark.gpu

GS = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)


@pytest.fixture()
def private_cache(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("FORMURA_TUNE_CACHE", str(path))
    yield path
    _lib.lib().fm_tune_clear()


def test_tune_ensemble_pick_runs_bit_exact_and_is_cached(cuda_device, private_cache, monkeypatch):
    sizes = [64, 128, 96, 64, 256]
    F = [0.02, 0.03, 0.045, 0.05, 0.06]
    k = [0.05, 0.06, 0.062, 0.065, 0.07]
    cands = [(64, 2), (32, 4), (1, 2), (1, 4)]
    res = autotune.tune_ensemble(sizes, F, k, sample_steps=16, candidates=cands)
    assert (res["tile"], res["tb"]) in cands
    assert len(res["timings"]) == len(cands) and private_cache.exists()
    # the winner is now the default (tile 0, tb 0 = tuned): bit-exact per instance
    steps = 30
    e = kernels.Ensemble(sizes, F, k, 2e-5, 1e-5, 1.0, 0.01)
    U0, V0 = inits.gs2d_ensemble_state(sizes, seed=12)
    U, V = torch.from_numpy(U0).cuda(), torch.from_numpy(V0).cuda()
    e.forward(U, V, torch.empty_like(U), torch.empty_like(V), steps, use_graph=True)
    e.status()
    Uc = U.cpu().numpy()
    for i, n in enumerate(sizes):
        o = int(e.offsets[i])
        uo, _ = oracle.gs2d_f32(U0[o:o + n * n].reshape(n, n), V0[o:o + n * n].reshape(n, n),
                                steps, F[i], k[i], 2e-5, 1e-5, 1.0, 0.01)
        assert same_bits(Uc[o:o + n * n].reshape(n, n), uo), i
    e.close()

    # second call: a cache hit, nothing is built or timed
    def no_build(*a, **kw):
        raise AssertionError("cache miss: the tuner timed a candidate again")

    monkeypatch.setattr(autotune.kernels, "Ensemble", no_build)
    assert autotune.tune_ensemble(sizes, F, k, sample_steps=16, candidates=cands) == res


def test_tune_gs3d_f32k_pick_runs_bit_exact_and_is_cached(cuda_device, private_cache, monkeypatch):
    shape = (48, 40, 64)
    res = autotune.tune_gs3d_f32k(shape, sample_steps=6)
    assert res["kernel"] in (0, 1, 2) and res["tb"] in (1, 2, 3, 4)
    U0, V0 = inits.gray_scott_3d(*shape, seed=6, ncubes=2, side=8)
    U = torch.from_numpy(U0.astype(np.float32)).cuda()
    V = torch.from_numpy(V0.astype(np.float32)).cuda()
    cU, cV = torch.zeros_like(U), torch.zeros_like(V)
    w = torch.empty(4 * U.numel(), dtype=torch.float32, device="cuda")
    kernels.gs3d_f32k_tb_forward(U, V, cU, cV, w, kernels.gs_params(**GS), 11)  # tuned tb
    Z = np.zeros(shape, np.float32)
    want = oracle.gs3d_f32k_fast(U0.astype(np.float32), V0.astype(np.float32), Z, Z, 11, **GS)
    assert same_bits(U.cpu().numpy(), want[0]) and same_bits(V.cpu().numpy(), want[1])

    def no_run(*a, **kw):
        raise AssertionError("cache miss: the tuner timed a candidate again")

    monkeypatch.setattr(autotune.kernels, "gs3d_f32k_tb_forward", no_run)
    assert autotune.tune_gs3d_f32k(shape, sample_steps=6) == res
