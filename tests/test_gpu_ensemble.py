"""Uneven 2D Gray-Scott ensembles in one persistent launch: bit-exact per
instance against the oracle's binary32 pearson-2d DAG, for every tile (32, 64; 1 = the
wavefront strips) and
blocking depth, with and without the captured CUDA graph."""
import numpy as np
import pytest
import torch

from formura_gb300 import inits, kernels
from oracle import oracle
from tests.bits import same_bits

pytestmark = pytest.mark.gpu

DU, DV, DT, DX = 2e-5, 1e-5, 1.0, 0.01


def oracle_instance(u0, v0, n, F, k, steps):
    return oracle.gs2d_f32(u0.reshape(n, n), v0.reshape(n, n), steps, F, k, DU, DV, DT, DX)


def run_ensemble(sizes, F, k, steps, tile, tb, use_graph, seed=3, calls=1):
    e = kernels.Ensemble(sizes, F, k, DU, DV, DT, DX, tile=tile, tb=tb)
    U0, V0 = inits.gs2d_ensemble_state(sizes, seed=seed)
    U = torch.from_numpy(U0).cuda()
    V = torch.from_numpy(V0).cuda()
    wU, wV = torch.empty_like(U), torch.empty_like(V)
    for _ in range(calls):
        e.forward(U, V, wU, wV, steps, use_graph=use_graph)
    e.status()
    torch.cuda.synchronize()
    return e, U0, V0, U.cpu().numpy(), V.cpu().numpy()


@pytest.mark.parametrize("tile,tb", [(64, 4), (32, 1), (32, 8), (64, 8), (64, 2), (32, 3),
                                     (1, 4), (1, 1), (1, 3), (1, 6), (1, 8), (1, 2)])
def test_ensemble_bit_exact(cuda_device, tile, tb):
    sizes = [64, 128, 32, 100, 64, 256, 48]   # includes sizes that are not tile multiples
    F = [0.02, 0.03, 0.04, 0.05, 0.06, 0.035, 0.045]
    k = [0.05, 0.055, 0.06, 0.065, 0.07, 0.052, 0.061]
    steps = 37                                # not a multiple of tb
    e, U0, V0, U, V = run_ensemble(sizes, F, k, steps, tile, tb, use_graph=False)
    for i, n in enumerate(sizes):
        o = e.offsets[i]
        uo, vo = oracle_instance(U0[o:o + n * n], V0[o:o + n * n], n, F[i], k[i], steps)
        assert same_bits(U[o:o + n * n].reshape(n, n), uo), (i, n)
        assert same_bits(V[o:o + n * n].reshape(n, n), vo), (i, n)
    e.close()


def test_ensemble_graph_replay_matches(cuda_device):
    sizes, F, k = inits.gs2d_ensemble(24, seed=5, sizes=(64, 128, 256))
    e1, U0, V0, Ua, Va = run_ensemble(sizes, F, k, 40, 64, 4, use_graph=False, calls=2)
    e2, _, _, Ub, Vb = run_ensemble(sizes, F, k, 40, 64, 4, use_graph=True, calls=2)
    assert np.array_equal(Ua, Ub) and np.array_equal(Va, Vb)
    i = 3
    n, o = sizes[i], e1.offsets[i]
    uo, vo = oracle_instance(U0[o:o + n * n], V0[o:o + n * n], n, F[i], k[i], 80)
    assert same_bits(Ub[o:o + n * n].reshape(n, n), uo)
    e1.close()
    e2.close()


def test_ensemble_rejects_unsupported_tiles(cuda_device):
    from formura_gb300._lib import FormuraError

    with pytest.raises(FormuraError):
        kernels.Ensemble([64], [0.04], [0.06], tile=128, tb=2)


def test_single_instance_kernel_matches_oracle(cuda_device):
    u0, v0 = inits.gray_scott_2d_square(96, 160, seed=2)
    u0, v0 = u0.astype(np.float32), v0.astype(np.float32)
    U, V = torch.from_numpy(u0).cuda(), torch.from_numpy(v0).cuda()
    kernels.gs2d_f32_forward(U, V, torch.empty_like(U), torch.empty_like(V),
                             kernels.gs_params(0.04, 0.06, DU, DV, DT, DX), 25)
    uo, vo = oracle.gs2d_f32(u0, v0, 25, 0.04, 0.06, DU, DV, DT, DX)
    assert same_bits(U.cpu().numpy(), uo) and same_bits(V.cpu().numpy(), vo)
