"""GPU parity of the persistent 2D diffusion kernel (bit-exact)."""
import numpy as np
import pytest
import torch

from formura_gb300 import inits, kernels
from formura_gb300.runtime import load_program
from oracle import oracle
from tests.bits import same_bits

pytestmark = pytest.mark.gpu


def run(d0, steps, dev, coef=0.4):
    d = torch.from_numpy(d0).to(dev)
    w = torch.empty_like(d)
    kernels.diff2d_f64_forward(d, w, coef, steps)
    torch.cuda.synchronize()
    return d.cpu().numpy()


@pytest.mark.parametrize("shape,steps", [((256, 256), 1000), ((64, 64), 101), ((1, 32), 9),
                                         ((37, 96), 50), ((1024, 512), 20)])
def test_diff2d_bit_exact(cuda_device, shape, steps):
    d0 = inits.diffusion_2d(*shape, seed=17)
    got = run(d0, steps, cuda_device)
    want = oracle.diff2d_f64(d0, steps, 0.4, 1.0)
    assert same_bits(got, want)


def test_diffusion_program_drop_in(cuda_device):
    prog = load_program("diffusion_2d")
    prog.init()
    d0 = inits.diffusion_2d(256, 256, seed=1)
    prog.state["dens"][...] = d0
    prog.forward()
    assert prog.navi.time_step == 1000
    want = oracle.diff2d_f64(d0, 1000, 0.4, 1.0)
    assert same_bits(prog.state["dens"], want)
    tot = prog.conserved_totals()
    assert abs(tot[0] - d0.sum()) < 1e-9 * d0.sum()


@pytest.mark.parametrize("tb", [0, 2, 4, 8])
@pytest.mark.parametrize("shape,steps", [((256, 256), 37), ((40, 64), 13), ((1, 32), 5),
                                         ((19, 96), 9)])
def test_diffusion_temporal_blocking_bit_exact(cuda_device, tb, shape, steps):
    """K steps per grid barrier on shared-memory tiles with a K-cell halo
    (diffusion.tb = K; 0 = one step per barrier), the exact x*0.5 and coef*g
    on the integer pipes: bit-exact for every K, step counts that are not
    multiples of K, and shapes that are not multiples of the 16 x 32 tile."""
    from formura_gb300 import _lib

    L = _lib.lib()
    try:
        L.fm_tune_set(b"diff2d.tb", tb)
        d0 = inits.diffusion_2d(*shape, seed=steps)
        d = torch.from_numpy(d0).cuda()
        kernels.diff2d_f64_forward(d, torch.empty_like(d), 0.1, steps)
        want = oracle.diff2d_f64(d0, steps, Dt=0.1, Dx=1.0)
        assert same_bits(d.cpu().numpy(), want)
    finally:
        L.fm_tune_clear()
