"""GPU parity of the 3D MHD kernels (examples/3d-mhd-rk4.fmr form).

FP64 path: bit-exact against the CPU oracle's restatement of the DAG.  FP32
path (binary32 bulk, FP64 energy update): scored by its error against the
FP64 oracle, as the precision form asks; tolerance written below.
"""
import numpy as np
import pytest
import torch

from formura_gb300 import inits, kernels
from oracle import oracle
from tests.bits import same_bits

pytestmark = pytest.mark.gpu


def gpu_run(fields, steps, dtype):
    n = fields[0].shape[0]
    t = [torch.from_numpy(np.ascontiguousarray(f)).to(dtype).cuda() for f in fields]
    work = torch.empty(18 * n ** 3, dtype=dtype, device="cuda")
    kernels.mhd_forward(t, work, steps)
    torch.cuda.synchronize()
    return t, [x.double().cpu().numpy() for x in t]


@pytest.mark.parametrize("n,steps", [(16, 3), (24, 2), (32, 2)])
def test_mhd_f64_bit_exact(cuda_device, n, steps):
    f0 = inits.mhd_3d(n, seed=n)
    _, got = gpu_run(f0, steps, torch.float64)
    want = oracle.mhd_f64(f0, steps)
    for name, g, w in zip(inits.MHD_FIELDS, got, want):
        assert same_bits(g, w), name


def test_mhd_f64_strong_perturbation_bit_exact(cuda_device):
    # large amplitudes switch the artificial-viscosity limiter on, and a
    # density trough just above -0.9 makes the floor fmax(dens, -0.9) act, so
    # every branch of the finishing kernel is exercised
    n = 16
    f0 = inits.mhd_3d(n, seed=3, amp=0.3)
    x = np.arange(n) / n
    f0[0] = (-0.85 + 0.06 * np.cos(2 * np.pi * x))[:, None, None] * np.ones((n, n, n))
    f0[1] = f0[1] + 0.5 * np.sin(2 * np.pi * x)[:, None, None]   # converging flow into x = 0.5
    _, got = gpu_run(f0, 2, torch.float64)
    want = oracle.mhd_f64(f0, 2)
    assert all(np.isfinite(w).all() for w in want)
    assert (want[0] == -0.9).any(), "density floor not exercised"
    for name, g, w in zip(inits.MHD_FIELDS, got, want):
        assert same_bits(g, w), name


def test_mhd_f64_signed_zeros_bit_exact(cuda_device):
    """Fields that are exactly +0 or -0 everywhere (vy = -0, Bz = +0, Psi = -0)
    make the Kronecker-delta term -(0*Psi) + x and the products of zeros
    produce signed zeros; compared bit for bit, the sign of zero included."""
    n = 12
    f0 = [np.array(f) for f in inits.mhd_3d(n, seed=7)]
    f0[2] = np.full((n, n, n), -0.0)
    f0[6] = np.zeros((n, n, n))
    f0[8] = np.full((n, n, n), -0.0)
    _, got = gpu_run(f0, 2, torch.float64)
    want = oracle.mhd_f64(f0, 2)
    for name, g, w in zip(inits.MHD_FIELDS, got, want):
        assert np.array_equal(g.view(np.int64), np.ascontiguousarray(w).view(np.int64)), name


def test_mhd_f32_error_against_f64(cuda_device):
    n, steps = 32, 40
    f0 = inits.mhd_3d(n, seed=5)
    _, got = gpu_run(f0, steps, torch.float32)
    want = oracle.mhd_f64(f0, steps)
    for name, g, w in zip(inits.MHD_FIELDS, got, want):
        scale = max(np.abs(w).max(), 1e-30)
        err = np.abs(g - w).max() / scale
        # binary32 bulk: rounding ~6e-8 relative per operation, a few hundred
        # operations per step, 40 steps; s (the heated entropy) starts at 0
        assert err < 5e-4, (name, err)


def test_mhd_totals_conserve_mass(cuda_device):
    n = 32
    f0 = inits.mhd_3d(n, seed=2)
    f0[0] = 0.01 * np.sin(2 * np.pi * np.arange(n) / n)[:, None, None] * np.ones((n, n, n))
    t, _ = gpu_run(f0, 0, torch.float64)
    tot0 = kernels.mhd_totals(t).cpu().numpy()
    work = torch.empty(18 * n ** 3, dtype=torch.float64, device="cuda")
    kernels.mhd_forward(t, work, 10)
    tot1 = kernels.mhd_totals(t).cpu().numpy()
    tot1b = kernels.mhd_totals(t).cpu().numpy()
    assert np.array_equal(tot1, tot1b)                 # deterministic
    assert abs(tot1[0] - tot0[0]) < 1e-12 * n ** 3     # sum of dens conserved
    # kinetic + magnetic energy exchanges with pressure and is dissipated by the
    # artificial viscosity and the Psi damping: finite and not growing
    assert np.isfinite(tot1).all() and tot1[1] < 1.001 * tot0[1]


@pytest.mark.parametrize("n", [12, 40])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_mhd_kernel_variants_agree(cuda_device, n, dtype):
    """The stage kernels (mhd.stage: 2 x-marching with a register ring, 1
    shared-memory tiled, 0 per-point), the finish kernels (mhd.finish: 2
    x-marching sharing slopes and faces of all fields per plane, several x
    chunks; 0 per-point) and, for FP64, the integer-pipe arithmetic
    (mhd.soft = 1) against the FP64 instructions (0) evaluate the same
    expressions: identical bits, also for sizes that are not multiples of the
    32 x 8 tile."""
    from formura_gb300 import _lib

    f0 = inits.mhd_3d(n, seed=11, amp=0.05)
    outs = []
    L = _lib.lib()
    try:
        for kern, fin, xc, soft in ((0, 0, 0, 0), (1, 2, 0, 1), (1, 2, 5, 0), (1, 2, 3, 1),
                                    (0, 2, 1, 1), (2, 0, 16, 1), (2, 0, 5, 0), (2, 2, 1, 1),
                                    (2, 2, 16, 0), (1, 0, 0, 1), (0, 2, 4, 1)):
            L.fm_tune_clear()
            L.fm_tune_set(b"mhd.stage", kern)
            L.fm_tune_set(b"mhd.finish", fin)
            L.fm_tune_set(b"mhd.xchunk", xc)
            L.fm_tune_set(b"mhd.stage_xchunk", xc if xc else 16)
            L.fm_tune_set(b"mhd.soft", soft)
            t = [torch.from_numpy(x).to(dtype).to(cuda_device) for x in f0]
            kernels.mhd_forward(t, torch.empty(18 * n ** 3, dtype=dtype, device=cuda_device), 3)
            outs.append([x.cpu().numpy() for x in t])
    finally:
        L.fm_tune_clear()
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)
