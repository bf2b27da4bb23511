"""GPU parity of the 3D Gray-Scott kernels against the CPU oracle.

FP64: bit-exact (the kernel evaluates the generated DAG in the same IEEE
order; divisions by dx are correctly rounded).  FP32+Kahan: bit-exact against
the binary32 restatement.  Sizes are ones the oracle finishes in seconds; at
the full 256^3 size the tests use properties that do not need the oracle.
"""
import numpy as np
import pytest
import torch

from formura_gb300 import _lib, backend, inits, kernels
from formura_gb300.runtime import FormuraProgram
from oracle import oracle
from tests.bits import same_bits

pytestmark = pytest.mark.gpu

GS = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)


def run_f64(U0, V0, steps, dev, params=GS):
    U = torch.from_numpy(U0).to(dev)
    V = torch.from_numpy(V0).to(dev)
    wU, wV = torch.empty_like(U), torch.empty_like(V)
    kernels.gs3d_f64_forward(U, V, wU, wV, kernels.gs_params(**params), steps)
    torch.cuda.synchronize()
    return U.cpu().numpy(), V.cpu().numpy()


@pytest.mark.parametrize("shape,steps", [((32, 32, 32), 40), ((17, 16, 64), 7),
                                         ((1, 16, 32), 5), ((48, 48, 96), 12)])
def test_gs3d_f64_bit_exact(cuda_device, shape, steps):
    U0, V0 = inits.gray_scott_3d(*shape, seed=21, ncubes=3, side=8)
    U, V = run_f64(U0, V0, steps, cuda_device)
    Uo, Vo = oracle.gs3d_f64(U0, V0, steps, **GS)
    assert same_bits(U, Uo) and same_bits(V, Vo)


@pytest.mark.parametrize("kernel,div,mul,xchunk,ry", [
    (1, 0, 0, 0, 4), (1, 1, 0, 0, 4), (1, 2, 0, 0, 4), (2, 0, 0, 0, 4), (2, 1, 0, 0, 4),
    (2, 2, 0, 0, 4), (2, 2, 0, 3, 4), (1, 2, 0, 5, 4), (1, 3, 0, 0, 4), (2, 3, 0, 0, 4),
    (2, 3, 1, 0, 4), (2, 3, 2, 0, 4), (1, 3, 2, 0, 4), (2, 3, 2, 3, 4), (2, 3, 0, 0, 2),
    (2, 3, 1, 0, 2), (2, 3, 2, 5, 2), (1, 3, 1, 0, 2), (2, 3, 1, 7, 2)])
def test_gs3d_f64_every_variant_bit_exact(cuda_device, kernel, div, mul, xchunk, ry):
    lib = _lib.lib()
    try:
        lib.fm_tune_set(b"gs3d_f64.kernel", kernel)
        lib.fm_tune_set(b"gs3d_f64.div", div)
        lib.fm_tune_set(b"gs3d_f64.mul", mul)
        lib.fm_tune_set(b"gs3d_f64.xchunk", xchunk)
        lib.fm_tune_set(b"gs3d_f64.ry", ry)
        for shape, steps in (((24, 32, 64), 9), ((9, 16, 256), 4), ((5, 48, 32), 3)):
            U0, V0 = inits.gray_scott_3d(*shape, seed=31, ncubes=3, side=8)
            U, V = run_f64(U0, V0, steps, cuda_device)
            Uo, Vo = oracle.gs3d_f64(U0, V0, steps, **GS)
            assert same_bits(U, Uo) and same_bits(V, Vo), (shape, kernel, div)
    finally:
        lib.fm_tune_clear()


@pytest.fixture(params=[(1, 0), (3, 0), (3, 1), (3, 2)],
                ids=["div1", "softdiv", "softdiv_softkmul", "softdiv_softmul"])
def arith(request):
    """Division / multiplication forms of the FP64 kernel (gs3d_f64.div, .mul)."""
    lib = _lib.lib()
    lib.fm_tune_set(b"gs3d_f64.div", request.param[0])
    lib.fm_tune_set(b"gs3d_f64.mul", request.param[1])
    yield request.param
    lib.fm_tune_clear()


def test_gs3d_f64_bit_exact_other_constants(cuda_device, arith):
    # tiny dt/dx and random fields exercise the division fast path widely
    rng = np.random.default_rng(0)
    U0 = rng.random((16, 32, 32))
    V0 = rng.random((16, 32, 32)) * 1e-3
    prm = dict(F=0.03, k=0.055, Du=1e-4, Dv=3e-5, dt=0.07, dx=0.0371)
    U, V = run_f64(U0, V0, 9, cuda_device, prm)
    Uo, Vo = oracle.gs3d_f64(U0, V0, 9, **prm)
    assert same_bits(U, Uo) and same_bits(V, Vo)


def test_gs3d_f64_subnormal_front(cuda_device, arith):
    # V values deep in the subnormal range take the IEEE-division fallback.
    U0 = np.ones((8, 16, 32))
    V0 = np.zeros((8, 16, 32))
    V0[4, 8, :] = np.ldexp(1.0, -1060)
    V0[2, 3, 5] = 0.25
    U, V = run_f64(U0, V0, 6, cuda_device)
    Uo, Vo = oracle.gs3d_f64(U0, V0, 6, **GS)
    assert same_bits(U, Uo) and same_bits(V, Vo)


def test_gs3d_f64_full_size_properties(cuda_device, arith):
    """256^3: a periodic shift of the input shifts the output exactly, and the
    uniform state is an exact fixed point."""
    n = 256
    U0, V0 = inits.gray_scott_3d(n, n, n, seed=1)
    steps = 6
    a = run_f64(U0, V0, steps, cuda_device)
    sh = (37, 101, 5)
    b = run_f64(np.roll(U0, sh, (0, 1, 2)), np.roll(V0, sh, (0, 1, 2)), steps, cuda_device)
    assert np.array_equal(np.roll(a[0], sh, (0, 1, 2)), b[0])
    assert np.array_equal(np.roll(a[1], sh, (0, 1, 2)), b[1])
    # one z-row of cells against the oracle on a sub-box: the oracle on the full
    # grid for 2 steps is cheap enough
    Uo, Vo = oracle.gs3d_f64(U0, V0, 2, **GS)
    U2, V2 = run_f64(U0, V0, 2, cuda_device)
    assert same_bits(U2, Uo) and same_bits(V2, Vo)
    one = np.ones((n, n, n))
    zero = np.zeros((n, n, n))
    u, v = run_f64(one, zero, 3, cuda_device)
    assert np.array_equal(u, one) and np.array_equal(v, zero)


def test_gs3d_program_forward_matches_oracle(cuda_device, tmp_path):
    p = backend.Program(name="gs_small", form="gs3d_f64", intra_node_shape=(32, 32, 64),
                        constants=GS, monitor_interval=20, mpi_grid_shape=(1, 1, 1))
    prog = FormuraProgram(p, backend.build_program(p, outdir=tmp_path))
    prog.init()
    U0, V0 = inits.gray_scott_3d(32, 32, 64, seed=8, ncubes=2, side=8)
    prog.state["U"][...] = U0
    prog.state["V"][...] = V0
    prog.forward()
    prog.forward()
    assert prog.navi.time_step == 40
    Uo, Vo = oracle.gs3d_f64(U0, V0, 40, **GS)
    assert same_bits(prog.state["U"], Uo) and same_bits(prog.state["V"], Vo)
    tot = prog.conserved_totals()
    np.testing.assert_allclose(tot, [Uo.sum(), Vo.sum()], rtol=1e-13)
    # resident path: upload once, advance twice, download
    prog.upload()
    prog.advance(2)
    prog.download()
    assert prog.navi.time_step == 80
    Uo, Vo = oracle.gs3d_f64(Uo, Vo, 40, **GS)
    assert same_bits(prog.state["U"], Uo)
    prog.finalize()


def run_f32k(U0, V0, steps, tb, dev, cU0=None, cV0=None):
    """tb None: the generated-DAG float kernel; else the temporally blocked fast form."""
    n = U0.size
    U = torch.from_numpy(U0.astype(np.float32)).to(dev)
    V = torch.from_numpy(V0.astype(np.float32)).to(dev)
    cU = torch.zeros_like(U) if cU0 is None else torch.from_numpy(cU0).to(dev)
    cV = torch.zeros_like(V) if cV0 is None else torch.from_numpy(cV0).to(dev)
    work = torch.empty(4 * n, dtype=torch.float32, device=dev)
    if tb is None:
        kernels.gs3d_f32k_forward(U, V, cU, cV, work, kernels.gs_params(**GS), steps)
    else:
        kernels.gs3d_f32k_tb_forward(U, V, cU, cV, work, kernels.gs_params(**GS), steps, tb)
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in (U, V, cU, cV)]


@pytest.mark.parametrize("shape,steps", [((32, 32, 32), 24), ((20, 24, 64), 16)])
def test_gs3d_f32k_dag_bit_exact(cuda_device, shape, steps):
    U0, V0 = inits.gray_scott_3d(*shape, seed=4, ncubes=3, side=8)
    got = run_f32k(U0, V0, steps, None, cuda_device)
    Z = np.zeros(shape, np.float32)
    want = oracle.gs3d_f32_kahan(U0.astype(np.float32), V0.astype(np.float32), Z, Z, steps, **GS)
    for g, w in zip(got, want):
        assert same_bits(g, w)


@pytest.mark.parametrize("kernel", [0, 1, 2, 3])
@pytest.mark.parametrize("tb", [1, 2, 3, 4])
@pytest.mark.parametrize("shape,steps", [((32, 32, 32), 13), ((20, 24, 64), 8), ((7, 45, 33), 5),
                                         ((64, 64, 64), 12), ((9, 70, 100), 7), ((5, 3, 2), 6)])
def test_gs3d_f32k_tb_bit_exact(cuda_device, shape, steps, tb, kernel):
    """Every blocking depth and every kernel form (0: one row per warp; 1, 2:
    4 or 2 rows per thread with shared face differences) gives the fast form's
    step-by-step result bit for bit, including ragged tiles (sizes not
    multiples of the output tile), axes shorter than a tile and a nonzero
    incoming compensation."""
    lib = _lib.lib()
    U0, V0 = inits.gray_scott_3d(*shape, seed=4, ncubes=3, side=min(4, *shape))
    rng = np.random.default_rng(1)
    cU0 = (rng.standard_normal(shape) * 1e-9).astype(np.float32)
    cV0 = (rng.standard_normal(shape) * 1e-9).astype(np.float32)
    try:
        lib.fm_tune_set(b"gs3d_f32k.kernel", kernel)
        got = run_f32k(U0, V0, steps, tb, cuda_device, cU0, cV0)
    finally:
        lib.fm_tune_clear()
    want = oracle.gs3d_f32k_fast(U0.astype(np.float32), V0.astype(np.float32), cU0, cV0, steps,
                                 **GS)
    for g, w in zip(got, want):  # bit patterns: signed zeros of the compensations included
        assert same_bits(g, w)


@pytest.mark.parametrize("kernel", [0, 1, 2, 3])
def test_gs3d_f32k_tb_xchunk_variants(cuda_device, kernel):
    lib = _lib.lib()
    U0, V0 = inits.gray_scott_3d(40, 32, 32, seed=9, ncubes=2, side=8)
    Z = np.zeros(U0.shape, np.float32)
    want = oracle.gs3d_f32k_fast(U0.astype(np.float32), V0.astype(np.float32), Z, Z, 8, **GS)
    try:
        lib.fm_tune_set(b"gs3d_f32k.kernel", kernel)
        for xc in (1, 3, 8, 40, 100, -1, 0):  # 0: balanced runs across columns
            lib.fm_tune_set(b"gs3d_f32k.xchunk", xc)
            got = run_f32k(U0, V0, 8, 4, cuda_device)
            for g, w in zip(got, want):
                assert same_bits(g, w), xc
    finally:
        lib.fm_tune_clear()


def test_gs3d_f32k_error_against_f64(cuda_device):
    U0, V0 = inits.gray_scott_3d(32, 32, 64, seed=2, ncubes=2, side=8)
    Uo, Vo = oracle.gs3d_f64(U0, V0, 400, **GS)
    for tb in (None, 4):
        U, V, _, _ = run_f32k(U0, V0, 400, tb, cuda_device)
        assert np.linalg.norm(U - Uo) / np.linalg.norm(Uo) < 1e-6
        assert np.linalg.norm(V - Vo) / np.linalg.norm(Vo) < 1e-5
