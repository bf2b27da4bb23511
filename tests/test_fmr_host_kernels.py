"""The CUDA kernels generated by the .fmr front end, compiled for the host
(tests/fmr_host.py) and run against the C oracle of the same program
(oracle/fmr_c.py): bit for bit, under every schedule the emitter has — one
cell per thread, chunks marching along axis 0 with carried values (chunks that
do and do not divide the axis), and pairs of cells along axis 1 sharing values
(with and without marching, forced onto shapes that do not allow them).

These check the generated arithmetic and the carrying and sharing of values
on the CPU; tests/test_gpu_fmr.py runs the same kernels on the GPU.
"""
from pathlib import Path

import numpy as np
import pytest

from formura_gb300 import inits
from formura_gb300.fmr import load_program
from oracle import fmr_c, oracle

from fmr_host import HostKernels

EX = Path(__file__).resolve().parents[1] / "examples"
REF = oracle.DEFAULT_REFERENCE  # FORMURA_REFERENCE, else the oracle recipe's location


def _state(p, seed):
    if p.fmr_source and "gray" in p.name:
        U0, V0 = inits.gray_scott_3d(*p.shape, seed=seed, ncubes=2, side=4)
        return {"U": U0, "V": V0}
    rng = np.random.default_rng(seed)
    return {name: rng.random(p.shape).astype(np.float32 if t == "float" else np.float64)
            for name, t in p.states()}


def _check(p, pair, steps, seed=5):
    hk = HostKernels(p.compiled(), p.march_chunk, pair)
    s0 = _state(p, seed)
    got = hk.run(s0, steps)
    want = fmr_c.FmrOracle(p.fmr_source, p.shape).run(s0, steps)
    for name in s0:
        assert np.array_equal(got[name], want[name]), name
    return hk.source


@pytest.mark.parametrize("fmr,kw,pair", [
    ("gray-scott-3d.fmr", dict(intra_node_shape=[16, 24, 40], march_chunk=1), 1),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[16, 24, 40], march_chunk=4), 1),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[16, 24, 40], march_chunk=4), 2),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[19, 8, 16], march_chunk=5), 2),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[6, 10, 12], march_chunk=1), 2),
    ("fmr-3d-advection.fmr", dict(march_chunk=6), 2),
    ("fmr-3d-advection.fmr", dict(intra_node_shape=[5, 4, 33], march_chunk=2), 2),
    ("fmr-3d-advection.fmr", dict(intra_node_shape=[5, 3, 33]), 0),
    ("fmr-features.fmr", {}, 0),
    ("fmr-features.fmr", dict(march_chunk=7), 0),
    ("fmr-features.fmr", dict(intra_node_shape=[7, 33], march_chunk=3), 2),
    ("fmr-limiter.fmr", dict(march_chunk=3), 0),
    ("fmr-1d-float.fmr", dict(intra_node_shape=[7]), 0),
    ("fmr-libm.fmr", {}, 0),
    ("diffusion-2d.fmr", dict(intra_node_shape=[64, 48], march_chunk=16), 0),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[1, 4, 1], march_chunk=3), 2),
    ("fmr-features.fmr", dict(intra_node_shape=[1, 1]), 0),
])
def test_host_kernels_match_c_oracle(fmr, kw, pair):
    p = load_program(EX / fmr, **kw)
    src = _check(p, pair, steps=7)
    paired = "c1b" in src
    assert paired == (pair == 2 and p.dim >= 3 and p.shape[1] % 2 == 0)


def test_pair_forced_on_odd_axis_falls_back():
    p = load_program(EX / "gray-scott-3d.fmr", intra_node_shape=[8, 7, 16], march_chunk=3)
    src = _check(p, 2, steps=4)
    assert "c1b" not in src and "ha" in src


@pytest.mark.skipif(not (REF / "examples" / "3d-mhd-rk4.fmr").exists(),
                    reason="reference tree absent")
def test_host_kernels_mhd_rk4_paired():
    """All 8 levels of the reference's 3d-mhd-rk4.fmr (72 manifest arrays),
    marching in chunks of 3 with pairs forced onto every level."""
    p = load_program(REF / "examples" / "3d-mhd-rk4.fmr", intra_node_shape=[8, 8, 8],
                     monitor_interval=2, mpi_grid_shape=[1, 1, 1], march_chunk=3)
    o = fmr_c.FmrOracle(p.fmr_source, p.shape)
    s0 = dict(zip(o.state_names, inits.mhd_3d(8, seed=3)))
    hk = HostKernels(p.compiled(), p.march_chunk, 2)
    assert hk.source.count("c1b + 1") >= 1
    got = hk.run(s0, 2)
    want = o.run(s0, 2)
    for name in s0:
        assert np.array_equal(got[name], want[name]), name


REF_EXAMPLES = [
    "2d-mhd-dc.fmr", "2d-mhd.fmr", "3d-localsun.fmr", "3d-mhd-lessM.fmr", "3d-mhd-rk4.fmr",
    "3d-mhd.fmr", "av-mhd.fmr", "champion.fmr", "diffusion.fmr", "finalist.fmr",
    "lotka-volterra.fmr", "move.fmr", "pearson-2d.fmr", "pearson-3d-0M-alt.fmr",
    "pearson-3d-0M.fmr", "pearson-3d-fast.fmr", "pearson-3d-lap.fmr", "pearson-3d.fmr",
    "pearson-3dx2.fmr", "pearson.fmr", "rule30.fmr"]


@pytest.mark.skipif(not (REF / "examples").exists(), reason="reference tree absent")
@pytest.mark.parametrize("name", REF_EXAMPLES)
def test_host_kernels_reference_examples(name):
    """Every example program of the reference in current syntax, on a 12^d
    grid, marching in chunks of 3 with pairs where the shape has 3 axes: the
    generated kernels equal the C oracle bit for bit after two steps."""
    from formura_gb300.fmr import compile_source
    from formura_gb300.fmr import parser as P

    src = (REF / "examples" / name).read_text()
    shape = [12] * P.parse(src).dimension
    o = fmr_c.FmrOracle(src, shape)
    rng = np.random.default_rng(0)
    s0 = {n: rng.random(shape) * 0.1 for n, _ in o.mmp.state}
    want = o.run(s0, 2)
    got = HostKernels(compile_source(src, tuple(shape)), 3, 2).run(s0, 2)
    for n in want:
        assert np.array_equal(got[n].view(np.uint8), want[n].view(np.uint8)), n


SCHEDULE_CASES = [
    ("gray-scott-3d.fmr", [19, 8, 16], 5, 2), ("gray-scott-3d.fmr", [16, 24, 40], 16, 2),
    ("gray-scott-3d.fmr", [7, 5, 9], 3, 2), ("gray-scott-3d.fmr", [6, 10, 12], 1, 2),
    ("gray-scott-3d.fmr", [33, 2, 3], 4, 1), ("fmr-3d-advection.fmr", [5, 4, 33], 2, 2),
    ("fmr-3d-advection.fmr", [9, 6, 7], 4, 2), ("fmr-features.fmr", [7, 33], 3, 1),
    ("fmr-limiter.fmr", [24, 40], 7, 1), ("fmr-1d-float.fmr", [97], 16, 1),
    ("diffusion-2d.fmr", [64, 48], 16, 1),
    # axes of extent 1 (every neighbour read wraps onto the cell itself), chunks longer
    # than the axis
    ("gray-scott-3d.fmr", [1, 4, 1], 3, 2), ("gray-scott-3d.fmr", [3, 1, 5], 50, 2),
    ("fmr-features.fmr", [1, 1], 1, 1), ("fmr-1d-float.fmr", [1], 16, 1),
]


@pytest.mark.parametrize("fmr,shape,chunk,pair", SCHEDULE_CASES)
def test_schedule_writes_every_cell_once(fmr, shape, chunk, pair):
    """The work items of a generated kernel (columns or column pairs along
    axis 1, chunks along axis 0, ragged last chunks) cover the grid exactly:
    in one step every cell of every array the program writes is stored once,
    and no store falls outside the array."""
    p = load_program(EX / fmr, intra_node_shape=shape, march_chunk=chunk)
    mmp = p.compiled()
    hk = HostKernels(mmp, chunk, pair, count_stores=True)
    hk.run(_state(p, 3), 1)
    arrays, lo, hi = hk.store_counts()
    assert (arrays, lo, hi) == (len(mmp.arrays), 1, 1)


# ---- temporally blocked kernels (emit_cuda.TBEmitter) ----------------------------

TB_CASES = [
    ("gray-scott-3d-float.fmr", [12, 20, 24]), ("gray-scott-3d-float.fmr", [9, 40, 70]),
    ("gray-scott-3d.fmr", [16, 16, 16]), ("gray-scott-3d.fmr", [5, 7, 33]),
    ("diffusion-2d.fmr", [40, 64]), ("diffusion-2d.fmr", [7, 300]),
    ("fmr-libm.fmr", [13, 17]), ("gray-scott-3d-float.fmr", [1, 4, 3]),
    ("heat-3d-float.fmr", [10, 40, 72]), ("heat-3d-float.fmr", [3, 5, 9]),
    # several levels per step (manifest intermediates read by later levels)
    ("fmr-limiter.fmr", [24, 40]), ("fmr-limiter.fmr", [9, 17]), ("fmr-features.fmr", [13, 33]),
    ("fmr-3d-advection.fmr", [8, 12, 20]), ("fmr-3d-advection.fmr", [5, 3, 33]),
]


@pytest.mark.parametrize("fmr,shape", TB_CASES)
@pytest.mark.parametrize("tb", [2, 3, 4])
@pytest.mark.parametrize("budget", [0, 24000])
def test_blocked_kernel_matches_c_oracle(fmr, shape, tb, budget):
    """The blocked kernel (tb steps per pass, each time level a ring of planes
    in shared memory) on the host: bit for bit the C oracle's steps, for
    every depth, with the default tile and with a small shared-memory budget
    (small tiles, many of them, halos wider than the tile), on ragged shapes
    and step counts that are not multiples of tb."""
    p = load_program(EX / fmr, intra_node_shape=shape)
    s0 = _state(p, 11)
    try:
        hk = HostKernels(p.compiled(), tb=tb, tb_budget=budget)
    except ValueError:
        pytest.skip("no tile fits this budget")
    got = hk.run(s0, 2 * tb + 1)
    want = fmr_c.FmrOracle(p.fmr_source, p.shape).run(s0, 2 * tb + 1)
    for name in s0:
        assert np.array_equal(got[name].view(np.uint8), want[name].view(np.uint8)), name


@pytest.mark.parametrize("fmr,shape", TB_CASES)
def test_blocked_kernel_writes_every_cell_once_per_pass(fmr, shape):
    p = load_program(EX / fmr, intra_node_shape=shape)
    mmp = p.compiled()
    if _fits(mmp, 3, 24000):
        hk = HostKernels(mmp, tb=3, tb_budget=24000, count_stores=True)
    elif _fits(mmp, 3, 200 * 1024):
        hk = HostKernels(mmp, tb=3, count_stores=True)
    else:
        pytest.skip("no tile fits in shared memory")
    hk.run(_state(p, 3), 3)  # one pass
    # the state arrays only: intermediate arrays live in the shared-memory rings
    assert hk.store_counts() == (len([a for a in mmp.arrays.values() if a.store_of]), 1, 1)


def _fits(mmp, tb, budget):
    from formura_gb300.fmr.emit_cuda import emit_tb_kernel

    return emit_tb_kernel(mmp, tb, budget=budget) is not None


def test_which_programs_are_blocked():
    """Programs on 2 or 3 axes whose states each have one store are blocked,
    single-level or not; 1D programs keep one launch per step, as does a
    halo that leaves no tile in shared memory."""
    from formura_gb300 import backend
    from formura_gb300.fmr.emit_cuda import tb_eligible

    assert tb_eligible(load_program(EX / "gray-scott-3d-float.fmr").compiled())
    assert tb_eligible(load_program(EX / "fmr-limiter.fmr").compiled())
    assert not tb_eligible(load_program(EX / "fmr-1d-float.fmr").compiled())
    p = load_program(EX / "gray-scott-3d-float.fmr")
    # by default a heavy step (56 arithmetic operations) stays one step per launch ...
    assert p.temporal_blocking_interval == 4 and backend.blocked_kernel(p) is None
    assert backend.blocked_kernel(load_program(EX / "gray-scott-3d-float.fmr", tb_kernel=1)) is not None
    assert backend.blocked_kernel(load_program(EX / "gray-scott-3d-float.fmr", tb_kernel=-1)) is None
    # ... and a light binary32 one (13) is blocked
    assert backend.blocked_kernel(load_program(EX / "heat-3d-float.fmr")) is not None
    assert backend.blocked_kernel(load_program(EX / "heat-3d-float.fmr", tb_kernel=-1)) is None
    assert backend.blocked_kernel(load_program(EX / "gray-scott-3d.fmr")) is None  # interval 1
    # FP64 with 8 steps per pass: the halo of 8 leaves no tile in shared memory
    assert backend.blocked_kernel(load_program(EX / "gray-scott-3d.fmr",
                                               temporal_blocking_interval=8, tb_kernel=1)) is None


def test_blocked_kernel_tma_geometry():
    """The TMA-staged tiles: 16-byte aligned origins and rows along the fastest
    axis (a halo rounded up to 4 floats or 2 doubles), boxes of at most 256
    elements per edge, ring planes padded to 128 bytes, and tiles away from
    the periodic boundary present on the shapes the GPU tests use."""
    from formura_gb300.fmr.emit_cuda import emit_tb_kernel

    for fmr, shape, tb in (("gray-scott-3d-float.fmr", [12, 80, 192], 4),
                           ("gray-scott-3d.fmr", [10, 70, 128], 2),
                           ("gray-scott-3d-float.fmr", [256, 256, 256], 4)):
        p = load_program(EX / fmr, intra_node_shape=shape)
        src, plan, _, _ = emit_tb_kernel(p.compiled(), tb)
        assert plan.tma and "cp.async.bulk" not in src  # the copies sit in fm_tc.cuh helpers
        assert "fm::tc::tma_load_3d" in src and "fm::tc::mbar_wait" in src
        elem = 4 if "float" in fmr else 8
        assert (plan.H[2] * elem) % 16 == 0 and (plan.TI[2] * elem) % 16 == 0
        assert plan.RG[1] <= 256 and plan.RG[2] <= 256 and (plan.PS * elem) % 128 == 0
        interior = [(t1, t2) for t1 in range(plan.NT[1]) for t2 in range(plan.NT[2])
                    if 0 <= t1 * plan.TI[1] - plan.H[1] and
                    t1 * plan.TI[1] - plan.H[1] + plan.RG[1] <= shape[1] and
                    0 <= t2 * plan.TI[2] - plan.H[2] and
                    t2 * plan.TI[2] - plan.H[2] + plan.RG[2] <= shape[2]]
        assert interior, (fmr, shape)
    # 2D programs gather every plane
    p = load_program(EX / "diffusion-2d.fmr", intra_node_shape=[64, 256])
    assert not emit_tb_kernel(p.compiled(), 4)[1].tma


ASAN_CASES = [("fmr-limiter.fmr", [24, 40], 2, 0), ("fmr-features.fmr", [13, 33], 3, 0),
              ("fmr-3d-advection.fmr", [8, 12, 20], 2, 0), ("heat-3d-float.fmr", [6, 20, 40], 4, 48000),
              ("gray-scott-3d.fmr", [5, 7, 33], 2, 0), ("diffusion-2d.fmr", [7, 300], 3, 0)]


@pytest.mark.parametrize("fmr,shape,tb,budget", ASAN_CASES)
def test_blocked_kernel_in_bounds_under_address_sanitizer(fmr, shape, tb, budget):
    """Every array and shared-memory access of the blocked kernel stays in
    bounds (AddressSanitizer build of the host kernels), for single- and
    multi-level programs, ragged tiles and small tile budgets."""
    from fmr_host import asan_run

    p = load_program(EX / fmr, intra_node_shape=shape)
    status, report = asan_run(p.compiled(), 2 * tb + 1, tb=tb, tb_budget=budget)
    assert status == 0 and "AddressSanitizer" not in report, report[:2000]


@pytest.mark.skipif(not (REF / "examples" / "pearson-2d.fmr").exists(), reason="reference tree absent")
@pytest.mark.parametrize("name", ["pearson-2d.fmr", "pearson.fmr", "lotka-volterra.fmr", "move.fmr"])
def test_blocked_kernel_reference_examples(name):
    """The reference's multi-level example programs through the blocked
    kernel (3 steps per pass) on the host: bit for bit the C oracle, and in
    bounds under AddressSanitizer."""
    from formura_gb300.fmr import compile_source
    from formura_gb300.fmr import parser as P
    from formura_gb300.fmr.emit_cuda import emit_tb_kernel
    from fmr_host import asan_run

    src = (REF / "examples" / name).read_text()
    shape = [12, 20, 16][:P.parse(src).dimension]
    mmp = compile_source(src, tuple(shape))
    if emit_tb_kernel(mmp, 3) is None:
        pytest.skip("not blocked")
    o = fmr_c.FmrOracle(src, shape)
    rng = np.random.default_rng(0)
    s0 = {n: rng.random(shape) * 0.1 for n, _ in o.mmp.state}
    got = HostKernels(mmp, tb=3).run(s0, 7)
    want = o.run(s0, 7)
    for n in want:
        assert np.array_equal(got[n].view(np.uint8), want[n].view(np.uint8)), n
    status, report = asan_run(mmp, 7, tb=3)
    assert status == 0 and "AddressSanitizer" not in report, report[:2000]
