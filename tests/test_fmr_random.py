"""Random .fmr programs (tests/fmr_random.py, seeded) through the front end:
the generated kernels, compiled for the host (tests/fmr_host.py) under a
random schedule (chunk along axis 0, pairs along axis 1), against the C
oracle of the same program (oracle/fmr_c.py), bit for bit after 5 steps.

Shapes include axes of extent 2 and 3, below the largest read offset (2), so
the modulo form of the periodic wrap runs as well as the conditional one.
The extended cases add 1D programs, deeper trees, let-in and a lambda.
"""
import random

import numpy as np
import pytest

from formura_gb300.fmr import compile_source
from oracle import fmr_c

from fmr_host import HostKernels
from fmr_random import random_program


def case(seed):
    """(source, shape, march_chunk, march_pair, float q) of one seed."""
    rng = random.Random(1000 + seed)
    dim = rng.choice([2, 3])
    float_q = rng.random() < 0.3
    if dim == 3:
        shape = (rng.randint(3, 9), rng.choice([2, 6, 8, 10]), rng.randint(2, 12))
    else:
        shape = (rng.randint(2, 12), rng.randint(2, 33))
    return (random_program(seed, dim, float_q), shape, rng.choice([1, 2, 3, 5, 16]),
            rng.choice([1, 2]), float_q)


def initial_state(seed, shape, float_q):
    r = np.random.default_rng(seed)
    return {"p": r.uniform(-2, 2, shape),
            "q": r.uniform(-2, 2, shape).astype(np.float32 if float_q else np.float64)}


@pytest.mark.parametrize("seed", range(24))
def test_random_program_host_kernels_match_c_oracle(seed):
    src, shape, chunk, pair, float_q = case(seed)
    hk = HostKernels(compile_source(src, shape), chunk, pair)
    s0 = initial_state(seed, shape, float_q)
    got = hk.run(s0, 5)
    want = fmr_c.FmrOracle(src, shape).run(s0, 5)
    for name in s0:
        assert np.array_equal(got[name].view(np.uint8), want[name].view(np.uint8)), (name, src)


def extended_case(seed):
    """(source, shape, march_chunk, march_pair, float q) with 1 to 3 axes,
    trees of depth 2 to 4, let-in and a lambda."""
    rng = random.Random(5000 + seed)
    dim = rng.choice([1, 2, 3])
    float_q = rng.random() < 0.3
    depth = rng.choice([2, 3, 4])
    shape = {3: lambda: (rng.randint(3, 9), rng.choice([2, 6, 8, 10]), rng.randint(2, 12)),
             2: lambda: (rng.randint(2, 12), rng.randint(2, 33)),
             1: lambda: (rng.randint(2, 40),)}[dim]()
    return (random_program(seed, dim, float_q, depth, extended=True), shape,
            rng.choice([1, 2, 3, 5, 16]), rng.choice([1, 2]), float_q)


@pytest.mark.parametrize("seed", range(16))
def test_extended_random_program_host_kernels_match_c_oracle(seed):
    src, shape, chunk, pair, float_q = extended_case(seed)
    hk = HostKernels(compile_source(src, shape), chunk, pair)
    s0 = initial_state(seed, shape, float_q)
    got = hk.run(s0, 5)
    want = fmr_c.FmrOracle(src, shape).run(s0, 5)
    for name in s0:
        assert np.array_equal(got[name].view(np.uint8), want[name].view(np.uint8)), (name, src)


@pytest.mark.parametrize("seed", range(6))
def test_random_program_plain_ieee_forms_match_c_oracle(seed):
    """The same kernels with the integer-pipe forms switched off (plain IEEE
    division, multiplication, fmax/fmin and comparisons)."""
    src, shape, chunk, pair, float_q = case(seed)
    hk = HostKernels(compile_source(src, shape), chunk, pair, soft=False)
    assert "fm::soft::" not in hk.source
    s0 = initial_state(seed, shape, float_q)
    got = hk.run(s0, 5)
    want = fmr_c.FmrOracle(src, shape).run(s0, 5)
    for name in s0:
        assert np.array_equal(got[name].view(np.uint8), want[name].view(np.uint8)), (name, src)


def test_random_programs_cover_the_operation_forms():
    """The emitted kernels of the seeds above use every integer-pipe form."""
    from formura_gb300.fmr.emit_cuda import emit_kernels

    text = ""
    for seed in range(24):
        src, shape, chunk, pair, _ = case(seed)
        text += emit_kernels(compile_source(src, shape), march_chunk=chunk, march_pair=pair)[0]
    for form in ("div_const_s", "div_var_s", "prep_div_s", "scale_pow2", "mul_const_s",
                 "max_s", "min_s", "lt_s", "le_s", "eq_s", "c1b", "ha"):
        assert form in text, form


@pytest.mark.parametrize("seed", range(24))
def test_random_program_schedule_writes_every_cell_once(seed):
    """Store counts of one step under each seed's schedule: every cell of
    every written array exactly once."""
    src, shape, chunk, pair, float_q = case(seed)
    mmp = compile_source(src, shape)
    hk = HostKernels(mmp, chunk, pair, count_stores=True)
    hk.run(initial_state(seed, shape, float_q), 1)
    assert hk.store_counts() == (len(mmp.arrays), 1, 1)



def blocked_cases(n=40):
    """Seeds whose random program the blocked kernel takes (a single level)."""
    from formura_gb300.fmr.emit_cuda import tb_eligible

    out = []
    for seed in range(200):
        src, shape, _, _, float_q = case(seed)
        if tb_eligible(compile_source(src, shape)):
            out.append(seed)
        if len(out) == n:
            break
    return out


@pytest.mark.parametrize("seed", blocked_cases(12))
def test_random_program_blocked_kernel_matches_c_oracle(seed):
    """Random single-level programs (reads at offsets up to 2 on every axis,
    modulo wraps on axes shorter than the halo) through the temporally
    blocked kernel, 2 to 4 steps per pass, small and default tiles."""
    src, shape, _, _, float_q = case(seed)
    tb = 2 + seed % 3
    mmp = compile_source(src, shape)
    s0 = initial_state(seed, shape, float_q)
    want = fmr_c.FmrOracle(src, shape).run(s0, 2 * tb + 1)
    for budget in (0, 16000):
        try:
            hk = HostKernels(mmp, tb=tb, tb_budget=budget)
        except ValueError:
            continue
        got = hk.run(s0, 2 * tb + 1)
        for name in s0:
            assert np.array_equal(got[name].view(np.uint8), want[name].view(np.uint8)), \
                (name, budget, src)


@pytest.mark.parametrize("seed", blocked_cases(12)[:6])
def test_random_program_blocked_kernel_in_bounds(seed):
    """The blocked kernels of random programs access nothing out of bounds
    (AddressSanitizer build of the host kernels, small tiles)."""
    from fmr_host import asan_run

    from formura_gb300.fmr.emit_cuda import emit_tb_kernel

    src, shape, _, _, float_q = case(seed)
    tb = 2 + seed % 3
    mmp = compile_source(src, shape)
    budget = next((b for b in (48000, 200 * 1024) if emit_tb_kernel(mmp, tb, budget=b)), None)
    if budget is None:
        pytest.skip("no tile fits in shared memory")
    status, report = asan_run(mmp, 2 * tb + 1, tb=tb, tb_budget=budget)
    assert status == 0 and "AddressSanitizer" not in report, report[:2000]
