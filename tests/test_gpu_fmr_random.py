"""Random .fmr programs (tests/fmr_random.py) compiled by the front end and
run on the GPU through the generated library (Formura_Init/Forward), against
the C oracle of the same program: bit-exact.  The CPU suite runs more seeds
of the same generator through host builds of the same kernels."""
import numpy as np
import pytest

from formura_gb300.fmr import load_program
from formura_gb300.runtime import load_program as load_lib
from oracle import fmr_c

from test_fmr_random import case, initial_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 4, 5, 6, 8, 11])
def test_random_program_on_gpu_matches_c_oracle(cuda_device, tmp_path, seed):
    src, shape, chunk, pair, float_q = case(seed)
    fmr = tmp_path / ("rand%d.fmr" % seed)
    fmr.write_text(src)
    p = load_program(fmr, name="fmr_rand%d" % seed, intra_node_shape=list(shape),
                     monitor_interval=3, march_chunk=chunk, march_pair=pair)
    prog = load_lib(p, outdir=tmp_path)
    prog.init()
    s0 = initial_state(seed, shape, float_q)
    for name, a in s0.items():
        prog.state[name][...] = a
    prog.forward()
    prog.forward()
    want = fmr_c.FmrOracle(src, shape).run(s0, 2 * p.steps_per_forward)
    for name in s0:
        assert np.array_equal(prog.state[name].view(np.uint8), want[name].view(np.uint8)), name
    prog.finalize()


@pytest.mark.parametrize("seed", [0, 3, 7, 13])
def test_random_program_blocked_on_gpu_matches_c_oracle(cuda_device, tmp_path, seed):
    """Random single-level programs through the temporally blocked kernel on
    the GPU (2 to 4 steps per pass), against the C oracle: bit-exact."""
    src, shape, _, _, float_q = case(seed)
    tb = 2 + seed % 3
    fmr = tmp_path / ("randtb%d.fmr" % seed)
    fmr.write_text(src)
    p = load_program(fmr, name="fmr_randtb%d" % seed, intra_node_shape=list(shape),
                     monitor_interval=2 * tb, temporal_blocking_interval=tb, tb_kernel=1)
    from formura_gb300 import backend

    assert backend.blocked_kernel(p) is not None
    prog = load_lib(p, outdir=tmp_path)
    prog.init()
    s0 = initial_state(seed, shape, float_q)
    for name, a in s0.items():
        prog.state[name][...] = a
    prog.forward()
    want = fmr_c.FmrOracle(src, shape).run(s0, p.steps_per_forward)
    for name in s0:
        assert np.array_equal(prog.state[name].view(np.uint8), want[name].view(np.uint8)), name
    prog.finalize()
