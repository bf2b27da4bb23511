"""Programs compiled by the .fmr front end, run on the GPU through the
generated library (Formura_Init / Formura_Forward and the global arrays),
against the C oracle of the same program (oracle/fmr_c.py): bit-exact.

The generated 3D Gray-Scott program is also compared with the hand-written
gs3d_f64_row kernel: two independent GPU paths, one value.
"""
import numpy as np
import pytest
import torch

from formura_gb300 import inits, kernels
from formura_gb300.fmr import load_program
from formura_gb300.runtime import load_program as load_lib
from oracle import fmr_c
from tests.bits import same_bits

pytestmark = pytest.mark.gpu

EX = __import__("pathlib").Path(__file__).resolve().parents[1] / "examples"
GS = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)


def _random_state(prog, rng):
    out = {}
    for name, t in prog.program.states():
        a = rng.random(prog.program.shape)
        out[name] = a.astype(np.float32 if t == "float" else np.float64)
    return out


@pytest.mark.parametrize("fmr,kw", [
    ("fmr-features.fmr", {}),
    ("fmr-features.fmr", dict(intra_node_shape=[7, 33], monitor_interval=3)),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[16, 24, 40], monitor_interval=5)),
    ("diffusion-2d.fmr", dict(intra_node_shape=[64, 48], monitor_interval=7)),
    ("fmr-1d-float.fmr", {}),
    ("fmr-1d-float.fmr", dict(intra_node_shape=[7], monitor_interval=5)),
    ("fmr-3d-advection.fmr", {}),
    ("fmr-3d-advection.fmr", dict(intra_node_shape=[5, 3, 33], monitor_interval=4)),
    ("fmr-limiter.fmr", {}),
    ("fmr-limiter.fmr", dict(intra_node_shape=[9, 17], monitor_interval=6)),
    # the x-marching kernels (values carried between consecutive cells along x),
    # chunks that divide the axis and chunks that do not
    ("gray-scott-3d.fmr", dict(intra_node_shape=[16, 24, 40], monitor_interval=5, march_chunk=4)),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[19, 8, 16], monitor_interval=3, march_chunk=5)),
    ("fmr-3d-advection.fmr", dict(march_chunk=6)),
    ("fmr-features.fmr", dict(march_chunk=7)),
    ("fmr-limiter.fmr", dict(march_chunk=3)),
    ("diffusion-2d.fmr", dict(intra_node_shape=[64, 48], monitor_interval=7, march_chunk=16)),
    # pairs of cells along y sharing values, with and without marching along x
    ("gray-scott-3d.fmr", dict(intra_node_shape=[16, 24, 40], monitor_interval=5, march_chunk=4,
                               march_pair=2)),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[19, 8, 16], monitor_interval=3, march_chunk=5,
                               march_pair=2)),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[6, 10, 12], monitor_interval=3, march_chunk=1,
                               march_pair=2)),
    ("fmr-3d-advection.fmr", dict(march_chunk=6, march_pair=2)),
    # the temporally blocked kernel: temporal_blocking_interval steps per pass, each
    # time level a ring of planes in shared memory (tb_kernel 1: whenever eligible)
    ("gray-scott-3d-float.fmr", dict(intra_node_shape=[24, 40, 72], monitor_interval=8,
                                     tb_kernel=1)),
    ("gray-scott-3d-float.fmr", dict(intra_node_shape=[9, 33, 20], monitor_interval=5,
                                     temporal_blocking_interval=3, tb_kernel=1)),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[16, 24, 40], monitor_interval=4,
                               temporal_blocking_interval=2, tb_kernel=1)),
    ("diffusion-2d.fmr", dict(intra_node_shape=[64, 48], monitor_interval=8,
                              temporal_blocking_interval=4, tb_kernel=1)),
    ("diffusion-2d.fmr", dict(intra_node_shape=[5, 700], monitor_interval=6,
                              temporal_blocking_interval=3, tb_kernel=1)),
    # shapes with tiles away from the periodic boundary: their input planes arrive by TMA
    ("gray-scott-3d-float.fmr", dict(intra_node_shape=[12, 80, 192], monitor_interval=8,
                                     tb_kernel=1)),
    ("gray-scott-3d.fmr", dict(intra_node_shape=[10, 70, 128], monitor_interval=4,
                               temporal_blocking_interval=2, tb_kernel=1)),
    ("heat-3d-float.fmr", dict(intra_node_shape=[20, 100, 192], monitor_interval=8)),
    ("heat-3d-float.fmr", dict(intra_node_shape=[7, 9, 20], monitor_interval=12,
                               temporal_blocking_interval=3)),
    # blocked programs of several levels per step (manifest intermediates in rings)
    ("fmr-limiter.fmr", dict(monitor_interval=4, temporal_blocking_interval=2, tb_kernel=1)),
    ("fmr-features.fmr", dict(monitor_interval=6, temporal_blocking_interval=3, tb_kernel=1)),
    ("fmr-3d-advection.fmr", dict(intra_node_shape=[16, 40, 128], monitor_interval=4,
                                  temporal_blocking_interval=2, tb_kernel=1)),
])
def test_generated_program_matches_c_oracle(cuda_device, tmp_path, fmr, kw):
    p = load_program(EX / fmr, **kw)
    prog = load_lib(p, outdir=tmp_path)
    prog.init()
    rng = np.random.default_rng(len(fmr))
    if fmr.startswith("gray"):
        U0, V0 = inits.gray_scott_3d(*p.shape, seed=4, ncubes=2, side=6)
        s0 = {"U": U0, "V": V0}
    else:
        s0 = _random_state(prog, rng)
    for name, a in s0.items():
        prog.state[name][...] = a
    prog.forward()
    prog.forward()
    assert prog.navi.time_step == 2 * p.steps_per_forward
    want = fmr_c.FmrOracle(p.fmr_source, p.shape).run(s0, 2 * p.steps_per_forward)
    for name in s0:
        assert same_bits(prog.state[name], want[name]), name


def test_generated_gs3d_equals_hand_kernel(cuda_device, tmp_path):
    p = load_program(EX / "gray-scott-3d.fmr", intra_node_shape=[32, 32, 64], monitor_interval=10)
    prog = load_lib(p, outdir=tmp_path)
    prog.init()
    U0, V0 = inits.gray_scott_3d(32, 32, 64, seed=9, ncubes=3, side=8)
    prog.state["U"][...] = U0
    prog.state["V"][...] = V0
    prog.upload()
    prog.advance(3)
    prog.download()
    U = torch.from_numpy(U0).cuda()
    V = torch.from_numpy(V0).cuda()
    kernels.gs3d_f64_forward(U, V, torch.empty_like(U), torch.empty_like(V),
                             kernels.gs_params(**GS), 30)
    assert same_bits(prog.state["U"], U.cpu().numpy())
    assert same_bits(prog.state["V"], V.cpu().numpy())
    tot = prog.conserved_totals()
    np.testing.assert_allclose(tot, [prog.state["U"].sum(), prog.state["V"].sum()], rtol=1e-12)


def test_generated_program_with_device_libm_within_tolerance(cuda_device, tmp_path):
    """`**` and extern exp on grid values run on the device's pow/exp, which
    are not bit-identical with the host's libm: agreement to 1e-12 relative."""
    p = load_program(EX / "fmr-libm.fmr")
    prog = load_lib(p, outdir=tmp_path)
    prog.init()
    a0 = np.random.default_rng(5).random(p.shape)
    prog.state["a"][...] = a0
    prog.forward()
    prog.forward()
    want = fmr_c.FmrOracle(p.fmr_source, p.shape).run({"a": a0}, 2 * p.steps_per_forward)["a"]
    np.testing.assert_allclose(prog.state["a"], want, rtol=1e-12, atol=1e-14)


def test_blocked_float_gs3d_equals_per_step_kernels(cuda_device, tmp_path):
    """examples/gray-scott-3d-float.fmr as configured (4 steps per pass of the
    blocked kernel) at 64^3 equals the same program run one step per launch,
    bit for bit, and the blocked kernel is the one the library runs."""
    from formura_gb300 import backend

    outs = []
    for tbk in (1, -1):
        p = load_program(EX / "gray-scott-3d-float.fmr", intra_node_shape=[64, 64, 64],
                         monitor_interval=40, tb_kernel=tbk, name="gsf_tb%d" % (tbk + 1))
        assert (backend.blocked_kernel(p) is not None) == (tbk == 1)
        prog = load_lib(p, outdir=tmp_path)
        prog.init()
        U0, V0 = inits.gray_scott_3d(64, 64, 64, seed=2, ncubes=4, side=8)
        prog.state["U"][...] = U0.astype(np.float32)
        prog.state["V"][...] = V0.astype(np.float32)
        prog.forward()
        outs.append((prog.state["U"].copy(), prog.state["V"].copy()))
        prog.finalize()
    assert same_bits(outs[0][0], outs[1][0]) and same_bits(outs[0][1], outs[1][1])
