"""Monitor output of the device-resident state (fm_snapshot_* and the
Formura_Monitor_* / Formura_Write_Monitor extensions of the generated API).

* a plane taken with monitor_begin is the state at that moment, even when the
  stepping continues before monitor_wait (the gather is ordered on the
  compute stream before the next kernels);
* Formura_Write_Monitor writes the files of examples/pearson-3d-main.cpp's
  write_monitor (6 ints: offsets and sizes, then the U rows and V rows of the
  mid x plane in monitorX-<step>-<rank>.txt, of the mid y plane in monitorY-...)
  byte for byte as that driver would from the downloaded globals.
"""
import numpy as np
import pytest

from formura_gb300 import backend, inits
from formura_gb300.fmr import load_program
from formura_gb300.runtime import load_program as load_lib
from tests.bits import same_bits

pytestmark = pytest.mark.gpu

EX = __import__("pathlib").Path(__file__).resolve().parents[1] / "examples"
GS = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)


def _gs_program(tmp_path):
    p = backend.Program(name="gs_monitor", form="gs3d_f64", intra_node_shape=(24, 32, 64),
                        constants=GS, monitor_interval=6, mpi_grid_shape=(1, 1, 1))
    prog = load_lib(p, outdir=tmp_path)
    prog.init()
    U0, V0 = inits.gray_scott_3d(24, 32, 64, seed=2, ncubes=3, side=6)
    prog.state["U"][...] = U0
    prog.state["V"][...] = V0
    return prog


def _plane(a, axis, index):
    return np.take(a, index, axis=axis)


@pytest.mark.parametrize("axis,index", [(0, 0), (0, 11), (1, 31), (2, 5)])
def test_plane_is_taken_when_begun(cuda_device, tmp_path, axis, index):
    prog = _gs_program(tmp_path)
    prog.upload()
    prog.advance(1)
    prog.download()
    want = {n: _plane(prog.state[n], axis, index).copy() for n in ("U", "V")}
    prog.monitor_begin(axis, index)
    prog.advance(2)              # the state changes before the plane is collected
    got = prog.monitor_wait()
    for n in ("U", "V"):
        assert same_bits(got[n], want[n]), n
    prog.download()
    assert not np.array_equal(_plane(prog.state["U"], axis, index), want["U"])


def test_write_monitor_matches_reference_driver_format(cuda_device, tmp_path):
    prog = _gs_program(tmp_path)
    prog.upload()
    prog.advance(2)
    out = tmp_path / "out"
    out.mkdir()
    prog.write_monitor(out, rank=3)
    prog.download()
    U, V = prog.state["U"], prog.state["V"]
    nx, ny, nz = U.shape
    head = np.array([0, 0, 0, nx, ny, nz], dtype=np.int32).tobytes()
    step = prog.navi.time_step
    x = nx // 2
    want_x = head + U[x].tobytes() + V[x].tobytes()
    y = ny // 2
    want_y = head + U[:, y, :].tobytes() + V[:, y, :].tobytes()
    assert (out / ("monitorX-%06d-3.txt" % step)).read_bytes() == want_x
    assert (out / ("monitorY-%06d-3.txt" % step)).read_bytes() == want_y
    assert not (out / ("monitorZ-%06d-3.txt" % step)).exists()


def test_monitor_of_generated_program_with_mixed_types(cuda_device, tmp_path):
    p = load_program(EX / "fmr-features.fmr")
    prog = load_lib(p, outdir=tmp_path)
    prog.init()
    rng = np.random.default_rng(4)
    prog.state["p"][...] = rng.random(p.shape)
    prog.state["q"][...] = rng.random(p.shape).astype(np.float32)
    prog.upload()
    prog.advance(1)
    prog.download()
    want = {n: prog.state[n][:, 7].copy() for n in ("p", "q")}
    prog.monitor_begin(1, 7)
    prog.advance(1)
    got = prog.monitor_wait()
    assert got["p"].dtype == np.float64 and got["q"].dtype == np.float32
    for n in ("p", "q"):
        assert same_bits(got[n], want[n])
