"""The C ABI library: loads, exports what include/*.h declares, validates
arguments before touching the device, and fails loudly without a GPU."""
import ctypes
import re
import subprocess

import pytest

from formura_gb300 import _lib, backend
from formura_gb300.build import INCLUDE, LIB
from tests.bits import same_bits

DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(fm_\w+)\s*\(", re.M)


def declared_symbols():
    names = set()
    for h in INCLUDE.glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(DECL.findall(text))
    return sorted(names)


def test_every_declared_symbol_is_exported(core_lib):
    syms = declared_symbols()
    assert len(syms) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", str(LIB)], capture_output=True, text=True,
                         check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if l.strip()}
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    for s in syms:
        assert hasattr(core_lib, s)
    # ctypes signatures cover the whole header
    assert set(syms) <= set(_lib.SIGNATURES), set(syms) - set(_lib.SIGNATURES)


def test_version_and_status_names(core_lib):
    assert b"sm_103a" in core_lib.fm_version()
    assert core_lib.fm_status_name(0) == b"FM_OK"
    assert core_lib.fm_status_name(3) == b"FM_ERR_TIMEOUT"
    assert core_lib.fm_device_count() >= 0


def test_argument_validation_precedes_device_work(core_lib):
    p = _lib.GsParams(0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01)
    fake = ctypes.c_void_p(0x1000)
    # nz not a multiple of 32
    st = core_lib.fm_gs3d_f64_forward(8, 16, 30, fake, fake, fake, fake, ctypes.byref(p), 1, None)
    assert st == 1 and b"nz" in core_lib.fm_last_error()
    # NULL pointer
    st = core_lib.fm_gs3d_f64_forward(8, 16, 32, None, fake, fake, fake, ctypes.byref(p), 1, None)
    assert st == 1
    # dx outside the exact-division range
    bad = _lib.GsParams(0.04, 0.06, 2e-5, 1e-5, 0.5, 1e-30)
    st = core_lib.fm_gs3d_f64_forward(8, 16, 32, fake, fake, fake, fake, ctypes.byref(bad), 1, None)
    assert st == 1 and b"dx" in core_lib.fm_last_error()
    st = core_lib.fm_diff2d_f64_forward(8, 30, fake, fake, 0.1, 1, None)
    assert st == 1
    st = core_lib.fm_gs3d_f32k_forward(8, 12, 32, fake, fake, fake, fake, fake, 1,
                                       ctypes.byref(p), None)
    assert st == 1
    st = core_lib.fm_gs3d_f32k_tb_forward(8, 16, 32, fake, fake, fake, fake, fake, 4, 5,
                                          ctypes.byref(p), None)
    assert st == 1 and b"tb" in core_lib.fm_last_error()
    # zero steps is a no-op that touches nothing
    st = core_lib.fm_gs3d_f64_forward(8, 16, 32, fake, fake, fake, fake, ctypes.byref(p), 0, None)
    assert st == 0


def test_no_cpu_fallback_without_gpu(core_lib):
    if core_lib.fm_device_count() > 0:
        pytest.skip("a GPU is present")
    p = _lib.GsParams(0.04, 0.06, 2e-5, 1e-5, 0.5, 0.01)
    fake = ctypes.c_void_p(0x1000)
    st = core_lib.fm_gs3d_f64_forward(8, 16, 32, fake, fake, fake, fake, ctypes.byref(p), 1, None)
    assert st == 2  # FM_ERR_CUDA: no device, nothing computed on the host
    ptr = ctypes.c_void_p()
    assert core_lib.fm_malloc(ctypes.byref(ptr), 64) in (2, 6)


def test_emitted_header_compiles_with_a_reference_style_driver(tmp_path):
    """A driver written like examples/diffusion-main.cpp compiles and links
    against an emitted program library."""
    p = backend.Program(name="drv_diff", form="diff2d_f64", intra_node_shape=(32, 64),
                        constants=dict(Dt=0.4, Dx=1.0), monitor_interval=20)
    so = backend.build_program(p, outdir=tmp_path)
    drv = tmp_path / "main.c"
    drv.write_text(
        '#include <stdio.h>\n#include "drv_diff.h"\n'
        "int main(void){ struct Formura_Navigator nv; Formura_Init(&nv, MPI_COMM_WORLD);\n"
        "  for(int x=nv.lower_x;x<nv.upper_x;++x) for(int y=nv.lower_y;y<nv.upper_y;++y) dens[x][y]=x+y;\n"
        "  int st = Formura_Forward(&nv);\n"
        '  printf("%d %d %d\\n", st, nv.time_step, NX*NY); return 0; }\n')
    exe = tmp_path / "drv"
    subprocess.run(["gcc", "-std=c11", "-I", str(tmp_path), "-I", str(INCLUDE), str(drv), "-o",
                    str(exe), "-L", str(tmp_path), "-ldrv_diff", "-Wl,-rpath," + str(tmp_path)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    st, ts, n = map(int, r.stdout.split())
    assert n == 32 * 64
    if _lib.lib().fm_device_count() == 0:
        assert st == 2 and ts == 0   # fails loudly, advances nothing
    else:
        assert st == 0 and ts == 20


def test_navigator_layout_matches_header(tmp_path):
    from formura_gb300.runtime import navigator_type

    p = backend.Program(name="lay3", form="gs3d_f64", intra_node_shape=(16, 16, 32),
                        constants=dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01),
                        monitor_interval=4)
    (tmp_path / "lay3.h").write_text(backend.emit_header(p))
    nav = navigator_type(p)
    fields = [f for f, _ in nav._fields_]
    src = tmp_path / "off.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lay3.h"\nint main(void){'
                   'printf("%zu", sizeof(struct Formura_Navigator));'
                   + "".join('printf(" %%zu", offsetof(struct Formura_Navigator, %s));' % f
                             for f in fields) + "return 0;}\n")
    exe = tmp_path / "off"
    subprocess.run(["gcc", "-I", str(tmp_path), "-I", str(INCLUDE), str(src), "-o", str(exe)],
                   check=True)
    vals = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()))
    assert vals[0] == ctypes.sizeof(nav)
    assert vals[1:] == [getattr(nav, f).offset for f in fields]


def test_argument_validation_of_the_other_entry_points(core_lib):
    fake = ctypes.c_void_p(0x1000)
    snap = ctypes.c_void_p()
    shape = (ctypes.c_int * 3)(8, 8, 8)
    assert core_lib.fm_snapshot_create(ctypes.byref(snap), 0, shape, 8) == 1
    assert core_lib.fm_snapshot_create(ctypes.byref(snap), 3, shape, 3) == 1
    bad = (ctypes.c_int * 3)(8, 0, 8)
    assert core_lib.fm_snapshot_create(ctypes.byref(snap), 3, bad, 8) == 1
    assert core_lib.fm_snapshot_plane_elems(None, 0) == -1
    assert core_lib.fm_snapshot_begin(None, fake, 0, 0, None) == 1
    fields = (ctypes.c_void_p * 9)(*([0x1000] * 9))
    assert core_lib.fm_mhd_forward_f32(4, fields, fake, 1, None) == 1  # n >= 5
    assert core_lib.fm_mhd_forward_f64(16, fields, None, 1, None) == 1
    ens = ctypes.c_void_p()
    sizes = (ctypes.c_int * 1)(64)
    F = (ctypes.c_double * 1)(0.04)
    k = (ctypes.c_double * 1)(0.06)
    assert core_lib.fm_gs2d_ensemble_create(ctypes.byref(ens), 1, sizes, F, k, 2e-5, 1e-5, 1.0,
                                            0.01, 128, 2) == 1
    assert core_lib.fm_gs2d_ensemble_create(ctypes.byref(ens), 1, sizes, F, k, 2e-5, 1e-5, 1.0,
                                            0.01, 1, 9) == 1
    err = ctypes.c_void_p(0x2000)
    assert core_lib.fm_conv3x3_fwd_bf16(1, 8, 8, 48, fake, fake, None, None, None, 0, None, fake,
                                        None, err, None) == 1  # cout 32 or 64
    assert core_lib.fm_diff2d_f64_forward_noalloc(2048, 1024, fake, 0.1, 1, None) == 1  # > 2^20


# A C++ driver in the shape of the reference's examples/diffusion-main.cpp:
# <mpi.h> (here the single-process header), `Formura_Navigator navi;`,
# MPI_Init, Formura_Init(&navi, MPI_COMM_WORLD), Formura_Forward in a loop until
# T_MAX, MPI_Finalize.  It also loads the initial state from argv[1] into the
# globals between lower and upper, and writes the final state to argv[2].
CPP_DRIVER = r'''
#include <stdio.h>
#include <mpi.h>
#include "%(name)s.h"

const int T_MAX = %(tmax)d;

int main (int argc, char **argv) {
  Formura_Navigator navi;
  MPI_Init(&argc, &argv);
  Formura_Init(&navi, MPI_COMM_WORLD);
  FILE *in = fopen(argv[1], "rb");
  for (int x = navi.lower_x; x < navi.upper_x; ++x)
    if (fread(%(state)s[x] + navi.lower_y, sizeof(double), navi.upper_y - navi.lower_y, in) == 0)
      return 3;
  fclose(in);
  while(navi.time_step < T_MAX) {
    if (Formura_Forward(&navi) != 0) { printf("error %%s\n", Formura_Last_Error()); return 2; }
    printf("t = %%d\n", navi.time_step);
  }
  FILE *out = fopen(argv[2], "wb");
  for (int x = navi.lower_x; x < navi.upper_x; ++x)
    fwrite(%(state)s[x] + navi.lower_y, sizeof(double), navi.upper_y - navi.lower_y, out);
  fclose(out);
  MPI_Finalize();
}
'''


def _build_cpp_driver(tmp_path, prog, state, tmax):
    so = backend.build_program(prog, outdir=tmp_path)
    src = tmp_path / "main.cpp"
    src.write_text(CPP_DRIVER % dict(name=prog.name, state=state, tmax=tmax))
    exe = tmp_path / "drv"
    subprocess.run(["g++", "-std=c++11", "-I", str(tmp_path), "-I", str(INCLUDE / "single_process_mpi"),
                    "-I", str(INCLUDE), str(src), "-o", str(exe), "-L", str(so.parent),
                    "-l" + prog.name, "-Wl,-rpath," + str(so.parent)], check=True)
    return exe


@pytest.mark.gpu
@pytest.mark.parametrize("fmr", [False, True])
def test_reference_style_driver_runs_on_gpu(tmp_path, cuda_device, fmr):
    """The driver loop of examples/diffusion-main.cpp on the GPU, against the
    hand-tuned diffusion program and against the same program compiled by the
    front end from examples/diffusion-2d.fmr: 5 Forwards of 20 steps on 64 x 96,
    the final state bit-exact with the oracle's 100 steps."""
    import numpy as np

    from formura_gb300 import inits
    from oracle import oracle

    if fmr:
        from formura_gb300.fmr import load_program

        prog = load_program(INCLUDE.parent / "examples" / "diffusion-2d.fmr", name="drv_fmr_diff",
                            intra_node_shape=[64, 96], monitor_interval=20,
                            mpi_grid_shape=[1, 1])
    else:
        prog = backend.Program(name="drv_diff_gpu", form="diff2d_f64", intra_node_shape=(64, 96),
                               constants=dict(Dt=0.4, Dx=1.0), monitor_interval=20)
    exe = _build_cpp_driver(tmp_path, prog, "dens", 100)
    d0 = inits.diffusion_2d(64, 96, seed=31)
    d0.tofile(tmp_path / "in.bin")
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.split("\n")[:5] == ["t = %d" % t for t in (20, 40, 60, 80, 100)]
    got = np.fromfile(tmp_path / "out.bin", dtype=np.float64).reshape(64, 96)
    assert same_bits(got, oracle.diff2d_f64(d0, 100, 0.4, 1.0))


def test_reference_diffusion_driver_compiles_unmodified(tmp_path):
    """The reference's own examples/diffusion-main.cpp, read where it lies,
    compiles and links unchanged against the library the front end emits for
    the reference's examples/diffusion.fmr (shape reduced to 16^3, one rank),
    with the single-process <mpi.h>.  (It is not run here: without a GPU,
    Formura_Forward fails and that driver's loop never ends.)"""
    from formura_gb300.fmr import load_program
    from oracle import oracle

    ref = oracle.DEFAULT_REFERENCE / "examples"
    if not (ref / "diffusion-main.cpp").exists():
        pytest.skip("reference tree absent")
    prog = load_program(ref / "diffusion.fmr", name="diffusion", intra_node_shape=[16, 16, 16],
                        mpi_grid_shape=[1, 1, 1])
    so = backend.build_program(prog, outdir=tmp_path)
    exe = tmp_path / "diffusion-main"
    subprocess.run(["g++", "-I", str(tmp_path), "-I", str(INCLUDE / "single_process_mpi"),
                    "-I", str(INCLUDE), str(ref / "diffusion-main.cpp"), "-o", str(exe),
                    "-L", str(so.parent), "-ldiffusion", "-Wl,-rpath," + str(so.parent)],
                   check=True)
    assert exe.exists()
