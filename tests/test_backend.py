"""Back-end emission: the generated-code API and its step-count semantics."""
from pathlib import Path

import pytest

from formura_gb300 import backend
from formura_gb300.programs import PROGRAMS

GS = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)


def prog(**kw):
    base = dict(name="t", form="gs3d_f64", intra_node_shape=(16, 16, 32), constants=GS,
                monitor_interval=20)
    base.update(kw)
    return backend.Program(**base)


@pytest.mark.parametrize("mi,tb,m", [(20, 1, 20), (20, 4, 24), (64, 8, 64), (65, 8, 80),
                                     (2000, 8, 2000), (1, 1, 2)])
def test_steps_per_forward_rounds_up_to_two_tb(mi, tb, m):
    # Translate.hs:1111-1113: the first multiple of 2*tb not below monitor_interval
    assert prog(monitor_interval=mi, temporal_blocking_interval=tb).steps_per_forward == m


def test_header_has_the_generated_api():
    h = backend.emit_header(prog())
    for s in ("#define NX  16", "#define NZ  32", "extern double U[16][16][32];",
              "extern double V[16][16][32];", "struct Formura_Navigator {", "int time_step;",
              "int lower_x;", "int upper_z;", "int offset_y;", "int mpi_my_rank;",
              "int mpi_rank__1_0_m1;", "extern struct Formura_Navigator navi;",
              "int Formura_Init (struct Formura_Navigator *navi, MPI_Comm comm);",
              "int Formura_Forward (struct Formura_Navigator *navi);"):
        assert s in h, s


def test_float_program_declares_float_state_and_compensation():
    h = backend.emit_header(prog(form="gs3d_f32k"))
    assert "extern float U[16][16][32];" in h
    assert "extern float U_compensation[16][16][32];" in h


def test_validation():
    with pytest.raises(ValueError, match="one GPU"):
        prog(mpi_grid_shape=(2, 1, 1)).validate()
    with pytest.raises(ValueError, match="unknown form"):
        prog(form="nope").validate()
    with pytest.raises(ValueError, match="missing"):
        prog(constants=dict(F=1)).validate()
    with pytest.raises(ValueError, match="3D"):
        prog(intra_node_shape=(16, 32)).validate()


def test_validation_of_generated_schedule_keys():
    from formura_gb300.fmr import load_program

    ex = Path(__file__).resolve().parents[1] / "examples" / "gray-scott-3d.fmr"
    load_program(ex, intra_node_shape=[8, 8, 8], march_chunk=3, march_pair=2).validate()
    with pytest.raises(ValueError, match="march_pair"):
        load_program(ex, intra_node_shape=[8, 8, 8], march_pair=3).validate()
    with pytest.raises(ValueError, match="march_chunk"):
        load_program(ex, intra_node_shape=[8, 8, 8], march_chunk=-1).validate()


def test_delta_rank_names_follow_toCName():
    # Translate.hs:406-407 with toCName (:317-343): "-" -> "m", MPIRank dropped
    assert backend._delta_name((1, 0, -1)) == "mpi_rank__1_0_m1"
    assert backend._delta_name((0, 0)) == "mpi_rank__0_0"


def test_shipped_programs_validate():
    for p in PROGRAMS.values():
        p.validate()
        backend.emit_source(p)
    assert PROGRAMS["gray_scott_3d"].steps_per_forward == 2000
    assert PROGRAMS["gray_scott_3d_f32k"].steps_per_forward == 2000
    assert PROGRAMS["diffusion_2d"].steps_per_forward == 1000
