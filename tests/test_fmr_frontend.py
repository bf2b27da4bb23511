"""The .fmr front end (formura_gb300/fmr) on the CPU.

Parser: the operator table and statement forms of src/Formura/Parser.hs.
Evaluation and manifestation: through the C oracle (oracle/fmr_c.py), the
front end reproduces bit for bit
  * the reference's generated examples-generated/pearson.c (golden SHA-256s
    in tests/golden/pearson_ref.json; the .fmr is read from the reference tree
    when it is present),
  * the hand-written restatements of the pearson-3d form (oracle.gs3d_f64),
    of the diffusion form (oracle.diff2d_f64) and of examples/3d-mhd-rk4.fmr
    (oracle.mhd_f64; reference tree needed for the .fmr).
"""
import hashlib
import json
import shutil
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from formura_gb300 import backend, inits
from formura_gb300.fmr import compile_source, config, load_program, mm, om
from formura_gb300.fmr import parser as P
from oracle import fmr_c, oracle

ROOT = Path(__file__).resolve().parents[1]
EX = ROOT / "examples"
REF = oracle.DEFAULT_REFERENCE  # FORMURA_REFERENCE, else the oracle recipe's location
GS = dict(F=0.04, k=0.06, Du=2e-5, Dv=1e-5, dt=0.5, dx=0.01)


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


# -- parser -------------------------------------------------------------------------

def expr(src):
    return P.Parser(src).rexpr()


def test_operator_precedence():
    # unary minus is looser than * (Parser.hs:201-203): -U*V*V = -((U*V)*V)
    e = expr("-U * V*V + F * (1-U)")
    assert isinstance(e, P.Binop) and e.op == "+"
    assert isinstance(e.a, P.Unop) and e.a.op == "-"
    assert e.a.a == P.Binop("*", P.Binop("*", P.Ident("U"), P.Ident("V")), P.Ident("V"))
    # application binds tighter than '.', '.' tighter than '*'
    e = expr("(∂ i . ∂ i) U")
    assert isinstance(e, P.Apply) and isinstance(e.f, P.Binop) and e.f.op == "."
    # a chain of one min/max operator is one n-ary node; comparison is loosest
    e = expr("a >? b >? c <= d")
    assert e.op == "<=" and isinstance(e.a, P.Nary) and len(e.a.items) == 3
    e = expr("a <% b <% c")
    assert isinstance(e, P.Nary) and e.op == "<%" and len(e.items) == 3
    # ** is left-assoc and above *
    e = expr("2 * a ** 2 ** 3")
    assert e.op == "*" and e.b.op == "**" and e.b.a.op == "**"


def test_grid_indices_and_statements():
    e = expr("a[i+1/2, j] - a[, j-3/2]")
    assert e.a.entries == [("i", Fraction(1, 2)), ("j", Fraction(0))]
    assert e.b.entries == [(None, Fraction(0)), ("j", Fraction(-3, 2))]
    prog = P.parse("dimension :: 1\naxes :: x\n# comment\n"
                   "double :: a = 1, b   # typed, one without value\n"
                   "manifest :: m = a + \\\n  b\n"
                   "begin function y = f(x)\n  y = x\nend function\n"
                   "begin function g(x, z) returns (z, x)\nend function\n")
    assert prog.dimension == 1 and prog.axes == ["x"]
    kinds = [type(s).__name__ for s in prog.stmts]
    assert kinds == ["TypeDecl", "TypeDecl", "Subst", "TypeDecl", "Subst", "Subst", "Subst"]
    assert prog.stmts[3].modifiers == ["manifest"]
    f = prog.stmts[5].rhs
    assert isinstance(f, P.Lambda) and isinstance(f.body, P.Let)


def test_parses_every_example():
    files = sorted(EX.glob("*.fmr"))
    if (REF / "examples").exists():
        files += sorted((REF / "examples").glob("*.fmr"))
    # outdated in-file configuration syntax or a syntax stress test: the
    # reference's own grammar rejects these too
    rejected = {"av-mhd-3d.fmr", "hydro.fmr", "mhd.fmr", "test.fmr"}
    for f in files:
        if f.name in rejected:
            with pytest.raises(P.FmrSyntaxError):
                P.parse_file(f)
        else:
            P.parse_file(f)


# -- evaluation -------------------------------------------------------------------------

def test_half_offsets_become_shifts():
    src = ("dimension :: 1\naxes :: x\n"
           "begin function init() returns u\n double [] :: u = 0\nend function\n"
           "begin function step(u) returns u_next\n"
           "  f = u[i+1/2] - u[i-1/2]\n  u_next = f[i+1/2] - f[i-1/2]\nend function\n")
    omp = om.build_om(P.parse(src), [8])
    shifts = sorted(n.args[0] for n in omp.step.nodes if n.kind == "shift")
    assert shifts == [(-1,), (1,)]
    mmp = mm.manifest(omp, [8])
    cursors = sorted(m.args[0] for m in mmp.levels[0].micro if m.kind == "loadS")
    assert cursors == [(-1,), (0,), (1,)]


def test_type_errors_are_reported():
    bad = ("dimension :: 1\naxes :: x\n"
           "begin function init() returns u\n double [] :: u = 0\nend function\n"
           "begin function step(u) returns u_next\n  u_next = u + u[i+1/2]\nend function\n")
    with pytest.raises(om.FmrSemanticError):
        om.build_om(P.parse(bad), [8])
    with pytest.raises(om.FmrSemanticError):
        om.build_om(P.parse(bad.replace("u + u[i+1/2]", "v")), [8])


def test_config_reader():
    cfg = config.loads("initial_walls:\n  x: [136]\n  z: [100,180]\nintra_node_shape: [256, 8]\n"
                       "monitor_interval: 64  # comment\noption_strings: ['omp', 'nbux2']\n")
    assert cfg == {"initial_walls": {"x": [136], "z": [100, 180]}, "intra_node_shape": [256, 8],
                   "monitor_interval": 64, "option_strings": ["omp", "nbux2"]}


def test_constants_follow_c_semantics():
    # folded on the host: the same double operations (and libm pow) as the C
    src = (EX / "fmr-features.fmr").read_text()
    mmp = compile_source(src, (40, 24))
    consts = {m.args[0] for L in mmp.levels for m in L.micro if m.kind == "const"}
    assert 0.25 ** 2 + 1.0 / 3.0 in consts


# -- pins through the C oracle ------------------------------------------------------------

def test_gray_scott_3d_matches_hand_oracle():
    o = fmr_c.FmrOracle((EX / "gray-scott-3d.fmr").read_text(), [16, 16, 32])
    U0, V0 = inits.gray_scott_3d(16, 16, 32, seed=3, ncubes=2, side=6)
    out = o.run({"U": U0, "V": V0}, 20)
    Uo, Vo = oracle.gs3d_f64(U0, V0, 20, **GS)
    assert np.array_equal(out["U"], Uo) and np.array_equal(out["V"], Vo)


def test_diffusion_2d_matches_hand_oracle():
    o = fmr_c.FmrOracle((EX / "diffusion-2d.fmr").read_text(), [64, 48])
    d0 = inits.diffusion_2d(64, 48, seed=2)
    assert np.array_equal(o.run({"dens": d0}, 30)["dens"], oracle.diff2d_f64(d0, 30, Dt=0.4, Dx=1.0))


@pytest.mark.skipif(not (REF / "examples-generated" / "pearson.fmr").exists(),
                    reason="reference tree not present")
def test_pearson_fmr_reproduces_reference_generated_c():
    g = json.loads((ROOT / "tests" / "golden" / "pearson_ref.json").read_text())
    o = fmr_c.FmrOracle((REF / "examples-generated" / "pearson.fmr").read_text(),
                        [g["n"], g["n"]])
    for case in g["cases"]:
        U0, V0 = inits.gray_scott_2d_square(g["n"], g["n"], seed=case["seed"], frac=0.05)
        out = o.run({"U": U0, "V": V0}, case["time_step"])
        assert sha(out["U"], out["V"]) == case["sha256"]


@pytest.mark.skipif(not (REF / "examples" / "3d-mhd-rk4.fmr").exists(),
                    reason="reference tree not present")
def test_mhd_rk4_matches_hand_oracle():
    n = 12
    o = fmr_c.FmrOracle((REF / "examples" / "3d-mhd-rk4.fmr").read_text(), [n, n, n])
    f0 = inits.mhd_3d(n, seed=3)
    out = o.run(dict(zip(o.state_names, f0)), 2)
    for name, r in zip(o.state_names, oracle.mhd_f64(f0, 2)):
        assert np.array_equal(out[name], r), name


# -- code generation -------------------------------------------------------------------------

@pytest.mark.skipif(shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists(),
                    reason="nvcc not available")
def test_generated_program_compiles(tmp_path):
    p = load_program(EX / "fmr-features.fmr")
    assert p.name == "fmr_fmr_features" and [t for _, t in p.states()] == ["double", "float"]
    hdr = backend.emit_header(p)
    assert "extern double p[40][24];" in hdr and "extern float q[40][24];" in hdr
    so = backend.build_program(p, outdir=tmp_path)
    syms = subprocess.run(["nm", "-D", str(so)], capture_output=True, text=True).stdout
    for name in ("Formura_Init", "Formura_Forward", "navi", "p", "q"):
        assert (" %s\n" % name) in syms, name


@pytest.mark.skipif(shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists(),
                    reason="nvcc not available")
def test_generated_integer_pipe_forms_compile(tmp_path):
    """fmr-limiter.fmr has run-time divisions (one divisor shared by two
    quotients), comparisons of doubles, power-of-two scalings and fmax/fmin
    chains: each is emitted in its integer-pipe form and the file compiles."""
    from formura_gb300.fmr.emit_cuda import emit_kernels

    p = load_program(EX / "fmr-limiter.fmr")
    kern, _ = emit_kernels(compile_source(p.fmr_source, tuple(p.shape)), march_chunk=1)
    for form in ("prep_div_s", "div_var_s", "scale_pow2", "max_s", "min_s", "lt_s", "le_s",
                 "eq_s", "mul_const_s"):
        assert "fm::soft::" + form in kern, form
    # the divisor 1 + a*a is prepared once for its two quotients (w and g)
    import collections
    import re
    uses = collections.Counter(re.findall(r"div_var_s\(a\d+, (dva\d+)\)", kern))
    assert max(uses.values()) == 2 and kern.count("prep_div_s(") == len(uses)
    assert "fmax(" not in kern and "fmin(" not in kern and " / " not in kern
    backend.build_program(p, outdir=tmp_path)


def test_marching_kernels_carry_shared_values():
    """In the x-marching form a thread evaluates a chunk of cells along axis 0;
    values a cell shares with the next one (loads at x+1 that become loads at
    x, the face flux at x+1/2 that becomes the one at x-1/2) are carried in
    registers, so the loop body of gray-scott-3d evaluates fewer loads and
    divisions than its first cell."""
    from formura_gb300.fmr.emit_cuda import emit_kernels

    p = load_program(EX / "gray-scott-3d.fmr")
    kern, _ = emit_kernels(compile_source(p.fmr_source, tuple(p.shape)), march_pair=1)
    first, loop = kern.split("for (int c0 = x0 + 1;")
    first = first[first.index("const int c0 = x0;"):]
    count = lambda text, s: text.count(s)
    assert count(loop, "s_U[") + count(loop, "s_V[") == 10   # 14 in the first cell
    assert count(first, "s_U[") + count(first, "s_V[") == 14
    assert count(loop, "div_const_s") == count(first, "div_const_s") - 2
    assert "ha0 = a" in loop and "= ha0;" in loop
    # one cell per thread when asked
    flat, _ = emit_kernels(compile_source(p.fmr_source, tuple(p.shape)), march_chunk=1,
                           march_pair=1)
    assert "x0" not in flat


def test_paired_kernels_share_values_along_axis_1():
    """With pairs a thread evaluates cells y and y+1 of each plane; the second
    takes from the first what they share (its centre and y-1 loads are the
    first cell's y+1 and centre loads, its face flux at y-1/2 is the first
    cell's at y+1/2).  Pairs are asked for (march_pair = 2); the default
    evaluates one cell per thread."""
    from formura_gb300.fmr.emit_cuda import emit_kernels

    p = load_program(EX / "gray-scott-3d.fmr")
    mmp = compile_source(p.fmr_source, tuple(p.shape))
    assert "c1b" not in emit_kernels(mmp)[0]
    kern, _ = emit_kernels(mmp, march_pair=2)
    assert "c1b" in kern
    first, loop = kern.split("for (int c0 = x0 + 1;")
    first = first[first.index("const int c0 = x0;"):]
    count = lambda text, s: text.count(s)
    # per pair: 10 + 8 loads in the loop (20 unpaired), 14 + 10 in the first cell
    assert count(loop, "s_U[") + count(loop, "s_V[") == 18
    assert count(first, "s_U[") + count(first, "s_V[") == 24
    # 16 + 14 divisions by dx in the loop (32 unpaired)
    assert count(loop, "div_const_s") == 30
    assert "w_st_U[idx + 256ull] = b" in loop


CURRENT_SYNTAX_EXAMPLES = [
    "2d-mhd-dc.fmr", "2d-mhd.fmr", "3d-localsun.fmr", "3d-mhd-lessM.fmr", "3d-mhd-rk4.fmr",
    "3d-mhd.fmr", "av-mhd.fmr", "champion.fmr", "diffusion.fmr", "finalist.fmr",
    "lotka-volterra.fmr", "move.fmr", "pearson-2d.fmr", "pearson-3d-0M-alt.fmr",
    "pearson-3d-0M.fmr", "pearson-3d-fast.fmr", "pearson-3d-lap.fmr", "pearson-3d.fmr",
    "pearson-3dx2.fmr", "pearson.fmr", "rule30.fmr"]


@pytest.mark.skipif(not (REF / "examples").exists(), reason="reference tree not present")
@pytest.mark.parametrize("name", CURRENT_SYNTAX_EXAMPLES)
def test_every_reference_example_compiles_and_runs(name):
    """Every example program of the reference in current syntax goes through
    the whole front end (parse, OM, manifestation) and runs two steps in the
    C oracle on a 12^d periodic grid with finite results; its CUDA source is
    generated as well."""
    src = (REF / "examples" / name).read_text()
    dim = P.parse(src).dimension
    o = fmr_c.FmrOracle(src, [12] * dim)
    rng = np.random.default_rng(0)
    state = {n: rng.random([12] * dim) * 0.1 for n, _ in o.mmp.state}
    out = o.run(state, 2)
    assert all(np.isfinite(v).all() for v in out.values())
    from formura_gb300.fmr.emit_cuda import emit_kernels

    kern, levels = emit_kernels(compile_source(src, tuple([12] * dim)))
    assert len(levels) == len(o.mmp.levels) and "__global__" in kern
