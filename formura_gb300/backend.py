"""The CUDA back end: emits the per-program host code of a Formura program.

Formura's C back end writes, for a program ``<name>.fmr`` with its numerical
config ``<name>.yaml``, a header and a C file that keep one API
(src/Formura/MPICxx/Translate.hs:973-1139):

* ``#define NX ...`` per axis = intra_node_shape x mpi_grid_shape (:1015-1019);
* ``extern <elem> <State>[NX][NY]...;`` — one global array per state
  variable, named after the arguments of ``step`` (:418-431);
* ``struct Formura_Navigator`` — ``time_step``; ``lower_/upper_/offset_`` per
  axis; ``mpi_comm``; ``mpi_my_rank``; ``mpi_rank_<delta>`` (:1038-1048);
  ``extern struct Formura_Navigator navi;`` (:1050-1051);
* ``int Formura_Init(struct Formura_Navigator*, MPI_Comm)`` (:1070-1092);
* ``int Formura_Forward(struct Formura_Navigator*)`` — advances the globals by
  M = monitor_interval rounded up to a multiple of 2*temporal_blocking_interval
  steps and adds M to ``time_step`` (:1106-1131).

This module emits the same API, but the body of ``Formura_Forward`` copies the
globals to the GPU, runs M steps through the thin C ABI of
``libformura_gb300.so`` (include/formura_gb300.h) and copies them back.  The
state is stored without a margin: ``lower_* = 0``, ``upper_* = N*``,
``offset_* = 0`` (the navigator of examples-generated/pearson.c:75-85).
One GPU, one rank: every ``mpi_rank_*`` neighbour is rank 0 and the halo
exchange is the kernels' periodic index wrap.

Extensions (not in the reference; all optional for a caller):
``Formura_Upload`` / ``Formura_Advance`` / ``Formura_Download`` split
``Formura_Forward`` so that state can stay resident on the GPU between calls;
``Formura_Device_State`` exposes the device copy of a state array;
``Formura_Set_Stream`` selects the CUDA stream; ``Formura_Conserved_Totals``
returns FP64 sums of the state arrays (mass/energy drift checks);
``Formura_Finalize`` frees the device copies.
"""
from __future__ import annotations

import dataclasses
import hashlib
import itertools
import os
import subprocess
from pathlib import Path
from typing import Dict, List, Optional, Sequence, Tuple

from . import build as _build

AXES3 = ("x", "y", "z")


@dataclasses.dataclass(frozen=True)
class Program:
    """A Formura program as the back end needs it.

    ``form`` names the kernel family that evaluates the program's ``step``:
      * ``gs3d_f64``   — examples/pearson-3d.fmr form, double
      * ``gs3d_f32k``  — the same DAG in float with Kahan time accumulation
      * ``gs3d_f32k_tb`` — the float fast form with Kahan accumulation,
        temporally blocked (``temporal_blocking_interval`` > 1 -> depth <= 4)
      * ``diff2d_f64`` — examples/diffusion.fmr form in 2D, double
      * ``fmr``        — any program: ``fmr_source`` is compiled by the front end
        (formura_gb300.fmr) into generated CUDA kernels
    ``constants`` are the .fmr constants of ``step`` (F, k, Du, Dv, dt, dx /
    Dt, Dx).  ``intra_node_shape``, ``mpi_grid_shape``, ``monitor_interval``
    and ``temporal_blocking_interval`` are the YAML keys of
    src/Formura/NumericalConfig.hs:17-34.
    """

    name: str
    form: str
    intra_node_shape: Sequence[int]
    constants: Dict[str, float]
    monitor_interval: int
    temporal_blocking_interval: int = 1
    mpi_grid_shape: Optional[Sequence[int]] = None
    axes: Optional[Sequence[str]] = None
    fmr_source: Optional[str] = None  # form "fmr": the program text
    # form "fmr": cells per thread along axis 0 in the generated kernels (values shared by
    # consecutive cells carried in registers); 0 = automatic (up to 16, keeping ~150k threads)
    march_chunk: int = 0
    # form "fmr": 2 = two cells per thread adjacent along axis 1, sharing values (needs 3+ axes
    # and an even extent of axis 1; measured slower on gray-scott-3d), 0 or 1 = one cell
    march_pair: int = 0
    # form "fmr": the temporally blocked kernel (temporal_blocking_interval steps per pass,
    # emit_cuda.TBEmitter): 0 = when the step is light and binary32 (emit_cuda.tb_profitable)
    # and its plane region (tile plus halo) holds at most twice the cells it writes,
    # 1 = whenever the program allows it,
    # -1 = never (one step per launch; temporal_blocking_interval then only rounds M)
    tb_kernel: int = 0

    @property
    def dim(self) -> int:
        return len(self.intra_node_shape)

    @property
    def axis_names(self) -> List[str]:
        if self.form == "fmr":
            return list(self.compiled().axes)
        return list(self.axes) if self.axes else list(AXES3[: self.dim])

    def compiled(self):
        """The manifested program of a form-"fmr" Program (cached)."""
        from .fmr import compile_source

        return compile_source(self.fmr_source, tuple(self.shape))

    def states(self) -> List[Tuple[str, str]]:
        """(name, C element type) of every global state array."""
        if self.form == "fmr":
            return list(self.compiled().state)
        return [(n, self.elem) for n in self.state_names + self.extra_state_names]

    @property
    def shape(self) -> List[int]:
        g = self.mpi_grid_shape or [1] * self.dim
        return [int(i) * int(m) for i, m in zip(self.intra_node_shape, g)]

    @property
    def steps_per_forward(self) -> int:
        """M of Translate.hs:1111-1113: monitor_interval rounded up to 2*tb."""
        tb2 = 2 * max(1, int(self.temporal_blocking_interval))
        m = int(self.monitor_interval)
        return ((m + tb2 - 1) // tb2) * tb2

    @property
    def elem(self) -> str:
        return "float" if "f32" in self.form else "double"

    @property
    def state_names(self) -> List[str]:
        return ["dens"] if self.form.startswith("diff") else ["U", "V"]

    @property
    def extra_state_names(self) -> List[str]:
        # Kahan compensation arrays carried between calls.
        return ["U_compensation", "V_compensation"] if "f32k" in self.form else []

    def validate(self) -> None:
        if self.mpi_grid_shape and any(int(m) != 1 for m in self.mpi_grid_shape):
            raise ValueError(
                "%s: mpi_grid_shape %s — this engine runs one GPU per program; the "
                "domain is periodic on that GPU (use [1,...])" % (self.name, list(self.mpi_grid_shape)))
        if self.form == "fmr":
            if not self.fmr_source:
                raise ValueError("%s: form fmr needs fmr_source" % self.name)
            if self.monitor_interval < 1:
                raise ValueError("%s: monitor_interval must be >= 1" % self.name)
            if self.march_chunk < 0:
                raise ValueError("%s: march_chunk must be >= 0 (0 = automatic)" % self.name)
            if self.march_pair not in (0, 1, 2):
                raise ValueError("%s: march_pair must be 0, 1 or 2" % self.name)
            if self.tb_kernel not in (-1, 0, 1):
                raise ValueError("%s: tb_kernel must be -1, 0 or 1" % self.name)
            self.compiled()
            return
        if self.form not in FORMS:
            raise ValueError("%s: unknown form %r (known: %s)" % (self.name, self.form, sorted(FORMS)))
        want_dim = FORMS[self.form]["dim"]
        if self.dim != want_dim:
            raise ValueError("%s: form %s is %dD, shape %s" % (self.name, self.form, want_dim,
                                                              list(self.intra_node_shape)))
        for key in FORMS[self.form]["constants"]:
            if key not in self.constants:
                raise ValueError("%s: constant %s missing" % (self.name, key))
        if self.monitor_interval < 1:
            raise ValueError("%s: monitor_interval must be >= 1" % self.name)


FORMS = {
    "gs3d_f64": {"dim": 3, "constants": ("F", "k", "Du", "Dv", "dt", "dx")},
    "gs3d_f32k": {"dim": 3, "constants": ("F", "k", "Du", "Dv", "dt", "dx")},
    "gs3d_f32k_tb": {"dim": 3, "constants": ("F", "k", "Du", "Dv", "dt", "dx")},
    "diff2d_f64": {"dim": 2, "constants": ("Dt", "Dx")},
}


def _delta_name(delta: Sequence[int]) -> str:
    # Translate.hs:406-407 + toCName (:317-343): "mpi_rank_" + "_1_0_m1"
    return "mpi_rank_" + "".join("_" + ("m%d" % -d if d < 0 else "%d" % d) for d in delta)


def _c_double(v: float) -> str:
    return repr(float(v))


def emit_header(p: Program) -> str:
    p.validate()
    ax = p.axis_names
    dims = "".join("[%d]" % n for n in p.shape)
    lines = [
        "/* %s.h — emitted by formura_gb300.backend (form %s). */" % (p.name, p.form),
        "",
        "#pragma once",
        "#ifdef __cplusplus",
        'extern "C"',
        "{",
        "#endif",
        "#include <stdint.h>",
        '#include "formura_mpi_stub.h"',
        "",
    ]
    for a, n in zip(ax, p.shape):
        lines.append("#define N%s  %d" % (a.upper(), n))
    lines.append("")
    for s, t in p.states():
        lines.append("extern %s %s%s;" % (t, s, dims))
    lines.append("")
    lines.append("struct Formura_Navigator {")
    lines.append("int time_step;")
    for a in ax:
        lines.append("int lower_%s;" % a)
        lines.append("int upper_%s;" % a)
        lines.append("int offset_%s;" % a)
    lines.append("union { MPI_Comm mpi_comm; uint64_t mpi_comm_storage_; };")
    lines.append("int mpi_my_rank;")
    for delta in itertools.product((-1, 0, 1), repeat=p.dim):
        lines.append("int %s;" % _delta_name(delta))
    lines.append("};")
    lines.append("extern struct Formura_Navigator navi;")
    lines.append("")
    lines.append("int Formura_Init (struct Formura_Navigator *navi, MPI_Comm comm);")
    lines.append("int Formura_Forward (struct Formura_Navigator *navi);")
    lines.append("")
    lines.append("/* Extensions of the GB300 engine (no counterpart in the generated C). */")
    lines.append("#define FORMURA_STEPS_PER_FORWARD %d" % p.steps_per_forward)
    lines.append("int Formura_Upload (void);")
    lines.append("int Formura_Advance (struct Formura_Navigator *navi, int n_forward);")
    lines.append("int Formura_Download (void);")
    lines.append("void *Formura_Device_State (int index);")
    lines.append("int Formura_Set_Stream (void *cuda_stream);")
    lines.append("int Formura_Conserved_Totals (double *totals);")
    lines.append("int Formura_Finalize (void);")
    lines.append("/* Number of state arrays whose host globals are page-locked (registered with")
    lines.append("   CUDA on the first device use), so that Forward's copies run at link speed;")
    lines.append("   a failed registration leaves its message in Formura_Last_Error. */")
    lines.append("int Formura_Host_Pinned (void);")
    lines.append("/* Monitor planes of the device state: Begin gathers plane `index` of axis")
    lines.append("   `axis` of every state array (asynchronous copy to the host); Wait writes")
    lines.append("   them, state after state, to `out`.  Write_Monitor writes the mid-planes of")
    lines.append("   axes 0..d-2 in the format of examples/pearson-3d-main.cpp write_monitor. */")
    lines.append("int Formura_Monitor_Begin (int axis, int index);")
    lines.append("int Formura_Monitor_Wait (void *out);")
    lines.append("int Formura_Write_Monitor (const char *dir, int rank);")
    lines.append("const char *Formura_Last_Error (void);")
    lines += ["", "#ifdef __cplusplus", "}", "#endif", ""]
    return "\n".join(lines)


def _forward_call(p: Program) -> str:
    c = p.constants
    nx = p.shape
    if p.form == "gs3d_f64":
        return (
            "fm_gs_params prm = {%s, %s, %s, %s, %s, %s};\n"
            "  return fm_gs3d_f64_forward(%d, %d, %d, (double*)g_dev[0], (double*)g_dev[1],"
            " (double*)g_work, (double*)g_work + NCELLS, &prm, steps, g_stream);"
            % (_c_double(c["F"]), _c_double(c["k"]), _c_double(c["Du"]), _c_double(c["Dv"]),
               _c_double(c["dt"]), _c_double(c["dx"]), nx[0], nx[1], nx[2]))
    if p.form == "gs3d_f32k":
        return (
            "fm_gs_params prm = {%s, %s, %s, %s, %s, %s};\n"
            "  return fm_gs3d_f32k_forward(%d, %d, %d, (float*)g_dev[0], (float*)g_dev[1],"
            " (float*)g_dev[2], (float*)g_dev[3], (float*)g_work, steps, &prm, g_stream);"
            % (_c_double(c["F"]), _c_double(c["k"]), _c_double(c["Du"]), _c_double(c["Dv"]),
               _c_double(c["dt"]), _c_double(c["dx"]), nx[0], nx[1], nx[2]))
    if p.form == "gs3d_f32k_tb":
        # depth per HBM pass: the kernel's tuned default (0) unless the YAML asks
        # for something smaller than the on-chip maximum of 4
        tb = int(p.temporal_blocking_interval)
        tb = tb if 1 <= tb < 4 else 0
        return (
            "fm_gs_params prm = {%s, %s, %s, %s, %s, %s};\n"
            "  return fm_gs3d_f32k_tb_forward(%d, %d, %d, (float*)g_dev[0], (float*)g_dev[1],"
            " (float*)g_dev[2], (float*)g_dev[3], (float*)g_work, steps, %d, &prm, g_stream);"
            % (_c_double(c["F"]), _c_double(c["k"]), _c_double(c["Du"]), _c_double(c["Dv"]),
               _c_double(c["dt"]), _c_double(c["dx"]), nx[0], nx[1], nx[2], tb))
    if p.form == "diff2d_f64":
        # node pair pow(Dx,2) then Dt/that, evaluated in double by host libm as the
        # generated C does (`**` -> pow, Translate.hs:594)
        return (
            "const double coef = %s / pow(%s, 2.0);\n"
            "  return fm_diff2d_f64_forward(%d, %d, (double*)g_dev[0], (double*)g_work, coef,"
            " steps, g_stream);" % (_c_double(c["Dt"]), _c_double(c["Dx"]), nx[0], nx[1]))
    raise ValueError(p.form)


def _work_elems(p: Program) -> str:
    if p.form == "gs3d_f64":
        return "2 * NCELLS"
    if p.form in ("gs3d_f32k", "gs3d_f32k_tb"):
        return "4 * NCELLS"
    return "NCELLS"




def blocked_kernel(p: Program):
    """The temporally blocked kernel of a form-"fmr" program, as
    emit_cuda.emit_tb_kernel returns it, when the program takes one (see
    Program.tb_kernel), else None."""
    from .fmr.emit_cuda import emit_tb_kernel, tb_profitable

    T = int(p.temporal_blocking_interval)
    if p.form != "fmr" or p.tb_kernel < 0 or T < 2:
        return None
    r = emit_tb_kernel(p.compiled(), T)
    if r is None:
        return None
    plan = r[1]
    cells = tile = 1
    for a in range(1, plan.dim):
        cells *= plan.RG[a]
        tile *= plan.TI[a]
    if p.tb_kernel == 0 and (cells > 2 * tile  # the halo would double the work per plane
                             or not tb_profitable(p.compiled())):
        return None
    return r


def _fmr_parts(p: Program):
    """Kernels, device buffers and the step loop of a form-"fmr" program."""
    from .fmr.emit_cuda import TB_THREADS, emit_kernels

    mmp = p.compiled()
    kern, levels = emit_kernels(mmp, march_chunk=p.march_chunk, march_pair=p.march_pair)
    tb = blocked_kernel(p)
    if tb is not None:
        kern += "\n" + tb[0]
    states = [n for n, _ in mmp.state]
    sidx = {n: i for i, n in enumerate(states)}
    arrays = sorted(mmp.arrays.values(), key=lambda a: a.node)
    aidx = {a.node: i for i, a in enumerate(arrays if arrays else [])}
    alloc = ["  for (int i = 0; i < kNState; ++i)",
             '    if ((st = fm_malloc(&g_next[i], kBytes[i]))) return fail(st, "fm_malloc(next)");']
    inner = [a for a in arrays if a.store_of is None]
    for a in inner:
        alloc.append('  if ((st = fm_malloc(&g_arr[%d], NCELLS * sizeof(%s)))) return fail(st, "fm_malloc(array)");'
                     % (aidx[a.node], a.ctype))
    alloc.append("  { int dev = 0; cudaGetDevice(&dev); int sms = 0;"
                 " cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);"
                 " long long need = ((long long)NCELLS + 255) / 256;"
                 " g_grid = (int)(need < (long long)sms * 16 ? need : (long long)sms * 16); }")
    run = ["  cudaStream_t s = (cudaStream_t)g_stream;", "  int t = 0;"]
    if tb is not None:
        _, plan, sn_tb, aw_tb = tb
        alloc.append("  if (cudaFuncSetAttribute(fmr_level_tb, cudaFuncAttributeMaxDynamicSharedMemorySize,"
                     " %d) != cudaSuccess) return fail(FM_ERR_CUDA, \"blocked kernel shared memory\");"
                     % plan.smem)
        alloc.append("  { int dev = 0; cudaGetDevice(&dev); int sms = 0;"
                     " cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);"
                     " g_grid_tb = %d < sms ? %d : sms; }" % (plan.ntiles, plan.ntiles))
        args = ["(const %s*)g_dev[%d]" % (dict(mmp.state)[n], sidx[n]) for n in sn_tb]
        args += ["(%s*)g_next[%d]" % (a.ctype, sidx[a.store_of]) for a in aw_tb]
        args += ["g_tm[g_dev[%d] == g_tm_base[0][%d] ? 0 : 1][%d]" % (sidx[n], sidx[n], sidx[n])
                 for n in sn_tb]
        args += ["g_use_tma", "g_err"]
        # the error word of the blocked kernel's bounded TMA waits, and the tensor maps of
        # both buffers of every state it reads (box: one plane of its tile region)
        alloc.append('  if ((st = fm_malloc((void**)&g_err, sizeof(int)))) return fail(st, "fm_malloc(err)");')
        alloc.append('  if ((st = fm_memset(g_err, 0, sizeof(int), g_stream))) return fail(st, "err");')
        if plan.tma:
            sh = p.shape
            alloc.append("  g_use_tma = 1;")
            for n in sn_tb:
                i = sidx[n]
                for b, buf in ((0, "g_dev"), (1, "g_next")):
                    alloc.append("  g_tm_base[%d][%d] = %s[%d];" % (b, i, buf, i))
                    alloc.append("  if (fm_tensor_map_3d(&g_tm[%d][%d], %s[%d], %d, %d, %d, %d, 1, %d, %d))"
                                 " g_use_tma = 0;  /* no encoder: gather every tile */"
                                 % (b, i, buf, i, plan.sizes[n], sh[0], sh[1], sh[2],
                                    plan.RG[1], plan.RG[2]))
        run += ["  /* %d steps per pass of the blocked kernel, the rest one step per launch */" % plan.T,
                "  for (; t + %d <= steps; t += %d) {" % (plan.T, plan.T),
                "    fmr_level_tb<<<g_grid_tb, %d, %d, s>>>(%s);" % (TB_THREADS, plan.smem,
                                                                   ", ".join(args)),
                "    for (int i = 0; i < kNState; ++i) { void *x = g_dev[i]; g_dev[i] = g_next[i]; g_next[i] = x; }",
                "  }"]
    run += ["  for (; t < steps; ++t) {"]
    for kname, sn, ar, aw in levels:
        args = ["(const %s*)g_dev[%d]" % (dict(mmp.state)[n], sidx[n]) for n in sn]
        args += ["(const %s*)g_arr[%d]" % (mmp.arrays[x].ctype, aidx[x]) if mmp.arrays[x].store_of is None
                 else "(const %s*)g_next[%d]" % (mmp.arrays[x].ctype, sidx[mmp.arrays[x].store_of])
                 for x in ar]
        for arr in aw:
            if arr.store_of is None:
                args.append("(%s*)g_arr[%d]" % (arr.ctype, aidx[arr.node]))
            else:
                args.append("(%s*)g_next[%d]" % (arr.ctype, sidx[arr.store_of]))
        run.append("    %s<<<g_grid, 256, 0, s>>>(%s);" % (kname, ", ".join(args)))
    run += ["    for (int i = 0; i < kNState; ++i) { void *x = g_dev[i]; g_dev[i] = g_next[i]; g_next[i] = x; }",
            "  }",
            "  cudaError_t e = cudaGetLastError();",
            "  if (e != cudaSuccess) {",
            '    snprintf(g_msg, sizeof g_msg, "generated kernels: %s", cudaGetErrorString(e));',
            "    return FM_ERR_CUDA;",
            "  }",
            "  return 0;"]
    free = ["  for (int i = 0; i < kNState; ++i) { fm_free(g_next[i]); g_next[i] = 0; }"]
    free += ["  fm_free(g_arr[%d]); g_arr[%d] = 0;" % (aidx[a.node], aidx[a.node]) for a in inner]
    decls = ["static void *g_next[%d] = {0};" % max(1, len(states)),
             "static void *g_arr[%d] = {0};" % max(1, len(arrays)),
             "static int g_grid = 1;", "static int g_grid_tb = 1;"]
    check = []
    if tb is not None:
        decls += ["alignas(64) static CUtensorMap g_tm[2][%d];" % max(1, len(states)),
                  "static void *g_tm_base[2][%d] = {{0}};" % max(1, len(states)),
                  "static int g_use_tma = 0;", "static int *g_err = 0;"]
        free += ["  fm_free(g_err); g_err = 0;"]
        # after Download's stream synchronization: did a bounded wait of the blocked kernel
        # give up since the last check?
        check = ["  { int e = 0;",
                 '    if ((st = fm_memcpy_d2h(&e, g_err, sizeof(int), g_stream)) || (st = fm_stream_sync(g_stream))) return fail(st, "error word");',
                 "    if (e) { fm_memset(g_err, 0, sizeof(int), g_stream); fm_stream_sync(g_stream);",
                 '      return fail(FM_ERR_TIMEOUT, "blocked kernel: a TMA wait gave up"); } }']
    return kern, decls, alloc, run, free, check


def emit_source(p: Program) -> str:
    """The host side of the generated-code API (``<name>.cpp``, or for form
    "fmr" ``<name>.cu`` with the generated kernels in front of it)."""
    p.validate()
    dims = "".join("[%d]" % n for n in p.shape)
    states = p.states()
    ncells = 1
    for n in p.shape:
        ncells *= n
    ax = p.axis_names
    fmr = p.form == "fmr"
    out: List[str] = []
    w = out.append
    w("/* %s.%s — emitted by formura_gb300.backend (form %s).\n"
      " * Host side of Formura's generated-code API on one GB300; the time steps run\n"
      " * in %s. */" % (p.name, "cu" if fmr else "cpp", p.form,
                       "the kernels generated below" if fmr else
                       "libformura_gb300.so (include/formura_gb300.h)"))
    w('#include "%s.h"' % p.name)
    w('#include "formura_gb300.h"')
    w("#include <math.h>")
    w("#include <ctype.h>")
    w("#include <stddef.h>")
    w("#include <stdio.h>")
    w("#include <stdlib.h>")
    if fmr:
        w("#include <cuda.h>")
        w("#include <cuda_runtime.h>")
        w('#include "fm_softfp.cuh"')
        w('#include "fm_tc.cuh"')
        w("#define FMR_TMAP const __grid_constant__ CUtensorMap")
    w("")
    w("#define NCELLS ((size_t)%d)" % ncells)
    w("#define FMR_EXPORT __attribute__((visibility(\"default\")))")
    w("")
    if fmr:
        kern, decls, alloc, run, free, check = _fmr_parts(p)
        w("namespace {")
        w(kern)
        w("}  // namespace")
        w("")
    w('extern "C" {')
    for sname, t in states:
        w("FMR_EXPORT %s %s%s __attribute__((aligned(4096)));" % (t, sname, dims))
    w("FMR_EXPORT struct Formura_Navigator navi;")
    w("}")
    w("")
    w("static const int kNState = %d;" % len(states))
    w("static void *const kHost[%d] = {%s};" % (len(states), ", ".join("(void*)%s" % n for n, _ in states)))
    w("static const size_t kBytes[%d] = {%s};" % (len(states), ", ".join("NCELLS * sizeof(%s)" % t for _, t in states)))
    w("static const int kIsDouble[%d] = {%s};" % (len(states), ", ".join("1" if t == "double" else "0" for _, t in states)))
    w("static const int kIsFloat[%d] = {%s};" % (len(states), ", ".join("1" if t == "float" else "0" for _, t in states)))
    w("static void *g_dev[%d] = {0};" % len(states))
    w("static void *g_work = 0;")
    w("static double *g_totals = 0;   /* device: per-state totals + scratch */")
    w("static void *g_stream = 0;")
    w("static int g_ready = 0;")
    w("static int g_pinned = 0;")
    w("static char g_msg[600];")
    w("static fm_snapshot *g_snap[%d] = {0};" % len(states))
    w("static int g_snap_axis = -1;")
    w("static const int kShape[%d] = {%s};" % (p.dim, ", ".join(str(n) for n in p.shape)))
    w("static const char *const kAxisNames[%d] = {%s};" % (p.dim, ", ".join('"%s"' % a for a in ax)))
    if fmr:
        for d in decls:
            w(d)
    w("")
    w("static int fail(int st, const char *where) {")
    w('  snprintf(g_msg, sizeof g_msg, "%s: %s (%s)", where, fm_status_name(st), fm_last_error());')
    w("  return st;")
    w("}")
    w("")
    w("static int ensure_device(void) {")
    w("  if (g_ready) return 0;")
    w("  int st;")
    w("  for (int i = 0; i < kNState; ++i) {")
    w('    if ((st = fm_malloc(&g_dev[i], kBytes[i]))) return fail(st, "fm_malloc(state)");')
    w("    /* page-locked host globals give full-speed copies; a failure is recorded, not fatal */")
    w("    if ((st = fm_host_register(kHost[i], kBytes[i])) == 0) ++g_pinned;")
    w('    else fail(st, "fm_host_register(state)");')
    w("  }")
    if fmr:
        for line in alloc:
            w(line)
    else:
        w('  if ((st = fm_malloc(&g_work, (%s) * sizeof(%s)))) return fail(st, "fm_malloc(work)");'
          % (_work_elems(p), p.elem))
    w("  const size_t scratch = fm_sum_f64_scratch_elems((int64_t)NCELLS);")
    w('  if ((st = fm_malloc((void**)&g_totals, (kNState + scratch) * sizeof(double)))) return fail(st, "fm_malloc(totals)");')
    w("  g_ready = 1;")
    w("  return 0;")
    w("}")
    w("")
    w("static int run_steps(int steps) {")
    if fmr:
        for line in run:
            w(line)
    else:
        w("  %s" % _forward_call(p))
    w("}")
    w("")
    w('extern "C" {')
    w("")
    w("FMR_EXPORT int Formura_Init (struct Formura_Navigator *nv, MPI_Comm comm) {")
    w("  nv->mpi_comm_storage_ = 0;")
    w("  nv->mpi_comm = comm;")
    w("  nv->mpi_my_rank = 0;")
    for delta in itertools.product((-1, 0, 1), repeat=p.dim):
        w("  nv->%s = 0;" % _delta_name(delta))
    w("  nv->time_step = 0;")
    for a, n in zip(ax, p.shape):
        w("  nv->offset_%s = 0; nv->lower_%s = 0; nv->upper_%s = %d;" % (a, a, a, n))
    w("  return 0;")
    w("}")
    w("")
    w("FMR_EXPORT int Formura_Upload (void) {")
    w("  int st = ensure_device(); if (st) return st;")
    w("  for (int i = 0; i < kNState; ++i)")
    w('    if ((st = fm_memcpy_h2d(g_dev[i], kHost[i], kBytes[i], g_stream))) return fail(st, "upload");')
    w("  return 0;")
    w("}")
    w("")
    w("FMR_EXPORT int Formura_Download (void) {")
    w("  int st = ensure_device(); if (st) return st;")
    w("  for (int i = 0; i < kNState; ++i)")
    w('    if ((st = fm_memcpy_d2h(kHost[i], g_dev[i], kBytes[i], g_stream))) return fail(st, "download");')
    w('  if ((st = fm_stream_sync(g_stream))) return fail(st, "download sync");')
    if fmr:
        for line in check:
            w(line)
    w("  return 0;")
    w("}")
    w("")
    w("FMR_EXPORT int Formura_Advance (struct Formura_Navigator *nv, int n_forward) {")
    w("  int st = ensure_device(); if (st) return st;")
    w("  if (n_forward < 0) return fail(FM_ERR_ARG, \"Formura_Advance: n_forward < 0\");")
    w("  for (int i = 0; i < n_forward; ++i) {")
    w('    if ((st = run_steps(FORMURA_STEPS_PER_FORWARD))) return fail(st, "Formura_Advance");')
    w("    nv->time_step += FORMURA_STEPS_PER_FORWARD;")
    w("  }")
    w("  return 0;")
    w("}")
    w("")
    w("FMR_EXPORT int Formura_Forward (struct Formura_Navigator *nv) {")
    w("  int st;")
    w("  if ((st = Formura_Upload())) return st;")
    w("  if ((st = Formura_Advance(nv, 1))) return st;")
    w("  return Formura_Download();")
    w("}")
    w("")
    w("FMR_EXPORT void *Formura_Device_State (int index) {")
    w("  if (ensure_device() || index < 0 || index >= kNState) return 0;")
    w("  return g_dev[index];")
    w("}")
    w("")
    w("FMR_EXPORT int Formura_Set_Stream (void *cuda_stream) { g_stream = cuda_stream; return 0; }")
    w("")
    w("FMR_EXPORT int Formura_Conserved_Totals (double *totals) {")
    w("  int st = ensure_device(); if (st) return st;")
    w("  if (!totals) return fail(FM_ERR_ARG, \"Formura_Conserved_Totals: NULL\");")
    w("  if ((st = fm_memset(g_totals, 0, kNState * sizeof(double), g_stream))) return fail(st, \"totals\");")
    w("  for (int i = 0; i < kNState; ++i) {")
    w("    if (kIsDouble[i])")
    w("      st = fm_sum_f64((int64_t)NCELLS, (const double*)g_dev[i], g_totals + kNState, g_totals + i, g_stream);")
    w("    else if (kIsFloat[i])")
    w("      st = fm_sum_f32_as_f64((int64_t)NCELLS, (const float*)g_dev[i], g_totals + kNState, g_totals + i, g_stream);")
    w('    if (st) return fail(st, "conserved totals");')
    w("  }")
    w('  if ((st = fm_memcpy_d2h(totals, g_totals, kNState * sizeof(double), g_stream))) return fail(st, "totals");')
    w('  if ((st = fm_stream_sync(g_stream))) return fail(st, "totals sync");')
    w("  for (int i = 0; i < kNState; ++i) if (!isfinite(totals[i])) return fail(FM_ERR_NONFINITE, \"non-finite state\");")
    w("  return 0;")
    w("}")
    w("")
    w("FMR_EXPORT int Formura_Finalize (void) {")
    w("  if (!g_ready) return 0;")
    w("  fm_stream_sync(g_stream);")
    w("  for (int i = 0; i < kNState; ++i) { fm_free(g_dev[i]); g_dev[i] = 0; fm_host_unregister(kHost[i]); }")
    w("  g_pinned = 0;")
    w("  fm_free(g_work); g_work = 0; fm_free(g_totals); g_totals = 0;")
    w("  for (int i = 0; i < kNState; ++i) { fm_snapshot_destroy(g_snap[i]); g_snap[i] = 0; }")
    w("  g_snap_axis = -1;")
    if fmr:
        for line in free:
            w(line)
    w("  g_ready = 0;")
    w("  return 0;")
    w("}")
    w("")
    w("FMR_EXPORT const char *Formura_Last_Error (void) { return g_msg; }")
    w("")
    w("FMR_EXPORT int Formura_Host_Pinned (void) { return g_pinned; }")
    w("")
    w("FMR_EXPORT int Formura_Monitor_Begin (int axis, int index) {")
    w("  int st = ensure_device(); if (st) return st;")
    w("  for (int i = 0; i < kNState; ++i) {")
    w("    if (!g_snap[i] && (st = fm_snapshot_create(&g_snap[i], %d, kShape, (int)(kBytes[i] / NCELLS))))" % p.dim)
    w('      return fail(st, "Formura_Monitor_Begin");')
    w("    if ((st = fm_snapshot_begin(g_snap[i], g_dev[i], axis, index, g_stream))) return fail(st, \"Formura_Monitor_Begin\");")
    w("  }")
    w("  g_snap_axis = axis;")
    w("  return 0;")
    w("}")
    w("")
    w("FMR_EXPORT int Formura_Monitor_Wait (void *out) {")
    w("  if (g_snap_axis < 0) return fail(FM_ERR_ARG, \"Formura_Monitor_Wait: no plane in flight\");")
    w("  char *o = (char*)out;")
    w("  int st;")
    w("  for (int i = 0; i < kNState; ++i) {")
    w("    if ((st = fm_snapshot_wait(g_snap[i], o))) return fail(st, \"Formura_Monitor_Wait\");")
    w("    o += (size_t)fm_snapshot_plane_elems(g_snap[i], g_snap_axis) * (kBytes[i] / NCELLS);")
    w("  }")
    w("  g_snap_axis = -1;")
    w("  return 0;")
    w("}")
    w("")
    w("FMR_EXPORT int Formura_Write_Monitor (const char *dir, int rank) {")
    w("  int st = ensure_device(); if (st) return st;")
    w("  int pos[%d];" % (2 * p.dim))
    w("  for (int a = 0; a < %d; ++a) { pos[a] = 0; pos[%d + a] = kShape[a]; }" % (p.dim, p.dim))
    w("  for (int a = 0; a + 1 < %d || (%d == 1 && a == 0); ++a) {" % (p.dim, p.dim))
    w("    size_t bytes = 0;")
    w("    for (int i = 0; i < kNState; ++i) bytes += (size_t)(NCELLS / kShape[a]) * (kBytes[i] / NCELLS);")
    w("    void *buf = malloc(bytes);")
    w('    if (!buf) return fail(FM_ERR_NOMEM, "Formura_Write_Monitor");')
    w("    if ((st = Formura_Monitor_Begin(a, kShape[a] / 2)) || (st = Formura_Monitor_Wait(buf))) { free(buf); return st; }")
    w("    char fn[1024], up[64];")
    w("    size_t k = 0;")
    w("    for (; kAxisNames[a][k] && k + 1 < sizeof up; ++k) up[k] = (char)toupper((unsigned char)kAxisNames[a][k]);")
    w("    up[k] = 0;")
    w('    snprintf(fn, sizeof fn, "%s/monitor%s-%06d-%d.txt", dir, up, navi.time_step, rank);')
    w('    FILE *fp = fopen(fn, "wb");')
    w('    if (!fp) { free(buf); snprintf(g_msg, sizeof g_msg, "cannot open %s", fn); return FM_ERR_ARG; }')
    w("    fwrite(pos, sizeof(int), %d, fp);" % (2 * p.dim))
    w("    fwrite(buf, 1, bytes, fp);")
    w("    fclose(fp);")
    w("    free(buf);")
    w("  }")
    w("  return 0;")
    w("}")
    w("")
    w("}  /* extern \"C\" */")
    w("")
    return "\n".join(out)


def program_dir(root: Optional[Path] = None) -> Path:
    return (root or _build.BUILD) / "programs"


def build_program(p: Program, outdir: Optional[Path] = None, verbose: bool = False) -> Path:
    """Emit ``<name>.h``/``<name>.cpp`` and compile ``lib<name>.so`` (g++)."""
    outdir = Path(outdir) if outdir else program_dir()
    outdir.mkdir(parents=True, exist_ok=True)
    hdr, src = emit_header(p), emit_source(p)
    lib = _build.LIB
    if not lib.exists():
        _build.build_library(verbose=verbose)
    key = hashlib.sha256((hdr + src + str(lib.stat().st_mtime_ns)).encode()).hexdigest()[:16]
    so = outdir / ("lib%s.so" % p.name)
    stamp = outdir / ("lib%s.stamp" % p.name)
    if so.exists() and stamp.exists() and stamp.read_text() == key:
        return so
    (outdir / (p.name + ".h")).write_text(hdr)
    if p.form == "fmr":
        # generated kernels: nvcc with the library's flags (sm_103a, no FMA contraction)
        (outdir / (p.name + ".cu")).write_text(src)
        cmd = [
            _build._nvcc(), *_build.NVCC_FLAGS, "-shared", "-I", str(outdir),
            "-I", str(_build.INCLUDE), "-I", str(_build.CSRC),
            "-o", str(so) + ".tmp", str(outdir / (p.name + ".cu")),
            "-L", str(lib.parent), "-lformura_gb300", "-cudart=shared",
            "-Xlinker", "-rpath," + str(lib.parent),
        ]
    else:
        (outdir / (p.name + ".cpp")).write_text(src)
        cmd = [
            os.environ.get("CXX", "g++"), "-O2", "-fPIC", "-shared", "-std=c++17",
            "-fvisibility=hidden", "-I", str(outdir), "-I", str(_build.INCLUDE),
            "-o", str(so) + ".tmp", str(outdir / (p.name + ".cpp")),
            "-L", str(lib.parent), "-lformura_gb300",
            "-Wl,-rpath," + str(lib.parent), "-lm",
        ]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("building %s failed:\n%s" % (p.name, r.stdout))
    os.replace(str(so) + ".tmp", so)
    stamp.write_text(key)
    return so


def build_programs(verbose: bool = False) -> List[Path]:
    from .programs import PROGRAMS

    return [build_program(p, verbose=verbose) for p in PROGRAMS.values()]
