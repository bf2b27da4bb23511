"""Host build of the CUDA kernels that the .fmr front end generates: test
infrastructure for the CPU suite.

The generated kernels are plain C++ apart from the launch qualifiers and the
grid-stride loop's built-in indices, and their exact binary64 forms
(csrc/fm_softfp.cuh) compile for the host as well.  So the emitted kernel
source is compiled with g++ under a prelude that defines those names for a
grid of one block of one thread: the single "thread" walks every item of the
grid-stride loop, i.e. every (column, chunk) work item of the marching and
pairing schedules, in order.  The step loop mirrors the generated host code
(formura_gb300/backend.py, `_fmr_parts`): each level reads the current state
and the arrays of earlier levels, and the state buffers swap after a step.
Floating-point contraction is off, as in the device build (--fmad=false).
"""
from __future__ import annotations

import ctypes
import hashlib
import re
import subprocess
import tempfile
from pathlib import Path
from typing import Dict

import numpy as np

from formura_gb300.fmr.emit_cuda import emit_kernels, emit_tb_kernel

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "formura_gb300" / "csrc"
BUILD = Path(tempfile.gettempdir()) / "fmr_host_kernels"
NP_TYPES = {"double": np.float64, "float": np.float32}

PRELUDE = r"""
#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include "fm_softfp.cuh"
#define __global__
#define __launch_bounds__(threads, blocks)
#define __syncthreads()
#define FMR_HOST_BUILD 1
#define FMR_TMAP const void *
namespace {
struct FmHostDim { unsigned x, y, z; };
// blockIdx and gridDim change only for the blocked kernel, whose blocks run one after another
FmHostDim blockIdx = {0u, 0u, 0u}, gridDim = {1u, 1u, 1u};
const FmHostDim threadIdx = {0u, 0u, 0u}, blockDim = {1u, 1u, 1u};
}  // namespace
"""


STORE = re.compile(r"^(\s*)(w_\w+)\[(.*)\] = (\w+);$")

COUNTING = r"""
#include <unordered_map>
#include <vector>
namespace {
std::unordered_map<const void *, std::vector<int>> g_store_count;
// Counts a store; false (and a count that fails the check) for an index out of range,
// whose store is then skipped.
bool count_store(const void *array, size_t i, size_t n) {
  std::vector<int> &c = g_store_count[array];
  if (c.empty()) c.assign(n, 0);
  if (i < n) { c[i] += 1; return true; }
  c[0] += 1000000;
  return false;
}
}  // namespace
extern "C" void fmr_host_store_counts(int *arrays, int *lo, int *hi) {
  int a = 0, mn = 1 << 30, mx = 0;
  for (auto &kv : g_store_count) {
    ++a;
    for (int c : kv.second) { mn = c < mn ? c : mn; mx = c > mx ? c : mx; }
  }
  *arrays = a; *lo = a ? mn : 0; *hi = mx;
  g_store_count.clear();
}
"""


def host_source(mmp, march_chunk: int = 0, march_pair: int = 0, soft: bool = True,
                count_stores: bool = False, tb: int = 1, tb_budget: int = 0, tb_grid: int = 5) -> str:
    """Host C++ of the generated kernels plus a step loop; `soft` False emits
    the plain IEEE operations instead of the integer-pipe forms.  With
    `count_stores` every store of a kernel also counts, per array and cell, how
    often it was written (read back by fmr_host_store_counts).  With tb >= 2
    the temporally blocked kernel runs tb steps per pass (the rest of the
    steps one per pass), as the generated host code does; `tb_budget` > 0
    shrinks its shared-memory budget (smaller tiles, more of them), and its
    `tb_grid` blocks run one after another, each marching its own contiguous
    run of column-planes (runs that start and end inside a column)."""
    kern, levels = emit_kernels(mmp, soft_div=soft, soft_mul=soft, soft_cmp=soft,
                                march_chunk=march_chunk, march_pair=march_pair)
    tbk = None
    if tb >= 2:
        kw = {"budget": tb_budget} if tb_budget else {}
        tbk = emit_tb_kernel(mmp, tb, soft_div=soft, soft_mul=soft, soft_cmp=soft, **kw)
        if tbk is None:
            raise ValueError("program cannot be temporally blocked")
        kern += "\n" + tbk[0]
    if count_stores:
        n = int(np.prod(mmp.shape))
        lines = []
        for line in kern.split("\n"):
            m = STORE.match(line)
            if m:
                line = "%sif (count_store(%s, (size_t)(%s), %dull)) %s[%s] = %s;" % (
                    m.group(1), m.group(2), m.group(3), n, m.group(2), m.group(3), m.group(4))
            lines.append(line)
        kern = "\n".join(lines)
    states = [n for n, _ in mmp.state]
    stype = dict(mmp.state)
    sidx = {n: i for i, n in enumerate(states)}
    arrays = sorted(mmp.arrays.values(), key=lambda a: a.node)
    aidx = {a.node: i for i, a in enumerate(arrays)}
    ncells = int(np.prod(mmp.shape))
    out = [PRELUDE, COUNTING if count_stores else "", "namespace {", kern, "}  // namespace", "",
           'extern "C" int fmr_host_run(int steps, void **state) {',
           "  const size_t n = %dull;" % ncells,
           "  void *cur[%d], *nxt[%d], *arr[%d];" % (len(states), len(states), max(1, len(arrays))),
           "  size_t bytes;"]
    w = out.append
    for i, s in enumerate(states):
        w("  bytes = n * sizeof(%s);" % stype[s])
        w("  cur[%d] = malloc(bytes); nxt[%d] = malloc(bytes);" % (i, i))
        w("  if (!cur[%d] || !nxt[%d]) return 1;" % (i, i))
        w("  memcpy(cur[%d], state[%d], bytes);" % (i, i))
    for a in arrays:
        if a.store_of is None:
            w("  arr[%d] = malloc(n * sizeof(%s)); if (!arr[%d]) return 1;" % (aidx[a.node], a.ctype,
                                                                                aidx[a.node]))
    w("  int t = 0;")
    if tbk is not None:
        _, plan, sn_tb, aw_tb = tbk
        args = ["(const %s*)cur[%d]" % (stype[s], sidx[s]) for s in sn_tb]
        args += ["(%s*)nxt[%d]" % (a.ctype, sidx[a.store_of]) for a in aw_tb]
        args += ["nullptr"] * len(sn_tb) + ["0", "&host_err"]  # no TMA on the host
        w("  int host_err = 0;")
        w("  for (; t + %d <= steps; t += %d) {" % (plan.T, plan.T))
        w("    gridDim.x = %du;" % tb_grid)
        w("    for (unsigned b = 0; b < %du; ++b) { blockIdx.x = b; fmr_level_tb(%s); }"
          % (tb_grid, ", ".join(args)))
        w("    gridDim.x = 1u; blockIdx.x = 0u;")
        w("    for (int i = 0; i < %d; ++i) { void *x = cur[i]; cur[i] = nxt[i]; nxt[i] = x; }"
          % len(states))
        w("  }")
    w("  for (; t < steps; ++t) {")
    for kname, sn, ar, aw in levels:
        args = ["(const %s*)cur[%d]" % (stype[s], sidx[s]) for s in sn]
        for x in ar:
            a = mmp.arrays[x]
            args.append("(const %s*)%s" % (a.ctype, "arr[%d]" % aidx[x] if a.store_of is None
                                           else "nxt[%d]" % sidx[a.store_of]))
        for a in aw:
            args.append("(%s*)%s" % (a.ctype, "arr[%d]" % aidx[a.node] if a.store_of is None
                                     else "nxt[%d]" % sidx[a.store_of]))
        w("    %s(%s);" % (kname, ", ".join(args)))
    w("    for (int i = 0; i < %d; ++i) { void *x = cur[i]; cur[i] = nxt[i]; nxt[i] = x; }"
      % len(states))
    w("  }")
    for i, s in enumerate(states):
        w("  memcpy(state[%d], cur[%d], n * sizeof(%s)); free(cur[%d]); free(nxt[%d]);"
          % (i, i, stype[s], i, i))
    for a in arrays:
        if a.store_of is None:
            w("  free(arr[%d]);" % aidx[a.node])
    w("  return 0;")
    w("}")
    return "\n".join(out) + "\n"


class HostKernels:
    """The generated kernels of one compiled program (mm.MMProgram), built for
    the host."""

    def __init__(self, mmp, march_chunk: int = 0, march_pair: int = 0, soft: bool = True,
                 count_stores: bool = False, tb: int = 1, tb_budget: int = 0):
        self.mmp = mmp
        self.source = host_source(mmp, march_chunk, march_pair, soft, count_stores, tb, tb_budget)
        key = hashlib.sha256((self.source + (CSRC / "fm_softfp.cuh").read_text()).encode())
        BUILD.mkdir(parents=True, exist_ok=True)
        so = BUILD / ("k_%s.so" % key.hexdigest()[:16])
        if not so.exists():
            src = so.with_suffix(".cpp")
            src.write_text(self.source)
            tmp = Path(str(so) + ".tmp")
            # -O0: the large generated programs compile 5x faster; the runs here are small
            subprocess.run(["g++", "-std=c++17", "-O0", "-ffp-contract=off", "-fPIC", "-shared",
                            "-w", "-I", str(CSRC), "-o", str(tmp), str(src), "-lm"], check=True)
            tmp.replace(so)
        self.lib = ctypes.CDLL(str(so))
        self.lib.fmr_host_run.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        self.count_stores = count_stores

    def run(self, state: Dict[str, np.ndarray], steps: int) -> Dict[str, np.ndarray]:
        arrs = [np.ascontiguousarray(state[n], dtype=NP_TYPES[t]).reshape(self.mmp.shape).copy()
                for n, t in self.mmp.state]
        ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        if self.lib.fmr_host_run(int(steps), ptrs) != 0:
            raise MemoryError("host kernel run: allocation failed")
        return {n: a for (n, _), a in zip(self.mmp.state, arrs)}

    def store_counts(self):
        """(arrays written, fewest and most writes of one cell) since the last
        call; needs count_stores."""
        assert self.count_stores
        a, lo, hi = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.lib.fmr_host_store_counts(ctypes.byref(a), ctypes.byref(lo), ctypes.byref(hi))
        return a.value, lo.value, hi.value


def asan_run(mmp, steps: int, tb: int = 1, tb_budget: int = 0):
    """Build the host kernels of `mmp` with AddressSanitizer into a standalone
    program, run `steps` steps on a fixed state, and return (exit status,
    sanitizer report).  Any access outside an array or outside the blocked
    kernel's shared-memory stand-in is reported, so a schedule that would read
    or write out of bounds on the GPU fails here, on the CPU."""
    src = host_source(mmp, tb=tb, tb_budget=tb_budget)
    n = int(np.prod(mmp.shape))
    lines = [src, "#include <stdio.h>", "int main() {"]
    for j, (_, t) in enumerate(mmp.state):
        lines.append("  static %s b%d[%d];" % (t, j, n))
        lines.append("  for (int i = 0; i < %d; ++i) b%d[i] = (%s)(0.3 + 0.001 * (i %% 97));" % (n, j, t))
    lines.append("  void *st[%d] = {%s};" % (len(mmp.state), ", ".join("b%d" % j for j in range(len(mmp.state)))))
    lines.append("  return fmr_host_run(%d, st);" % steps)
    lines.append("}")
    key = hashlib.sha256(("\n".join(lines) + (CSRC / "fm_softfp.cuh").read_text()).encode())
    BUILD.mkdir(parents=True, exist_ok=True)
    exe = BUILD / ("asan_%s" % key.hexdigest()[:16])
    if not exe.exists():
        cpp = exe.with_suffix(".cpp")
        cpp.write_text("\n".join(lines) + "\n")
        tmp = Path(str(exe) + ".tmp")
        subprocess.run(["g++", "-std=c++17", "-O0", "-g", "-fsanitize=address", "-ffp-contract=off",
                        "-w", "-I", str(CSRC), "-o", str(tmp), str(cpp), "-lm"], check=True)
        tmp.replace(exe)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    return r.returncode, r.stderr
