"""CPU oracle for programs compiled by the .fmr front end (test infrastructure).

Emits plain C loop nests for a manifested program the way the reference's C
back end writes them (src/Formura/MPICxx/Translate.hs:481-629, 671-737): one
temporary per node in the node's C type, literals as the correctly rounded
double of the exact rational (Translate.hs:585), constant sub-expressions
computed at run time in C (``fold_constants=False``), ``**`` -> ``pow``,
``>?``/``<?`` -> right-folded ``fmax``/``fmin`` (:604-609), ``<%`` ->
``fmin(0.0, fmax(..)) + fmax(0.0, fmin(..))``, ``if`` -> ``?:`` (:597-601),
periodic wrap of every cursor (:1062-1068).  Compiled with gcc
``-O2 -ffp-contract=off``.

It shares the parser, the OM evaluation and the manifestation with the
product path, so it checks the code generators, not the front end; the front
end is pinned separately: pearson.fmr through it reproduces the reference's
generated pearson.c bit for bit, and the forms that have hand-written
restatements (fmr_oracle.c, fmr_mhd.c) agree with it bit for bit
(tests/test_fmr_frontend.py).
"""
from __future__ import annotations

import ctypes
import hashlib
import subprocess
from pathlib import Path
from typing import Dict, List, Sequence

import numpy as np

from formura_gb300.fmr import mm as MM
from formura_gb300.fmr import om as OM
from formura_gb300.fmr import parser as P

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"

NP_TYPES = {"double": np.float64, "float": np.float32, "int": np.int32, "bool": np.bool_}


def _literal(v, ctype: str) -> str:
    return MM.c_literal(v, ctype)


def emit_c(mmp: MM.MMProgram) -> str:
    dim, shape = mmp.dim, mmp.shape
    ncells = int(np.prod(shape))
    out: List[str] = ["#include <math.h>", "#include <stdbool.h>", "#include <stddef.h>",
                      "#include <stdlib.h>", "#include <string.h>", ""]
    w = out.append
    stypes = dict(mmp.state)
    states = [n for n, _ in mmp.state]
    arrays = sorted(mmp.arrays.values(), key=lambda a: a.node)
    for a, n in enumerate(shape):
        w("#define N%d %d" % (a, n))
    w("")
    w("static int wrap(int c, int n) { c %= n; return c < 0 ? c + n : c; }")
    w("")
    # one function per level
    for li, L in enumerate(mmp.levels):
        w("static void level_%d(void **cur, void **arr, void **nxt) {" % li)
        for i, n in enumerate(states):
            w("  const %s *s_%s = (const %s*)cur[%d];" % (stypes[n], n, stypes[n], i))
        for j, a in enumerate(arrays):
            if a.store_of is None:
                w("  %s *r_%s = (%s*)arr[%d];" % (a.ctype, a.name, a.ctype, j))
            else:
                w("  %s *r_%s = (%s*)nxt[%d];" % (a.ctype, a.name, a.ctype, states.index(a.store_of)))
        loops = ["c%d" % a for a in range(dim)]
        for a in range(dim):
            w("  " * (a + 1) + "for (int c%d = 0; c%d < N%d; ++c%d) {" % (a, a, a, a))
        ind = "  " * (dim + 1)

        def idx(cursor):
            e = "(size_t)wrap(c0 + (%d), N0)" % cursor[0]
            for a in range(1, dim):
                e = "(%s * N%d + wrap(c%d + (%d), N%d))" % (e, a, a, cursor[a], a)
            return e

        for i, m in enumerate(L.micro):
            t, k = m.ctype, m.kind
            nm = "a%d" % i
            if k == "imm":
                w(ind + "%s %s = %s;" % (t, nm, _literal(float(m.args[0]) if t != "float" else
                                                         np.float32(float(m.args[0])), t)))
            elif k == "const":
                w(ind + "%s %s = %s;" % (t, nm, _literal(m.args[0], t)))
            elif k == "loadS":
                w(ind + "%s %s = s_%s[%s];" % (t, nm, m.args[1], idx(m.args[0])))
            elif k == "loadM":
                a = mmp.arrays[m.args[1]]
                w(ind + "%s %s = r_%s[%s];" % (t, nm, a.name, idx(m.args[0])))
            elif k == "index":
                w(ind + "%s %s = (%s)c%d;" % (t, nm, t, m.args[0]))
            elif k == "uni":
                op, a = m.args
                if op.startswith("external-call/"):
                    w(ind + "%s %s = (%s(a%d));" % (t, nm, op.split("/", 1)[1], a))
                else:
                    w(ind + "%s %s = (%sa%d);" % (t, nm, op, a))
            elif k == "bin":
                op, a, b = m.args
                if op == "**":
                    w(ind + "%s %s = pow(a%d, a%d);" % (t, nm, a, b))
                else:
                    w(ind + "%s %s = (a%d %s a%d);" % (t, nm, a, op, b))
            elif k == "ite":
                c, a, b = m.args
                w(ind + "%s %s = (a%d ? a%d : a%d);" % (t, nm, c, a, b))
            elif k == "nary":
                op, xs = m.args
                names = ["a%d" % x for x in xs]

                def chain(fn, items):
                    acc = items[-1]
                    for it in reversed(items[:-1]):
                        acc = "%s(%s, %s)" % (fn, it, acc)
                    return acc

                if op == ">?":
                    e = chain("fmax", names)
                elif op == "<?":
                    e = chain("fmin", names)
                else:
                    e = "fmin(0.0, %s) + fmax(0.0, %s)" % (chain("fmax", names), chain("fmin", names))
                w(ind + "%s %s = %s;" % (t, nm, e))
            else:
                raise OM.FmrSemanticError("oracle: cannot emit %s" % k)
        lin = "c0"
        for a in range(1, dim):
            lin = "(%s * N%d + c%d)" % (lin, a, a)
        for arr in L.arrays:
            w(ind + "r_%s[(size_t)%s] = a%d;" % (arr.name, lin, arr.root))
        for a in reversed(range(dim)):
            w("  " * (a + 1) + "}")
        w("}")
        w("")
    w("int fmr_run(int steps, void **state) {")
    w("  const size_t n = %d;" % ncells)
    w("  void *cur[%d], *nxt[%d], *arr[%d];" % (len(states), len(states), max(1, len(arrays))))
    sizes = ["sizeof(%s)" % stypes[s] for s in states]
    for i, s in enumerate(states):
        w("  cur[%d] = malloc(n * %s); nxt[%d] = malloc(n * %s);" % (i, sizes[i], i, sizes[i]))
        w("  if (!cur[%d] || !nxt[%d]) return 1;" % (i, i))
        w("  memcpy(cur[%d], state[%d], n * %s);" % (i, i, sizes[i]))
    for j, a in enumerate(arrays):
        w("  arr[%d] = %s;" % (j, "malloc(n * sizeof(%s))" % a.ctype if a.store_of is None else "0"))
    w("  for (int t = 0; t < steps; ++t) {")
    for li in range(len(mmp.levels)):
        w("    level_%d(cur, arr, nxt);" % li)
    w("    for (int i = 0; i < %d; ++i) { void *x = cur[i]; cur[i] = nxt[i]; nxt[i] = x; }" %
      len(states))
    w("  }")
    for i, s in enumerate(states):
        w("  memcpy(state[%d], cur[%d], n * %s); free(cur[%d]); free(nxt[%d]);" % (i, i, sizes[i], i, i))
    for j, a in enumerate(arrays):
        if a.store_of is None:
            w("  free(arr[%d]);" % j)
    w("  return 0;")
    w("}")
    return "\n".join(out) + "\n"


class FmrOracle:
    """The C oracle of one program at one grid shape."""

    def __init__(self, source: str, shape: Sequence[int]):
        prog = P.parse(source)
        omp = OM.build_om(prog, list(shape))
        self.mmp = MM.manifest(omp, list(shape), fold_constants=False)
        code = emit_c(self.mmp)
        key = hashlib.sha256(code.encode()).hexdigest()[:16]
        BUILD.mkdir(parents=True, exist_ok=True)
        so = BUILD / ("fmr_%s.so" % key)
        if not so.exists():
            src = BUILD / ("fmr_%s.c" % key)
            src.write_text(code)
            subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o",
                            str(so) + ".tmp", str(src), "-lm"], check=True)
            so_tmp = Path(str(so) + ".tmp")
            so_tmp.replace(so)
        self.lib = ctypes.CDLL(str(so))
        self.lib.fmr_run.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
        self.shape = list(shape)

    @property
    def state_names(self) -> List[str]:
        return [n for n, _ in self.mmp.state]

    def run(self, state: Dict[str, np.ndarray], steps: int) -> Dict[str, np.ndarray]:
        arrs = []
        for n, t in self.mmp.state:
            a = np.ascontiguousarray(state[n], dtype=NP_TYPES[t]).reshape(self.shape).copy()
            arrs.append(a)
        ptrs = (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        if self.lib.fmr_run(int(steps), ptrs) != 0:
            raise MemoryError("oracle allocation failed")
        return {n: a for (n, _), a in zip(self.mmp.state, arrs)}
