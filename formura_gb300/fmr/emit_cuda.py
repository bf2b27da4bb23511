"""CUDA code generation for a manifested Formura program.

One kernel per level of the manifested program (mm.Level): every thread
evaluates the level's cell program for one cell and writes each of the
level's arrays.  Arrays are dense, row-major, last axis fastest, with
periodic boundaries: a read at cursor c of axis a uses the wrapped coordinate
(x_a + c) mod N_a, computed once per (axis, cursor) per cell.  The grid
shape is a compile-time constant of the generated file.

Arithmetic keeps the C semantics of the reference's generated code
(src/Formura/MPICxx/Translate.hs:568-620): one IEEE operation per node in
the node's C type, ``**`` -> ``pow``, ``>?``/``<?`` -> right-folded
``fmax``/``fmin`` chains, ``<%`` -> ``fmin(0, fmax(..)) + fmax(0, fmin(..))``,
``if`` -> ``?:``, extern functions called on doubles.  The file is compiled
with ``--fmad=false``, so no multiply-add is contracted.  Exact
substitutions of binary64 operations by integer-pipe forms (bit-identical
results, csrc/fm_softfp.cuh), because the FP64 pipe is the scarce one:
  * x * 2^k and x / 2^k (a power-of-two constant): ``scale_pow2``;
  * x / d for another positive normal constant: ``div_const_s``;
  * x * y for another nonzero normal constant: ``mul_const_s``;
  * x / y for a run-time y: ``div_var_s``, one ``prep_div_s`` reciprocal
    per divisor node shared by all its quotients;
  * ``fmax``/``fmin`` chains (``>?``, ``<?``, ``<%``) and ``< <= > >= == !=``
    of two doubles: ``max_s``/``min_s`` and the ordered-key comparisons.
A float node whose C expression promotes a float operand against a double
constant that is exactly a float (``1``, ``0.5``, ``2``...) is evaluated in
float: the same bits (double rounding of binary32 operations through
binary64 is innocuous), without the FP64 pipe.
"""
from __future__ import annotations

import math
import struct
from typing import Dict, List, Optional, Sequence, Tuple

from . import mm as MM

AXVARS = ["c%d" % i for i in range(8)]


def _double_fields(d: float):
    b = struct.unpack("<Q", struct.pack("<d", d))[0]
    return b, (b & ((1 << 52) - 1)) | (1 << 52), (b >> 52) & 0x7FF


def div_const_fields(d: float) -> str:
    """Initializer of fm::soft::DivConstS for a positive normal d."""
    _, md, ed = _double_fields(d)
    R = -(-(1 << 115) // md)
    return "{%du, %du, %du, %du, %d, %s}" % (R >> 32, R & 0xFFFFFFFF, md >> 32, md & 0xFFFFFFFF,
                                           ed, float(d).hex())


def mul_const_fields(y: float) -> str:
    """Initializer of fm::soft::MulConstS for a nonzero normal y."""
    b, my, ey = _double_fields(y)
    bb = my << 11
    return "{%du, %du, %du, %du, %du, %d, %s}" % (bb >> 32, bb & 0xFFFFFFFF, my >> 32,
                                                 my & 0xFFFFFFFF, (b >> 32) & 0x80000000, ey,
                                                 float(y).hex())


def _normal_double(v) -> bool:
    if not isinstance(v, float):
        return False
    a = abs(v)
    return math.isfinite(a) and a >= 2.2250738585072014e-308


def _float_exact(v) -> bool:
    """A finite double constant that binary32 represents exactly."""
    if not isinstance(v, float) or not math.isfinite(v):
        return False
    return float(struct.unpack("<f", struct.pack("<f", v))[0]) == v


def _pow2_exponent(v):
    """k if v == 2**k for an integer |k| <= 62, else None."""
    if not isinstance(v, float) or not math.isfinite(v) or v <= 0:
        return None
    m, e = math.frexp(v)
    if m != 0.5 or abs(e - 1) > 62:
        return None
    return e - 1


CMP_SOFT = {"<": "fm::soft::lt_s(%s, %s)", "<=": "fm::soft::le_s(%s, %s)",
            ">": "fm::soft::lt_s(%s, %s)", ">=": "fm::soft::le_s(%s, %s)",
            "==": "fm::soft::eq_s(%s, %s)", "!=": "!fm::soft::eq_s(%s, %s)"}


def _wrap_name(ax: int, c: int, lane: str = "") -> str:
    """Variable holding the wrapped coordinate x_ax + c; `lane` "b" names the
    second cell of a thread's pair along axis 1."""
    base = AXVARS[ax] + (lane if ax == 1 else "")
    if c == 0:
        return base
    return "%s_%s%d" % (base, "p" if c > 0 else "m", abs(c))


class LevelEmitter:
    def __init__(self, mmp: MM.MMProgram, level: MM.Level, li: int, soft_div: bool,
                 soft_mul: bool, soft_cmp: bool = True, march_chunk: int = 0,
                 march_pair: int = 0):
        self.mmp, self.level, self.li = mmp, level, li
        self.soft_div, self.soft_mul, self.soft_cmp = soft_div, soft_mul, soft_cmp
        self.march_chunk, self.march_pair = march_chunk, march_pair
        self.shape = mmp.shape
        self.dim = mmp.dim

    def idx_expr(self, cursor: Sequence[int], lane: str = "") -> str:
        parts = [_wrap_name(a, c, lane) for a, c in enumerate(cursor)]
        e = "(size_t)%s" % parts[0]
        for a in range(1, self.dim):
            e = "(%s * %d + %s)" % (e, self.shape[a], parts[a])
        return e

    def _emit_ops(self, which, alias: Dict[int, str], w, ind: str, pfx: str = "a",
                  lane: str = "", ext_prep: Optional[Dict[int, str]] = None,
                  load_state=None, load_array=None) -> Dict[int, str]:
        """C statements for the micro ops in `which` (topological order), one
        `const` temporary <pfx><i> each; an op in `alias` is bound to that C
        expression (a value carried from the previous cell, or the other cell
        of the pair) instead.  `lane` selects the axis-1 coordinate variables
        of the cell; `ext_prep` names run-time reciprocals prepared already
        (divisor op -> DivVarS variable); `load_state(name, cursor)`, when
        given, is the C expression of a state read (else the global array at
        the wrapped cursor).  Returns the reciprocals this call can share:
        divisor op -> variable name."""
        L = self.level
        n = lambda i: "%s%d" % (pfx, i)  # noqa: E731
        const_vals: Dict[int, object] = {}
        for i, m in enumerate(L.micro):
            if m.kind == "const":
                const_vals[i] = m.args[0]
        prepared: Dict[int, str] = dict(ext_prep or {})
        for i in which:
            m = L.micro[i]
            if i in alias:
                w(ind + "const %s %s = %s;" % (m.ctype, n(i), alias[i]))
                continue
            t = m.ctype
            name = n(i)
            k = m.kind
            if k == "const":
                const_vals[i] = m.args[0]
                w(ind + "const %s %s = %s;" % (t, name, MM.c_literal(m.args[0], t)))
            elif k == "loadS":
                src = (load_state(m.args[1], m.args[0]) if load_state is not None else
                       "s_%s[%s]" % (m.args[1], self.idx_expr(m.args[0], lane)))
                w(ind + "const %s %s = %s;" % (t, name, src))
            elif k == "loadM":
                arr = self.mmp.arrays[m.args[1]]
                src = (load_array(m.args[1], m.args[0]) if load_array is not None else
                       "r_%s[%s]" % (arr.name, self.idx_expr(m.args[0], lane)))
                w(ind + "const %s %s = %s;" % (t, name, src))
            elif k == "index":
                w(ind + "const %s %s = (%s)%s;" % (t, name, t, _wrap_name(m.args[0], 0, lane)))
            elif k == "uni":
                op, a = m.args
                if op.startswith("external-call/"):
                    f = op.split("/", 1)[1]
                    w(ind + "const %s %s = %s((double)%s);" % (t, name, f, n(a)))
                else:
                    w(ind + "const %s %s = (%s%s);" % (t, name, op, n(a)))
            elif k == "bin":
                op, a, b = m.args
                ta, tb = L.micro[a].ctype, L.micro[b].ctype
                dd = t == "double" and ta == "double" and tb == "double"
                fa = ta == "float" and tb == "double" and b in const_vals and _float_exact(const_vals[b])
                fb = tb == "float" and ta == "double" and a in const_vals and _float_exact(const_vals[a])
                if op in ("+", "-", "*", "/") and t == "float" and (fa or fb):
                    # C evaluates float (op) double in double and rounds to float; with the
                    # constant exactly a float that equals the float operation: a binary64
                    # (53-bit) result of two binary32 (24-bit) operands rounded again to
                    # binary32 is the correctly rounded binary32 result, since 53 >= 2*24 + 2
                    # (S. A. Figueroa, "When is double rounding innocuous?", SIGNUM
                    # Newsletter 30(3), 1995).  Keeps float programs off the FP64 pipe.
                    xa = n(a) if ta == "float" else MM.c_literal(const_vals[a], "float")
                    xb = n(b) if tb == "float" else MM.c_literal(const_vals[b], "float")
                    w(ind + "const float %s = (%s %s %s);" % (name, xa, op, xb))
                elif (t == "float" and ta == "float" and tb == "double" and b in const_vals and
                      _normal_double(const_vals[b]) and
                      ((op == "/" and self.soft_div and const_vals[b] > 0) or
                       (op == "*" and self.soft_mul))):
                    # (float)((double)x op c) with the widening exact, the binary64 operation
                    # correctly rounded and the narrowing to nearest even, all on the
                    # integer pipes (fm_softfp.cuh): the same bits as the promoted C
                    cv = const_vals[b]
                    xd = "fm::soft::f2d_s(%s)" % n(a)
                    k2 = _pow2_exponent(cv)
                    if k2 is not None:
                        e = "fm::soft::scale_pow2(%s, %d)" % (xd, -k2 if op == "/" else k2)
                    elif op == "/":
                        e = "fm::soft::div_const_s(%s, fm::soft::DivConstS%s)" % (xd, div_const_fields(cv))
                    else:
                        e = "fm::soft::mul_const_s(%s, fm::soft::MulConstS%s)" % (xd, mul_const_fields(cv))
                    w(ind + "const float %s = fm::soft::d2f_s(%s);" % (name, e))
                elif (t == "float" and op == "*" and self.soft_mul and tb == "float" and
                      ta == "double" and a in const_vals and _normal_double(const_vals[a])):
                    cv = const_vals[a]
                    w(ind + "const float %s = fm::soft::d2f_s(fm::soft::mul_const_s("
                            "fm::soft::f2d_s(%s), fm::soft::MulConstS%s));"
                      % (name, n(b), mul_const_fields(cv)))
                elif op == "**":
                    w(ind + "const %s %s = pow((double)%s, (double)%s);" % (t, name, n(a), n(b)))
                elif (op == "/" and self.soft_div and dd and b in const_vals and
                      _pow2_exponent(const_vals[b]) is not None):
                    w(ind + "const %s %s = fm::soft::scale_pow2(%s, %d);" %
                      (t, name, n(a), -_pow2_exponent(const_vals[b])))
                elif (op == "/" and self.soft_div and dd and b in const_vals and
                      _normal_double(const_vals[b]) and const_vals[b] > 0):
                    w(ind + "const %s %s = fm::soft::div_const_s(%s, fm::soft::DivConstS%s);" %
                      (t, name, n(a), div_const_fields(const_vals[b])))
                elif op == "/" and self.soft_div and dd and b not in const_vals:
                    if b not in prepared:
                        prepared[b] = "dv" + n(b)
                        w(ind + "const fm::soft::DivVarS %s = fm::soft::prep_div_s(%s);" %
                          (prepared[b], n(b)))
                    w(ind + "const %s %s = fm::soft::div_var_s(%s, %s);" % (t, name, n(a),
                                                                            prepared[b]))
                elif (op == "*" and self.soft_mul and dd and
                      (b in const_vals or a in const_vals) and
                      _pow2_exponent(const_vals[b] if b in const_vals else const_vals[a])
                      is not None):
                    x, c = (a, b) if b in const_vals else (b, a)
                    w(ind + "const %s %s = fm::soft::scale_pow2(%s, %d);" %
                      (t, name, n(x), _pow2_exponent(const_vals[c])))
                elif (op == "*" and self.soft_mul and t == "double" and
                      ((b in const_vals and ta == "double" and _normal_double(const_vals[b])) or
                       (a in const_vals and tb == "double" and _normal_double(const_vals[a])))):
                    x, c = (a, b) if b in const_vals else (b, a)
                    w(ind + "const %s %s = fm::soft::mul_const_s(%s, fm::soft::MulConstS%s);" %
                      (t, name, n(x), mul_const_fields(const_vals[c])))
                elif (op in CMP_SOFT and self.soft_cmp and ta == "double" and tb == "double"):
                    x, y = (b, a) if op in (">", ">=") else (a, b)
                    w(ind + "const %s %s = %s;" % (t, name, CMP_SOFT[op] % (n(x), n(y))))
                else:
                    w(ind + "const %s %s = (%s %s %s);" % (t, name, n(a), op, n(b)))
            elif k == "ite":
                c, a, b = m.args
                w(ind + "const %s %s = (%s ? %s : %s);" % (t, name, n(c), n(a), n(b)))
            elif k == "nary":
                op, xs = m.args
                names = ["(double)%s" % n(x) for x in xs]

                def chain(fn, items):
                    acc = items[-1]
                    for it in reversed(items[:-1]):
                        acc = "%s(%s, %s)" % (fn, it, acc)
                    return acc

                soft = self.soft_cmp and t == "double" and all(
                    L.micro[x].ctype == "double" for x in xs)
                fmax_, fmin_ = ("fm::soft::max_s", "fm::soft::min_s") if soft else ("fmax", "fmin")
                if op == ">?":
                    e = chain(fmax_, names)
                elif op == "<?":
                    e = chain(fmin_, names)
                else:
                    e = "%s(0.0, %s) + %s(0.0, %s)" % (fmin_, chain(fmax_, names), fmax_,
                                                       chain(fmin_, names))
                w(ind + "const %s %s = %s;" % (t, name, e))
            else:
                raise MM.OM.FmrSemanticError("cannot emit %s" % k)
        return prepared

    # -- marching along axis 0, pairs along axis 1 ---------------------------------------
    def _shifted(self, axis: int = 0) -> Dict[int, int]:
        """For each micro op i, the op j whose value at a cell equals op i's
        value at the next cell along `axis` (i itself for values that do not
        depend on the position along that axis), where the level has one."""
        L = self.level
        index = {(m.kind, m.args, m.ctype): i for i, m in enumerate(L.micro)}
        memo: Dict[int, Optional[int]] = {}

        def sh(i: int) -> Optional[int]:
            if i in memo:
                return memo[i]
            m = L.micro[i]
            k, args = m.kind, m.args
            r: Optional[int] = None
            if k in ("const", "imm"):
                r = i
            elif k == "index":
                r = None if args[0] == axis else i
            elif k in ("loadS", "loadM"):
                c = list(args[0])
                c[axis] += 1
                r = index.get((k, (tuple(c), args[1]), m.ctype))
            else:
                ops = MM._Builder._operands(k, args)
                new = [sh(j) for j in ops]
                if all(j is not None for j in new):
                    if k == "uni":
                        a2 = (args[0], new[0])
                    elif k == "bin":
                        a2 = (args[0], new[0], new[1])
                    elif k == "ite":
                        a2 = tuple(new)
                    else:  # nary
                        a2 = (args[0], tuple(new))
                    r = index.get((k, a2, m.ctype))
            memo[i] = r
            return r

        out = {}
        for i in range(len(L.micro)):
            j = sh(i)
            if j is not None and L.micro[i].kind not in ("const", "imm"):
                out[i] = j
        return out

    def _march_plan(self):
        """(ops the loop body needs, carried ops {i: j}): op i is taken from op
        j's value at the previous cell; everything else is computed."""
        L = self.level
        carried_all = self._shifted(0)
        need = set()
        carried = {}
        stack = [a.root for a in L.arrays]
        need.update(stack)
        while stack:
            i = stack.pop()
            if i in carried_all:
                j = carried_all[i]
                carried[i] = j
                if j not in need:
                    need.add(j)
                    stack.append(j)
            else:
                for j in MM._Builder._operands(L.micro[i].kind, L.micro[i].args):
                    if j not in need:
                        need.add(j)
                        stack.append(j)
        return need, carried

    def _pair_plan(self, need_a):
        """Plan of the second cell (axis-1 coordinate + 1) of a thread's pair,
        evaluated after the first: (ops its loop body needs, ops taken from
        the first cell {i: j}, ops carried from its previous cell {i: j}).
        An op whose shifted form the first cell evaluates anyway is taken from
        there; otherwise carried along axis 0 where possible, else computed."""
        L = self.level
        from_a_all = self._shifted(1)
        carried_all = self._shifted(0)
        need = set()
        from_a, carried = {}, {}
        stack = [a.root for a in L.arrays]
        need.update(stack)
        while stack:
            i = stack.pop()
            j = from_a_all.get(i)
            if j is not None and j in need_a:
                from_a[i] = j
            elif i in carried_all:
                j = carried_all[i]
                carried[i] = j
                if j not in need:
                    need.add(j)
                    stack.append(j)
            else:
                for j in MM._Builder._operands(L.micro[i].kind, L.micro[i].args):
                    if j not in need:
                        need.add(j)
                        stack.append(j)
        return need, from_a, carried, from_a_all

    def _wrap_lines(self, w, ind: str, axes, lane: str = "") -> None:
        needed = set()
        for m in self.level.micro:
            if m.kind in ("loadS", "loadM"):
                for a, c in enumerate(m.args[0]):
                    if c and a in axes:
                        needed.add((a, c))
        for a, c in sorted(needed):
            n = self.shape[a]
            v = _wrap_name(a, c, lane)
            x = _wrap_name(a, 0, lane)
            if abs(c) < n:
                if c > 0:
                    w(ind + "const int %s = %s + %d >= %d ? %s + %d : %s + %d;" %
                      (v, x, c, n, x, c - n, x, c))
                else:
                    w(ind + "const int %s = %s - %d < 0 ? %s + %d : %s - %d;" %
                      (v, x, -c, x, n + c, x, -c))
            else:
                w(ind + "const int %s = ((%s + %d) %% %d + %d) %% %d;" % (v, x, c, n, n, n))

    def _march_body(self, need, carried, chunk: int, pair: int):
        """Kernel body: each thread takes one column (a cell of axes 1..d-1), or
        with pair = 2 two columns adjacent along axis 1, and a chunk of `chunk`
        cells along axis 0.  The first cell evaluates every op, the following
        ones take the carried ops from the previous cell; the second column of
        a pair takes the ops it shares with the first from there (same
        operations on the same values: bit-identical)."""
        L = self.level
        ncol = 1
        for n in self.shape[1:]:
            ncol *= n
        s1 = ncol // self.shape[1]  # stride of axis 1
        n0 = self.shape[0]
        nchunk = (n0 + chunk - 1) // chunk
        nitem_col = ncol // pair
        body: List[str] = []
        w = body.append
        if pair == 1:
            w("    const long long col = item %% %dll;" % ncol)
        else:
            w("    const long long colp = item %% %dll;" % nitem_col)
            w("    const long long col = colp / %dll * %dll + colp %% %dll;" % (s1, 2 * s1, s1))
        w("    const int x0 = (int)(item / %dll) * %d;" % (nitem_col, chunk))
        w("    const int x1 = x0 + %d < %d ? x0 + %d : %d;" % (chunk, n0, chunk, n0))
        w("    size_t rest = (size_t)col;")
        for a in reversed(range(1, self.dim)):
            if a == 1:
                w("    const int %s = (int)rest;" % AXVARS[a])
            else:
                w("    const int %s = (int)(rest %% %du); rest /= %du;" % (AXVARS[a], self.shape[a],
                                                                       self.shape[a]))
        self._wrap_lines(w, "    ", set(range(1, self.dim)))
        live_a = sorted(i for i in carried if i in need)
        for i in live_a:
            w("    %s ha%d;" % (L.micro[i].ctype, i))  # value held from the previous cell
        if pair == 2:
            need_b, from_a, carried_b, from_a_all = self._pair_plan(need)
            w("    const int %s = %s + 1;" % (_wrap_name(1, 0, "b"), AXVARS[1]))  # c1 even
            self._wrap_lines(w, "    ", {1}, "b")
            live_b = sorted(i for i in carried_b if i in need_b)
            for i in live_b:
                w("    %s hb%d;" % (L.micro[i].ctype, i))

        def cell(which_a, alias_a, which_b, alias_b_of):
            prep = self._emit_ops(which_a, alias_a, w, "      ")
            for arr in L.arrays:
                w("      w_%s[idx] = a%d;" % (arr.name, arr.root))
            if pair == 2:
                alias_b = alias_b_of()
                ext = {i: prep[j] for i, j in from_a_all.items() if j in prep}
                self._emit_ops(which_b, alias_b, w, "      ", "b", "b", ext)
                for arr in L.arrays:
                    w("      w_%s[idx + %dull] = b%d;" % (arr.name, s1, arr.root))
            for i in live_a:
                w("      ha%d = a%d;" % (i, carried[i]))
            if pair == 2:
                for i in live_b:
                    w("      hb%d = b%d;" % (i, carried_b[i]))

        # first cell of the chunk: every op (the second column takes whatever
        # the first evaluates)
        w("    {")
        w("      const int c0 = x0;")
        w("      const size_t idx = (size_t)c0 * %dull + (size_t)col;" % ncol)
        self._wrap_lines(w, "      ", {0})
        cell(range(len(L.micro)), {}, range(len(L.micro)),
             lambda: {i: "a%d" % j for i, j in from_a_all.items()})
        w("    }")
        # the rest of the chunk
        # A light cell (at most 16 arithmetic operations) is bound by load latency: unrolled
        # by 4, the loads of several cells are in flight together (float heat-3d at 256^3:
        # 273 -> 402 GLUP/s).  Heavier cells are bound by arithmetic and lose occupancy to
        # the unrolled registers (gray-scott-3d: 17.4 -> 13.6), so they keep one cell.
        arith = sum(1 for i in need if i not in carried and
                    L.micro[i].kind in ("bin", "uni", "nary", "ite"))
        if arith <= LIGHT_ARITH:
            w("#pragma unroll 4")
        w("    for (int c0 = x0 + 1; c0 < x1; ++c0) {")
        w("      const size_t idx = (size_t)c0 * %dull + (size_t)col;" % ncol)
        self._wrap_lines(w, "      ", {0})

        def steady_b():
            al = {i: "a%d" % j for i, j in from_a.items()}
            al.update({i: "hb%d" % i for i in live_b})
            return al

        cell(sorted(need), {i: "ha%d" % i for i in live_a},
             sorted(need_b) if pair == 2 else (), steady_b)
        w("    }")
        return body, nitem_col * nchunk

    def _pair_choice(self) -> int:
        """Cells along axis 1 per thread (1 or 2).  A pair needs at least three
        axes (axis 1 is then not the coalesced one) and an even extent of axis
        1; `march_pair` 2 asks for pairs where the shape allows them, 0 and 1
        give one cell.  Pairs are not the default because they measured slower:
        gray-scott-3d at 256^3 ran 15.7 GLUP/s paired (101 registers, 2 CTAs
        per SM) and 17.2 paired at 3 CTAs per SM (80 registers) against 17.4
        unpaired (74 registers); the saved division, two subtractions and two
        loads per pair do not pay for the longer live ranges."""
        if self.dim < 3 or self.shape[1] % 2:
            return 1
        return 2 if self.march_pair == 2 else 1

    def emit(self) -> Tuple[str, List[str], List[int], List[MM.Array]]:
        """Kernel source of the level.  Launch bounds (256 threads, 2 CTAs per SM) cap
        large levels at 128 registers: the generated 3d-mhd-rk4 program at 256^3 ran
        0.170 GLUP/s unbounded (up to 228 registers, 1 CTA per SM), 0.192 with 2 CTAs
        per SM (spilling), 0.172 with 3 and 0.167 with 4."""
        L = self.level
        state_names = sorted({s for s, _ in L.reads_state})
        arr_ids = sorted({a for a, _ in L.reads_arrays})
        stypes = dict(self.mmp.state)
        params = []
        for s in state_names:
            params.append("const %s *__restrict__ s_%s" % (stypes[s], s))
        for a in arr_ids:
            arr = self.mmp.arrays[a]
            params.append("const %s *__restrict__ r_%s" % (arr.ctype, arr.name))
        for arr in L.arrays:
            params.append("%s *__restrict__ w_%s" % (arr.ctype, arr.name))
        ncells = 1
        for n in self.shape:
            ncells *= n
        kname = "fmr_level_%d" % self.li
        # automatic (march_chunk = 0): chunks of up to 16 cells that leave ~150k
        # threads (the generated MHD program at 64^3 ran slower with chunks of 3 and
        # 53k threads than with one cell per thread; at 256^3 chunks of 16 gain 12-14 %)
        if self.march_chunk > 0:
            chunk = min(self.march_chunk, self.shape[0])
        else:
            chunk = min(16, self.shape[0], max(1, ncells // 150000))
        march, pair = False, 1
        if self.dim >= 2:
            need, carried = self._march_plan()
            march = chunk > 1 and any(i in need for i in carried)
            pair = self._pair_choice()
        if march or pair == 2:
            body, nitems = self._march_body(need, carried, chunk if march else 1, pair)
            src = ["__global__ void __launch_bounds__(256, 2) %s(%s) {" % (kname, ", ".join(params)),
                   "  for (long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;"
                   " item < %dll; item += (long long)gridDim.x * blockDim.x) {" % nitems]
            src += body
            src += ["  }", "}", ""]
            return "\n".join(src), state_names, arr_ids, L.arrays
        body: List[str] = []
        w = body.append
        # coordinates
        w("    size_t rest = (size_t)idx;")
        for a in reversed(range(self.dim)):
            if a == 0:
                w("    const int %s = (int)rest;" % AXVARS[a])
            else:
                w("    const int %s = (int)(rest %% %du); rest /= %du;" % (AXVARS[a], self.shape[a],
                                                                       self.shape[a]))
        self._wrap_lines(w, "    ", set(range(self.dim)))
        self._emit_ops(range(len(L.micro)), {}, w, "    ")
        for arr in L.arrays:
            w("    w_%s[idx] = a%d;" % (arr.name, arr.root))
        src = ["__global__ void __launch_bounds__(256, 2) %s(%s) {" % (kname, ", ".join(params)),
               "  for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < %dll;"
               " idx += (long long)gridDim.x * blockDim.x) {" % ncells]
        src += body
        src += ["  }", "}", ""]
        return "\n".join(src), state_names, arr_ids, L.arrays


# ---------------------------------------------------------------------------
# Temporal blocking of single-level programs

LIGHT_ARITH = 16  # arithmetic operations of a light level (bound by loads, not arithmetic)


def arith_ops(level) -> int:
    """Arithmetic operations of one level's cell (binary, unary, n-ary, select)."""
    return sum(1 for mi in level.micro if mi.kind in ("bin", "uni", "nary", "ite"))


def tb_profitable(mmp: MM.MMProgram) -> bool:
    """Whether blocking pays off: the program is binary32 throughout and light
    (at most 24 arithmetic operations per cell and step), so one step per pass
    is bound by memory traffic, which blocking divides by T.  A heavier or
    binary64 step is bound by arithmetic already (binary64 runs on the slow
    FP64 or integer pipes), and T unrolled copies of a heavy step outgrow the
    instruction cache: float gray-scott-3d at 256^3 ran 6 GLUP/s blocked against
    16.4 one step per pass, float heat-3d 476 against 403."""
    if any(t != "float" for _, t in mmp.state):
        return False
    if any(a.ctype != "float" for a in mmp.arrays.values()):
        return False
    return sum(arith_ops(L) for L in mmp.levels) <= 24

TB_SMEM_BUDGET = 200 * 1024  # bytes of shared memory a blocked kernel may take
TB_THREADS = 1024


def tb_eligible(mmp: MM.MMProgram) -> bool:
    """A program can be temporally blocked here when it has 2 or 3 axes and
    every state variable has exactly one store (its next value): then T steps
    are the step's levels applied T times, each (step, level) a stage of the
    blocked kernel's pipeline."""
    if mmp.dim not in (2, 3) or not mmp.levels:
        return False
    stores = [a.store_of for L in mmp.levels for a in L.arrays if a.store_of is not None]
    return sorted(stores) == sorted(n for n, _ in mmp.state)


class TBPlan:
    """Geometry of the blocked kernel over the stages (t, k) = (time step t of
    the pass, level k of the step), stage index g = t * K + k.

    * A ring is one array's recent planes in shared memory: ("in", state) for
      the pass's input state, (g, node) for array `node` produced by stage g
      and read by a later stage (a manifest intermediate of the same step, or
      a store that becomes the state of the next step).  A state read in step
      t is the ring of its store in step t-1 (the input ring when t = 0).
    * lag[g]: stage g evaluates plane i - lag[g] at iteration i; it reads ring
      planes within its x-reach R0 of that plane, all written in earlier
      iterations (lag[g] >= lag[producer] + R0 + 1), so one barrier per
      iteration orders every stage.
    * Margins, from the end backwards: a stage whose arrays are the final
      stores (step T-1) is computed on the interior; a producer on its
      readers' boxes widened by their reach.  m[g][a] along each axis (axis 0:
      planes before and after the chunk), H[a] = the input ring's margin (the
      halo; along the fastest axis rounded up to 16 bytes for TMA).
    * NS[ring] = planes a ring keeps: the span of its readers' planes; the
      input ring keeps PD more (planes brought ahead of their first use).
    * TI, RG = TI + 2 H: the plane tile's interior and region, sized to the
      shared-memory budget; PS = ring plane stride (region padded to 128 B).
    * XC: planes along axis 0 per tile; tma: whether tiles away from the
      periodic boundary load the input planes with TMA."""

    def __init__(self, mmp: MM.MMProgram, T: int, budget: int = TB_SMEM_BUDGET,
                 sms: int = 152, tma: bool = True):
        d = mmp.dim
        self.T, self.dim, self.shape = T, d, list(mmp.shape)
        levels = mmp.levels
        K = len(levels)
        self.K = K
        self.nstage = T * K
        stype = dict(mmp.state)
        size = {"double": 8, "float": 4, "int": 4, "bool": 1}
        level_of = {a.node: k for k, L in enumerate(levels) for a in L.arrays}
        store_of = {a.store_of: (k, a.node) for k, L in enumerate(levels) for a in L.arrays
                    if a.store_of is not None}
        self.elem = {}  # ring -> C type
        # reads[g] = {ring: (reach per axis)} and the ring of each (kind, key) read
        self.reads = []
        self.src = []  # per stage: {("S", name) or ("M", node): ring}
        for g in range(self.nstage):
            t, k = divmod(g, K)
            L = levels[k]
            rmap, reach = {}, {}
            for name, cur in L.reads_state:
                ring = ("in", name) if t == 0 else (g - K + store_of[name][0] - k, store_of[name][1])
                rmap[("S", name)] = ring
                self.elem[ring] = stype[name]
                r = reach.setdefault(ring, [0] * d)
                for a, c in enumerate(cur):
                    r[a] = max(r[a], abs(c))
            for node, cur in L.reads_arrays:
                ring = (t * K + level_of[node], node)
                rmap[("M", node)] = ring
                self.elem[ring] = mmp.arrays[node].ctype
                r = reach.setdefault(ring, [0] * d)
                for a, c in enumerate(cur):
                    r[a] = max(r[a], abs(c))
            self.src.append(rmap)
            self.reads.append(reach)
        # lags, forwards
        lag = [0] * self.nstage
        for g in range(self.nstage):
            lag[g] = max([0] + [(0 if ring[0] == "in" else lag[ring[0]]) + r[0] + 1
                                for ring, r in self.reads[g].items()])
        self.lag = lag
        # margins, backwards
        final = {g for g in range(self.nstage)
                 if g // K == T - 1 and any(a.store_of for a in levels[g % K].arrays)}
        m = [[None] * d for _ in range(self.nstage)]
        for g in final:
            m[g] = [0] * d
        min_in = [0] * d
        for g in reversed(range(self.nstage)):
            if m[g][0] is None:
                m[g] = [0] * d  # an array no later stage reads (not expected)
            for ring, r in self.reads[g].items():
                need = [m[g][a] + r[a] for a in range(d)]
                if ring[0] == "in":
                    min_in = [max(x, y) for x, y in zip(min_in, need)]
                else:
                    p = ring[0]
                    m[p] = [need[a] if m[p][a] is None else max(m[p][a], need[a]) for a in range(d)]
        self.m = m
        self.min_in = min_in
        self.read = sorted({ring[1] for reach in self.reads for ring in reach if ring[0] == "in"})
        self.sizes = {n: size[stype[n]] for n in self.read}
        sz = list(self.sizes.values()) or [8]
        A = max(16 // s for s in sz) if all(s in (4, 8) for s in sz) else 0
        self.tma = bool(tma and d == 3 and A and self.shape[2] % A == 0)
        self.A = A if self.tma else 1
        self.PD = 2  # planes brought ahead of their first use (TMA or cp.async)
        # ring planes kept
        span = {}
        for g in range(self.nstage):
            for ring, r in self.reads[g].items():
                pl = 0 if ring[0] == "in" else lag[ring[0]]
                span[ring] = max(span.get(ring, 0), lag[g] - pl + r[0] + 1)
        # the input rings share one plane count (one slot index and one mbarrier per plane)
        ns_in = max([n for ring, n in span.items() if ring[0] == "in"] or [0]) + self.PD
        self.NS = {ring: (ns_in if ring[0] == "in" else n) for ring, n in span.items()}
        self.rings = sorted(self.NS, key=lambda r: (-1, r[1]) if r[0] == "in" else (r[0], r[1]))
        H = [min_in[0]] + [min_in[a] for a in range(1, d)]
        if self.tma:
            H[2] = -(-H[2] // A) * A
        self.H = H
        bytes_per_pos = sum(size[self.elem[r]] * self.NS[r] for r in self.rings)
        TI = [0] * d
        if d == 3:
            TI[2] = min(self.shape[2], max(8, 64 - 2 * H[2]))
            if self.tma and TI[2] < self.shape[2]:
                TI[2] = max(A, TI[2] // A * A)
            rg2 = TI[2] + 2 * H[2]
            rg1 = budget // max(1, bytes_per_pos * rg2)
            TI[1] = min(self.shape[1], rg1 - 2 * H[1])
            if self.tma:
                TI[1] = min(TI[1], 256 - 2 * H[1])  # a TMA box edge is at most 256
        else:
            TI[1] = min(self.shape[1], budget // max(1, bytes_per_pos) - 2 * H[1], 4096)
        self.ok = all(TI[a] >= 1 for a in range(1, d))
        while True:
            self.TI = TI
            self.RG = [0] + [TI[a] + 2 * H[a] for a in range(1, d)]
            self.plane = 1
            for a in range(1, d):
                self.plane *= self.RG[a]
            self.PS = -(-self.plane // 32) * 32
            self.smem = bytes_per_pos * self.PS
            if not self.ok or self.smem <= budget or TI[1] <= 1:
                break
            TI = list(TI)
            TI[1] -= 1
        self.ok = self.ok and self.smem <= budget
        if self.ok:
            # balanced edges: the same number of tiles along each axis, none of them mostly
            # outside the array (a tile costs its whole region however little of it is written)
            TI = list(TI)
            for a in range(1, d):
                ti = -(-self.shape[a] // -(-self.shape[a] // TI[a]))
                if self.tma and a == 2:
                    ti = -(-ti // A) * A
                TI[a] = min(TI[a], ti)
            self.TI = TI
            self.RG = [0] + [TI[a] + 2 * H[a] for a in range(1, d)]
            self.plane = 1
            for a in range(1, d):
                self.plane *= self.RG[a]
            self.PS = -(-self.plane // 32) * 32
            self.smem = bytes_per_pos * self.PS
        if self.tma and self.ok and (self.RG[1] > 256 or self.RG[2] > 256):
            self.tma = False
        self.NT = [0] + [(self.shape[a] + self.TI[a] - 1) // self.TI[a] if self.ok else 1
                         for a in range(1, d)]
        self.offset = {}
        off = 0
        for r in self.rings:
            self.offset[r] = off
            off += size[self.elem[r]] * self.NS[r] * self.PS
        nyz = 1
        for a in range(1, d):
            nyz *= self.NT[a]
        # the kernel splits the nyz * n0 column-planes into one contiguous run per CTA;
        # XC is the run's length (planes per CTA)
        n0 = self.shape[0]
        self.ntiles = nyz * n0
        self.XC = -(-self.ntiles // sms)
        self.nchunk = -(-n0 // self.XC)
        self.final = sorted(final)


class TBEmitter(LevelEmitter):
    """Kernel ``fmr_level_tb``: T steps of the program per pass over the state.
    A CTA owns a plane tile (axes 1..d-1, region = interior plus the halo of T
    steps) and marches along axis 0 over a chunk of planes.  Every stage (a
    level of one of the T steps) evaluates, at iteration i, its plane
    i - lag on the cells it must provide, reading the rings of the arrays it
    needs (planes written in earlier iterations, so one __syncthreads per
    iteration orders every stage) and writing its own arrays' rings; the
    final step's stores go to the output arrays on the tile's interior.  Each
    cell evaluates a level's operations in the per-step kernel's order on the
    same values, so the results equal T steps of the per-step kernels bit for
    bit (the reference's temporal blocking unrolls the step graph the same
    way, src/Formura/OrthotopeMachine/TemporalBlocking.hs:49-134).

    Input planes: a tile whose region lies inside the array (no periodic
    wrap) receives each input plane by one TMA copy per state array
    (cp.async.bulk.tensor, issued by one thread PD planes ahead, completing on
    the slot's mbarrier; every wait is bounded and a wait that gives up sets
    the error word); tiles at the periodic boundary gather the plane with
    wrapped indices by per-thread cp.async, also PD planes ahead."""

    def __init__(self, mmp, plan: TBPlan, soft_div=True, soft_mul=True, soft_cmp=True):
        super().__init__(mmp, mmp.levels[0], 0, soft_div, soft_mul, soft_cmp)
        self.plan = plan

    def emit(self) -> Tuple[str, List[str], List[MM.Array]]:
        P = self.plan
        d, T, K, RG, TI, H = P.dim, P.T, P.K, P.RG, P.TI, P.H
        stypes = dict(self.mmp.state)
        state_names = list(P.read)
        outputs = [a for g in P.final for a in self.mmp.levels[g % K].arrays if a.store_of]
        params = ["const %s *__restrict__ s_%s" % (stypes[n], n) for n in state_names]
        params += ["%s *__restrict__ w_%s" % (a.ctype, a.name) for a in outputs]
        params += ["FMR_TMAP tm_%s" % n for n in state_names]
        params += ["int use_tma", "int *__restrict__ fmr_err"]
        plane, PS = P.plane, P.PS
        NS0 = P.NS[("in", state_names[0])] if state_names else 1
        out: List[str] = []
        w = out.append
        n0 = self.shape[0]
        i0 = "(x0 - %d)" % H[0]  # relative plane index k = i - i0
        w("#ifdef FMR_HOST_BUILD")
        w("static unsigned char fmr_tb_smem[%d];" % max(16, P.smem))
        w("#endif")
        w("__global__ void __launch_bounds__(%d, 1) fmr_level_tb(%s) {" % (TB_THREADS, ", ".join(params)))
        w("#ifndef FMR_HOST_BUILD")
        w("  extern __shared__ __align__(128) unsigned char fmr_tb_smem[];")
        w("  __shared__ __align__(8) uint64_t fmr_bar[%d];" % max(1, NS0))
        w("  __shared__ int fmr_fail;")
        w("#endif")
        rname = {}
        for r in P.rings:
            nm = "m_%s" % r[1] if r[0] == "in" else "m%d_%d" % (r[0], r[1])
            rname[r] = nm
            w("  %s *const %s = (%s *)(fmr_tb_smem + %d);  // ring of %d planes"
              % (P.elem[r], nm, P.elem[r], P.offset[r], P.NS[r]))
        tx_bytes = sum(P.sizes[n] for n in state_names) * plane
        w("#ifdef FMR_HOST_BUILD")
        w("  const int fmr_tx = threadIdx.x % 64, fmr_ty = threadIdx.x / 64;")
        w("  const int fmr_cs = blockDim.x < 64 ? blockDim.x : 64;")
        w("  const int fmr_rs = blockDim.x < 64 ? 1 : blockDim.x / 64;")
        w("#else  // the launch's block: %d threads, 64 along the fastest axis" % TB_THREADS)
        w("  const int fmr_tx = threadIdx.x & 63, fmr_ty = threadIdx.x >> 6;")
        w("  constexpr int fmr_cs = 64, fmr_rs = %d;" % (TB_THREADS // 64))
        w("  if (threadIdx.x == 0) fmr_fail = 0;")
        w("#endif")
        # The nyz * n0 column-planes are split into gridDim.x contiguous runs; a CTA marches
        # its run, refilling the pipeline only where the run crosses into the next column.
        w("  const long long fmr_total = %dll;" % P.ntiles)
        w("  int fmr_q = (int)(fmr_total * blockIdx.x / gridDim.x);")
        w("  const int fmr_qend = (int)(fmr_total * (blockIdx.x + 1) / gridDim.x);")
        w("  while (fmr_q < fmr_qend) {")
        w("    int rest = fmr_q / %d;  // the (y, z) column" % n0)
        w("    const int x0 = fmr_q - rest * %d;" % n0)
        w("    const int x1 = x0 + (fmr_qend - fmr_q) < %d ? x0 + (fmr_qend - fmr_q) : %d;" % (n0, n0))
        w("    fmr_q += x1 - x0;")
        for a in reversed(range(1, d)):
            w("    const int o%d = (rest %% %d) * %d - %d;  // region origin along axis %d"
              % (a, P.NT[a], TI[a], H[a], a))
            w("    rest /= %d;" % P.NT[a])
        w("    const int kend = x1 + %d - %s;  // input planes: k in [0, kend)" % (H[0], i0))
        gx_of = lambda kk: "(((x0 - %d + (%s)) %% %d) + %d) %% %d" % (H[0], kk, n0, n0, n0)

        nq = -(-plane // TB_THREADS)  # gathered cells per thread and plane (device build)
        pstride = 1
        for a in range(1, d):
            pstride *= self.shape[a]
        w("#ifndef FMR_HOST_BUILD")
        w("    // in-plane offsets of this thread's gathered cells (wrapped), fixed for the piece")
        w("    int fmr_go[%d];" % nq)
        w("#pragma unroll")
        w("    for (int r = 0; r < %d; ++r) {" % nq)
        w("      const int q = threadIdx.x + r * %d;" % TB_THREADS)
        if d == 3:
            w("      const int j1 = q / %d, j2 = q %% %d;" % (RG[2], RG[2]))
        else:
            w("      const int j1 = q;")
        go = "0"
        for a in range(1, d):
            w("      const int g%d = (((o%d + j%d) %% %d) + %d) %% %d;" %
              (a, a, a, self.shape[a], self.shape[a], self.shape[a]))
            go = "(%s * %d + g%d)" % (go, self.shape[a], a)
        w("      fmr_go[r] = %s;" % go)
        w("    }")
        w("#endif")

        def gather(kk: str, ind: str, asynchronous: bool):
            """Input plane kk (relative) of every state into its slot, wrapped."""
            w(ind + "{")
            w(ind + "  const int gx = %s;" % gx_of(kk))
            w(ind + "  const int sl = (%s) %% %d;" % (kk, NS0))
            if asynchronous:  # device build: the offsets computed for the piece
                w(ind + "  const size_t gb = (size_t)gx * %d;" % pstride)
                w("#pragma unroll")
                w(ind + "  for (int r = 0; r < %d; ++r) {" % nq)
                w(ind + "    const int q = threadIdx.x + r * %d;" % TB_THREADS)
                w(ind + "    if (r + 1 < %d || q < %d) {  // only the last round can run past the plane"
                  % (nq, plane))
                for n in state_names:
                    w(ind + "      fmr_cp_async%d(%s + sl * %d + q, s_%s + gb + fmr_go[r]);" %
                      (P.sizes[n], rname[("in", n)], PS, n))
                w(ind + "    }")
                w(ind + "  }")
                w(ind + "}")
                return
            w(ind + "  for (int q = threadIdx.x; q < %d; q += blockDim.x) {" % plane)
            if d == 3:
                w(ind + "    const int j1 = q / %d, j2 = q %% %d;" % (RG[2], RG[2]))
            else:
                w(ind + "    const int j1 = q;")
            gi = "(size_t)gx"
            for a in range(1, d):
                w(ind + "    const int g%d = (((o%d + j%d) %% %d) + %d) %% %d;" %
                  (a, a, a, self.shape[a], self.shape[a], self.shape[a]))
                gi = "(%s * %d + g%d)" % (gi, self.shape[a], a)
            for n in state_names:
                if asynchronous:
                    w(ind + "    fmr_cp_async%d(%s + sl * %d + q, s_%s + %s);" %
                      (P.sizes[n], rname[("in", n)], PS, n, gi))
                else:
                    w(ind + "    %s[sl * %d + q] = s_%s[%s];" % (rname[("in", n)], PS, n, gi))
            w(ind + "  }")
            w(ind + "}")

        w("#ifndef FMR_HOST_BUILD")
        if P.tma:
            conds = " && ".join("o%d >= 0 && o%d + %d <= %d" % (a, a, RG[a], self.shape[a])
                                for a in range(1, d))
            w("    const bool tma = use_tma && %s;" % conds)
            w("    if (tma) {")
            w("      if (threadIdx.x == 0) {")
            w("        for (int b = 0; b < %d; ++b) fm::tc::mbar_init(&fmr_bar[b], 1);" % NS0)
            w('        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");')
            w("        fm::tc::fence_proxy_async_smem();")
            w("      }")
            w("      __syncthreads();")
            w("      if (threadIdx.x == 0)")
            w("        for (int k = 0; k < %d && k < kend; ++k) fmr_tb_issue(k);" % P.PD)
            w("    } else {")
        else:
            w("    const bool tma = false;")
            w("    {")
        w("      for (int kk = 0; kk < %d; ++kk) {  // cp.async of the first planes, one group each"
          % P.PD)
        w("        if (kk < kend)")
        gather("kk", "        ", True)
        w("        fmr_cp_async_commit();")
        w("      }")
        w("    }")
        w("#endif")
        last = max(P.lag[g] for g in P.final)
        w("    for (int i = x0 - %d; i < x1 + %d; ++i) {" % (H[0], last))
        w("      const int k = i - %s;" % i0)
        w("#ifdef FMR_HOST_BUILD")
        w("      if (k < kend)")
        gather("k", "      ", False)
        w("#else")
        w("      if (tma) {")
        if P.tma:
            w("        if (threadIdx.x == 0 && k + %d < kend) fmr_tb_issue(k + %d);" % (P.PD, P.PD))
            w("        // the first reader of input plane k - 1 runs in this iteration: wait for it")
            w("        if (k >= 1 && k - 1 < kend && !fmr_fail &&")
            w("            !fm::tc::mbar_wait(&fmr_bar[(k - 1) %% %d], ((k - 1) / %d) & 1)) {"
              % (NS0, NS0))
            w("          fmr_fail = 1;")
            w("          atomicExch(fmr_err, 1);")
            w("        }")
        w("      } else {")
        w("        if (k + %d < kend)" % P.PD)
        gather("k + %d" % P.PD, "        ", True)
        w("        fmr_cp_async_commit();")
        w("      }")
        w("#endif")

        def pidx(js):
            return "(%s) * %d + (%s)" % (js[1], RG[2], js[2]) if d == 3 else js[1]

        for g in range(P.nstage):
            t, kl = divmod(g, K)
            L = self.mmp.levels[kl]
            self.level = L
            lo = [0] + [H[a] - P.m[g][a] for a in range(1, d)]
            hi = [0] + [H[a] + TI[a] + P.m[g][a] for a in range(1, d)]
            xs = H[0] - P.m[g][0]
            w("      {  // stage %d: step %d, level %d: plane i - %d" % (g, t, kl, P.lag[g]))
            w("        const int kq = k - %d;  // its relative plane index" % P.lag[g])
            w("        if (kq >= %d && kq < kend - %d) {" % (xs, xs))
            w("          const int p = i - %d;" % P.lag[g])
            slots = {}
            for ring, r in P.reads[g].items():
                for c0 in range(-r[0], r[0] + 1):
                    v = "sl%d_%s%d" % (len(slots), "m" if c0 < 0 else "p", abs(c0))
                    slots[(ring, c0)] = v
                    w("          const int %s = (kq %+d) %% %d;" % (v, c0, P.NS[ring]))
            own = [a for a in L.arrays if (g, a.node) in P.NS]
            if own:
                w("          const int so = kq %% %d;" % min(P.NS[(g, a.node)] for a in own))
                ns_own = {a.node: P.NS[(g, a.node)] for a in own}
                for a in own:
                    w("          const int so_%d = kq %% %d;" % (a.node, ns_own[a.node]))
            has_index = {mi.args[0] for mi in L.micro if mi.kind == "index"}
            if 0 in has_index:
                w("          const int c0 = ((p %% %d) + %d) %% %d;" % (n0, n0, n0))
            if d == 3 and RG[2] <= 64:
                w("#ifdef FMR_HOST_BUILD")
                w("          for (int j1 = %d + fmr_ty; j1 < %d; j1 += fmr_rs)" % (lo[1], hi[1]))
                w("          for (int j2 = %d + fmr_tx; j2 < %d; j2 += fmr_cs) {" % (lo[2], hi[2]))
                w("#else  // at most 64 columns: one per thread")
                if arith_ops(L) <= LIGHT_ARITH:
                    w("#pragma unroll  // a light cell: the loads of its rows in flight together")
                else:
                    w("#pragma unroll 1  // a heavy cell: one copy of its code")
                w("          for (int fmr_r = 0; fmr_r < %d; ++fmr_r)"
                  % -(-(hi[1] - lo[1]) // (TB_THREADS // 64)))
                w("          if (const int j1 = %d + fmr_ty + %d * fmr_r, j2 = %d + fmr_tx;"
                  % (lo[1], TB_THREADS // 64, lo[2]))
                w("              j1 < %d && j2 < %d) {" % (hi[1], hi[2]))
                w("#endif")
            else:
                cnt = 1
                for a in range(1, d):
                    cnt *= hi[a] - lo[a]
                w("          for (int q = threadIdx.x; q < %d; q += blockDim.x) {" % cnt)
                if d == 3:
                    w("            const int j1 = %d + q / %d, j2 = %d + q %% %d;" %
                      (lo[1], hi[2] - lo[2], lo[2], hi[2] - lo[2]))
                else:
                    w("            const int j1 = %d + q;" % lo[1])
            for a in range(1, d):
                if a in has_index:
                    w("            const int c%d = (((o%d + j%d) %% %d) + %d) %% %d;" %
                      (a, a, a, self.shape[a], self.shape[a], self.shape[a]))

            def ring_load(ring, cur, _sl=slots):
                js = [None] + ["j%d%s" % (a, "" if cur[a] == 0 else "%+d" % cur[a])
                               for a in range(1, d)]
                return "%s[%s * %d + %s]" % (rname[ring], _sl[(ring, cur[0])], PS, pidx(js))

            src = P.src[g]
            self._emit_ops(range(len(L.micro)), {}, w, "            ",
                           load_state=lambda name, cur, _s=src: ring_load(_s[("S", name)], cur),
                           load_array=lambda node, cur, _s=src: ring_load(_s[("M", node)], cur))
            for a in own:
                w("            %s[so_%d * %d + %s] = a%d;" %
                  (rname[(g, a.node)], a.node, PS, pidx([None, "j1", "j2"]), a.root))
            if g in P.final:
                # the tile's interior only: the stage's box is wider when a later stage of the
                # same step reads its other arrays
                conds = ["p >= x0", "p < x1"]
                gidx = "(size_t)p"
                for a in range(1, d):
                    if P.m[g][a]:
                        conds.append("j%d >= %d && j%d < %d" % (a, H[a], a, H[a] + TI[a]))
                    conds.append("o%d + j%d < %d" % (a, a, self.shape[a]))
                    gidx = "(%s * %d + (o%d + j%d))" % (gidx, self.shape[a], a, a)
                stores = [a for a in L.arrays if a.store_of]
                if stores:
                    w("            if (%s) {" % " && ".join(conds))
                    w("              const size_t gi = %s;" % gidx)
                    for a in stores:
                        w("              w_%s[gi] = a%d;" % (a.name, a.root))
                    w("            }")
            w("          }")
            w("        }")
            w("      }")
        w("#ifndef FMR_HOST_BUILD")
        w("      // the gathered plane k has landed (at most the %d newest groups pending)" % P.PD)
        w("      if (!tma) fmr_cp_async_wait<%d>();" % P.PD)
        w("#endif")
        w("      __syncthreads();")
        w("    }")
        w("  }")
        w("}")
        w("")
        src = "\n".join(out)
        helpers = ["#ifndef FMR_HOST_BUILD",
                   "__device__ __forceinline__ void fmr_cp_async4(void *dst, const void *src) {",
                   '  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::'
                   ' "r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src) : "memory");',
                   "}",
                   "__device__ __forceinline__ void fmr_cp_async8(void *dst, const void *src) {",
                   '  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::'
                   ' "r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src) : "memory");',
                   "}",
                   "__device__ __forceinline__ void fmr_cp_async_commit() {",
                   '  asm volatile("cp.async.commit_group;" ::: "memory");',
                   "}",
                   "template <int N> __device__ __forceinline__ void fmr_cp_async_wait() {",
                   '  asm volatile("cp.async.wait_group %0;" :: "n"(N) : "memory");',
                   "}",
                   "#endif", ""]
        src = "\n".join(helpers) + src
        if P.tma:
            # the copy of relative input plane k into its slot, one TMA box per state array
            iss = ["#ifndef FMR_HOST_BUILD",
                   "#define fmr_tb_issue(KK) do { \\",
                   "    const int kk_ = (KK); \\",
                   "    const int gx_ = (((x0 - %d + kk_) %% %d) + %d) %% %d; \\"
                   % (H[0], n0, n0, n0),
                   "    uint64_t *bar_ = &fmr_bar[kk_ %% %d]; \\" % NS0,
                   "    fm::tc::mbar_arrive_expect_tx(bar_, %du); \\" % tx_bytes]
            for n in state_names:
                iss.append("    fm::tc::tma_load_3d(%s + (kk_ %% %d) * %d, &tm_%s, o2, o1, gx_, bar_); \\"
                           % (rname[("in", n)], NS0, PS, n))
            iss += ["  } while (0)", "#endif", ""]
            src = "\n".join(iss) + src
        return src, state_names, outputs


def emit_tb_kernel(mmp: MM.MMProgram, T: int, soft_div: bool = True, soft_mul: bool = True,
                   soft_cmp: bool = True, budget: int = TB_SMEM_BUDGET, tma: bool = True):
    """(source, plan, state names read, arrays written) of the blocked kernel
    ``fmr_level_tb`` (T steps per pass), or None when the program is not
    eligible (`tb_eligible`) or its halo leaves no room in shared memory."""
    if T < 2 or not tb_eligible(mmp):
        return None
    plan = TBPlan(mmp, T, budget, tma=tma)
    if not plan.ok or not plan.read:
        return None
    src, sn, aw = TBEmitter(mmp, plan, soft_div, soft_mul, soft_cmp).emit()
    return src, plan, sn, aw


def emit_kernels(mmp: MM.MMProgram, soft_div: bool = True, soft_mul: bool = True,
                 soft_cmp: bool = True, march_chunk: int = 0, march_pair: int = 0):
    """Kernel source and, per level, (kernel name, state names read, arrays
    read, arrays written).  A thread evaluates a chunk of cells along axis 0
    and carries the values a cell shares with the next one: march_chunk cells
    (1: one cell per thread), or with 0 up to 16 while ~150k threads remain.
    march_pair 2 gives a thread two cells along axis 1 that share values
    (where the shape allows it), 0 or 1 one cell (`LevelEmitter._pair_choice`)."""
    parts = []
    levels = []
    for li, L in enumerate(mmp.levels):
        src, sn, ar, aw = LevelEmitter(mmp, L, li, soft_div, soft_mul, soft_cmp,
                                       march_chunk, march_pair).emit()
        parts.append(src)
        levels.append(("fmr_level_%d" % li, sn, ar, aw))
    return "\n".join(parts), levels
