"""Seeded random .fmr programs for the front-end parity tests (test
infrastructure).

A program has two state grids p and q (q optionally float, updated from q
alone so that its type stays float), constants, and a step whose updates are
random expression trees over: neighbour reads at offsets up to +-2 on every
axis, constants, a linear function of the coordinates, + - *, division by a
constant (powers of two included), division by a positive run-time value
(1.5 + e*e), n-ary max/min (>? <?), the limiter (<%), if-then-else on each of
the six comparisons, negation, and optionally a manifest half-offset grid
differenced along the first axis; `extended` adds let-in, a lambda (a
second difference along the first axis) applied to the grids, a second
manifest grid reading the first (a second level) and a tuple binding with
tuple arithmetic.  The updates
are clamped to [-4, 4] with >? and <?, which also maps a NaN to the bound
(C fmax/fmin semantics), so long runs stay finite while every operation form
is exercised.
"""
from __future__ import annotations

import random
from typing import List

IDX = ["i", "j", "k"]
AXES = ["x", "y", "z"]


def random_program(seed: int, dim: int, float_q: bool = False, depth: int = 3,
                   extended: bool = False) -> str:
    rng = random.Random(seed)
    idx = IDX[:dim]
    states = ["p", "q"]

    def ref(s: str) -> str:
        offs = [rng.randint(-2, 2) if rng.random() < 0.6 else 0 for _ in range(dim)]
        return "%s[%s]" % (s, ", ".join(v + ("%+d" % o if o else "") for v, o in zip(idx, offs)))

    def const() -> str:
        return rng.choice(["ca", "cb", "0.5", "2", "0.125", "3.7", "(1/3)", "(-1.25)"])

    def leaf() -> str:
        r = rng.random()
        if extended and r < 0.1:
            return "(d2 %s)" % rng.choice(states)
        if r < 0.7:
            return ref(rng.choice(states))
        if r < 0.9 or "p" not in states:
            return const()
        return "ramp"

    def expr(d: int) -> str:
        if d == 0:
            return leaf()
        r = rng.random()
        sub = lambda: expr(d - 1)  # noqa: E731
        if r < 0.30:
            return "(%s %s %s)" % (sub(), rng.choice("+-*"), sub())
        if r < 0.40:
            return "(%s / %s)" % (sub(), rng.choice(["4", "3", "0.1", "cb", "7.5", "0.25"]))
        if r < 0.50:
            e = sub()
            return "(%s / (1.5 + %s * %s))" % (sub(), e, e)
        if r < 0.60:
            return "(%s %s %s %s %s)" % (sub(), rng.choice([">?", "<?"]), sub(),
                                         rng.choice([">?", "<?"]), sub())
        if r < 0.67:
            return "(%s <%% %s)" % (sub(), sub())
        if r < 0.77:
            return "(if %s %s %s then %s else %s)" % (
                sub(), rng.choice([">", "<", ">=", "<=", "==", "!="]), sub(), sub(), sub())
        if r < (0.82 if extended else 0.85):
            return "(-%s)" % sub()
        if extended and r < 0.86:
            return "(let t = %s in t * t - %s)" % (sub(), sub())
        return "(%s * %s)" % (const(), sub())

    out: List[str] = ["dimension :: %d" % dim, "axes :: %s" % ", ".join(AXES[:dim]), ""]
    out.append("double :: ca = %r, cb = %r" % (round(rng.uniform(-1, 1), 3),
                                              rng.choice([0.5, 0.25, 2.0, 0.1, 3.0])))
    if extended:
        out.append("d2 = fun(a) (a[%s] + a[%s]) - 2 * a" % (
            ", ".join(["i+1"] + idx[1:]), ", ".join(["i-1"] + idx[1:])))
    out += ["", "begin function init() returns (p, q)", "  double [] :: p = 0",
            "  %s [] :: q = 0" % ("float" if float_q else "double"), "end function", "",
            "begin function step(p, q) returns (p_next, q_next)"]
    out.append("  ramp[%s] = %s" % (", ".join(idx), " + ".join(
        "%r * %s" % (round(rng.uniform(-0.02, 0.02), 4), v) for v in idx)))
    flux = ""
    if rng.random() < 0.5:
        rest = ", ".join(idx[1:])
        sep = ", " if rest else ""
        out.append("  manifest :: f")
        out.append("  f[i+1/2%s%s] = %s" % (sep, rest, expr(depth - 1)))
        flux = " + (f[i+1/2%s%s] - f[i-1/2%s%s])" % (sep, rest, sep, rest)
        if extended and rng.random() < 0.6:
            # a second manifest grid reading the first: one more level
            out.append("  manifest :: g")
            out.append("  g = %s + 0.5 * (f[i+1/2%s%s] + f[i-1/2%s%s])" % (
                expr(depth - 2), sep, rest, sep, rest))
            flux += " + 0.1 * (g[%s] - g)" % ", ".join(["i+1"] + idx[1:])
    if extended and rng.random() < 0.5:
        # tuple binding and tuple arithmetic
        out.append("  (u1, u2) = (%s, %s) * 0.5 + (%s, %s)" % (
            expr(depth - 2), expr(depth - 2), expr(depth - 2), expr(depth - 2)))
        flux += " + u1 * 0.5 - u2"
    out.append("  p_next = ((p + 0.01 * (%s%s)) >? -4) <? 4" % (expr(depth), flux))
    if float_q:
        states = ["q"]  # a float update reads float grids only (no promotion to double)
    out.append("  q_next = ((q + 0.01 * (%s)) >? -4) <? 4" % expr(depth))
    out.append("end function")
    return "\n".join(out) + "\n"
