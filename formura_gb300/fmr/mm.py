"""Manifestation: from the orthotope-machine graph to per-array cell programs.

Follows src/Formura/OrthotopeMachine/Manifestation.hs.  Every node marked
manifest (``manifest ::`` declarations and the ``store`` of each state
variable) becomes an array of the grid's shape; its cell program is its
expression with every non-manifest node inlined (recomputed) and every
``shift`` folded into a cursor — the integer offset at which a manifest
array or a state array is read.  ``load`` becomes a read of the state array
at the cursor, a manifest node a read of its array at the cursor, ``index``
the cell's own coordinate (the cursor is not applied to it, as in
Manifestation.hs:131).  Within one cell program a (cursor, node) pair is
computed once.

Two GPU-side decisions are made here:

* **levels**: manifest arrays that do not read each other are computed by one
  kernel (a level); a cell program shared by several arrays of one level is
  evaluated once per cell.  Values are unchanged (each IEEE operation gets
  the same operands).
* **constants**: sub-expressions that read no array and no coordinate are
  evaluated once on the host with the C semantics of the generated code
  (``double`` arithmetic for literals, libm ``pow``/``fmax``/``fmin`` and
  extern functions), so that the device code holds them as exact literals.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import om as OM
from .parser import COMPARISON_OPS

C_TYPES = {"Rational": "double", "double": "double", "float": "float", "real": "double",
           "Real": "double", "int": "int", "bool": "bool", "void": "void"}


@dataclasses.dataclass
class Micro:
    kind: str      # imm const loadS loadM index uni bin ite nary
    args: tuple
    ctype: str     # C type of the temporary


@dataclasses.dataclass
class Array:
    """A manifest array: a state variable's next value or a manifest node."""
    node: int
    name: str
    ctype: str
    store_of: Optional[str]  # state variable this array becomes (store nodes)
    root: int = -1           # micro node holding its value


@dataclasses.dataclass
class Level:
    arrays: List[Array]
    micro: List[Micro]
    reads_state: List[Tuple[str, Tuple[int, ...]]]
    reads_arrays: List[Tuple[int, Tuple[int, ...]]]


@dataclasses.dataclass
class MMProgram:
    dim: int
    axes: List[str]
    shape: List[int]
    state: List[Tuple[str, str]]  # name, C element type
    levels: List[Level]
    arrays: Dict[int, Array]


# ---------------------------------------------------------------------------
# constants with C semantics

def _to_ctype(v, ctype: str):
    if ctype == "float":
        return np.float32(v)
    if ctype == "double":
        return float(v)
    if ctype == "int":
        return int(v)
    if ctype == "bool":
        return bool(v)
    raise OM.FmrSemanticError("unsupported constant type %s" % ctype)


def _promote(a, b):
    """C usual arithmetic conversions between two constant operands."""
    if isinstance(a, float) or isinstance(b, float):
        return float(a), float(b)
    if isinstance(a, np.float32) or isinstance(b, np.float32):
        return np.float32(a), np.float32(b)
    return a, b


def _c_fmax(a: float, b: float) -> float:
    if math.isnan(a):
        return b
    if math.isnan(b):
        return a
    return a if a >= b else b


def _c_fmin(a: float, b: float) -> float:
    if math.isnan(a):
        return b
    if math.isnan(b):
        return a
    return a if a <= b else b


def _fold_chain(fn, xs):
    acc = xs[-1]
    for x in reversed(xs[:-1]):
        acc = fn(x, acc)
    return acc


EXTERN_FNS = {"exp": math.exp, "log": math.log, "sqrt": math.sqrt, "sin": math.sin,
              "cos": math.cos, "tan": math.tan, "fabs": math.fabs, "tanh": math.tanh,
              "atan": math.atan, "cbrt": lambda x: math.copysign(abs(x) ** (1.0 / 3.0), x)}


def eval_const(kind: str, args: tuple, vals: List, ctype: str):
    """Value of one constant micro node from its operands' values."""
    if kind == "imm":
        return _to_ctype(float(args[0]), ctype)
    if kind == "uni":
        op = args[0]
        a = vals[0]
        if op == "-":
            return _to_ctype(-a, ctype)
        if op == "+":
            return _to_ctype(a, ctype)
        if op.startswith("external-call/"):
            f = op.split("/", 1)[1]
            if f not in EXTERN_FNS:
                raise OM.FmrSemanticError("unknown extern function %s" % f)
            return _to_ctype(EXTERN_FNS[f](float(a)), ctype)
        raise OM.FmrSemanticError("unknown unary operator %s" % op)
    if kind == "bin":
        op = args[0]
        a, b = _promote(vals[0], vals[1])
        with np.errstate(all="ignore"):
            if op == "+":
                r = a + b
            elif op == "-":
                r = a - b
            elif op == "*":
                r = a * b
            elif op == "/":
                if b == 0:
                    r = math.copysign(math.inf, a) * math.copysign(1.0, b) if a != 0 else math.nan
                else:
                    r = a / b
            elif op == "**":
                r = math.pow(float(a), float(b))
            elif op in COMPARISON_OPS:
                r = {"<": a < b, "<=": a <= b, ">": a > b, ">=": a >= b, "==": a == b,
                     "!=": a != b}[op]
            else:
                raise OM.FmrSemanticError("unknown binary operator %s" % op)
        return _to_ctype(r, ctype)
    if kind == "ite":
        c, a, b = vals
        a, b = _promote(a, b)
        return _to_ctype(a if c else b, ctype)
    if kind == "nary":
        op = args[0]
        xs = [float(v) for v in vals]
        if op == ">?":
            r = _fold_chain(_c_fmax, xs)
        elif op == "<?":
            r = _fold_chain(_c_fmin, xs)
        elif op == "<%":
            r = _c_fmin(0.0, _fold_chain(_c_fmax, xs)) + _c_fmax(0.0, _fold_chain(_c_fmin, xs))
        else:
            raise OM.FmrSemanticError("unknown n-ary operator %s" % op)
        return _to_ctype(r, ctype)
    raise OM.FmrSemanticError("cannot fold %s" % kind)


def c_literal(v, ctype: str) -> str:
    """An exact C literal of a constant."""
    if ctype == "bool":
        return "true" if v else "false"
    if ctype == "int":
        return "%d" % int(v)
    x = float(v)
    if math.isnan(x):
        return "(0.0/0.0)" if ctype == "double" else "(0.0f/0.0f)"
    if math.isinf(x):
        s = "-" if x < 0 else ""
        return "(%s1.0/0.0)" % s if ctype == "double" else "(%s1.0f/0.0f)" % s
    lit = float(x).hex()
    return lit if ctype == "double" else "%sf" % lit


# ---------------------------------------------------------------------------
# manifestation

def _ctype_of(t: OM.NodeType) -> str:
    e = OM.elem_of(t)
    if e not in C_TYPES:
        raise OM.FmrSemanticError("element type %s has no C type" % e)
    return C_TYPES[e]


class _Builder:
    def __init__(self, g: OM.Graph, manifest: Dict[int, Array], fold: bool):
        self.g = g
        self.manifest = manifest
        self.fold = fold
        self.micro: List[Micro] = []
        self.memo: Dict[Tuple[Tuple[int, ...], int], int] = {}
        self.const_vals: Dict[int, object] = {}
        self.structural: Dict[tuple, int] = {}

    def add(self, key, kind, args, ctype) -> int:
        if key in self.memo:
            return self.memo[key]
        operand_ids = self._operands(kind, args)
        if self.fold and (kind == "imm" or (kind in ("uni", "bin", "ite", "nary") and operand_ids
                                            and all(i in self.const_vals for i in operand_ids))):
            # constant folding: a host-evaluated literal (exact, C semantics)
            val = eval_const(kind, args, [self.const_vals[i] for i in operand_ids], ctype)
            skey = ("const", repr(val), type(val).__name__, ctype)
            kind, args = "const", (val,)
        else:
            val = None
            skey = (kind, args, ctype)
        # the same operation on the same operands has the same value: share it
        idx = self.structural.get(skey)
        if idx is None:
            self.micro.append(Micro(kind, args, ctype))
            idx = len(self.micro) - 1
            self.structural[skey] = idx
            if kind == "const":
                self.const_vals[idx] = val
        self.memo[key] = idx
        return idx

    @staticmethod
    def _operands(kind, args) -> List[int]:
        if kind == "uni":
            return [args[1]]
        if kind == "bin":
            return [args[1], args[2]]
        if kind == "ite":
            return list(args)
        if kind == "nary":
            return list(args[1])
        return []

    def at(self, cursor, nid: int) -> int:
        if nid in self.manifest:
            a = self.manifest[nid]
            return self.add((cursor, nid), "loadM", (cursor, nid), a.ctype)
        return self.delayed(cursor, nid)

    def delayed(self, cursor, nid: int) -> int:
        key = (cursor, nid)
        if key in self.memo:
            return self.memo[key]
        n = self.g.nodes[nid]
        ct = _ctype_of(n.type) if n.kind != "store" else None
        k = n.kind
        if k == "imm":
            return self.add(key, "imm", n.args, ct)
        if k == "uni":
            a = self.at(cursor, n.args[1])
            return self.add(key, "uni", (n.args[0], a), ct)
        if k == "bin":
            a = self.at(cursor, n.args[1])
            b = self.at(cursor, n.args[2])
            return self.add(key, "bin", (n.args[0], a, b), ct)
        if k == "ite":
            c = self.at(cursor, n.args[0])
            a = self.at(cursor, n.args[1])
            b = self.at(cursor, n.args[2])
            return self.add(key, "ite", (c, a, b), ct)
        if k == "nary":
            xs = tuple(self.at(cursor, x) for x in n.args[1])
            return self.add(key, "nary", (n.args[0], xs), ct)
        if k == "shift":
            c2 = tuple(c + v for c, v in zip(cursor, n.args[0]))
            r = self.at(c2, n.args[1])
            self.memo[key] = r
            return r
        if k == "load":
            return self.add(key, "loadS", (cursor, n.args[0]), ct)
        if k == "index":
            return self.add(key, "index", n.args, ct)
        if k == "store":
            r = self.at(cursor, n.args[1])
            self.memo[key] = r
            return r
        raise OM.FmrSemanticError("manifestation of %s is not implemented" % k)


def _arrays_of(g: OM.Graph) -> Dict[int, Array]:
    arrays: Dict[int, Array] = {}
    for i, n in enumerate(g.nodes):
        if not n.manifest:
            continue
        if n.kind == "store":
            name, src = n.args
            ct = _ctype_of(g.nodes[src].type)
            arrays[i] = Array(i, "st_%s" % name, ct, name)
        else:
            arrays[i] = Array(i, "m%d" % i, _ctype_of(n.type), None)
    return arrays


def _deps(g: OM.Graph, arrays: Dict[int, Array], root: int) -> set:
    """Manifest arrays read by the cell program of `root`."""
    out, seen, stack = set(), set(), [root]
    first = True
    while stack:
        nid = stack.pop()
        if nid in seen:
            continue
        seen.add(nid)
        if nid in arrays and not first:
            out.add(nid)
            continue
        first = False
        n = g.nodes[nid]
        if n.kind in ("uni",):
            stack.append(n.args[1])
        elif n.kind == "bin":
            stack += [n.args[1], n.args[2]]
        elif n.kind == "ite":
            stack += list(n.args)
        elif n.kind == "nary":
            stack += list(n.args[1])
        elif n.kind in ("shift", "store"):
            stack.append(n.args[1])
    return out


def manifest(omp: OM.OMProgram, shape: Sequence[int], graph: str = "step",
             fold_constants: bool = True) -> MMProgram:
    """Manifest the step (or init) graph.  With ``fold_constants`` False the
    literals stay ``imm`` nodes and constant sub-expressions stay operations,
    as in the reference's generated C."""
    g = omp.step if graph == "step" else omp.init
    arrays = _arrays_of(g)
    deps = {a: _deps(g, arrays, a) for a in arrays}
    level_of: Dict[int, int] = {}
    for a in sorted(arrays):
        level_of[a] = 1 + max((level_of[d] for d in deps[a]), default=-1)
    nlev = 1 + max(level_of.values(), default=-1)
    levels: List[Level] = []
    for L in range(nlev):
        members = [arrays[a] for a in sorted(arrays) if level_of[a] == L]
        b = _Builder(g, arrays, fold_constants)
        zero = tuple(0 for _ in range(omp.dim))
        for arr in members:
            arr.root = b.delayed(zero, arr.node)
        rs = sorted({(m.args[1], m.args[0]) for m in b.micro if m.kind == "loadS"})
        ra = sorted({(m.args[1], m.args[0]) for m in b.micro if m.kind == "loadM"})
        levels.append(Level(members, b.micro, rs, ra))
    state = [(name, _ctype_of(t)) for name, t in omp.state]
    return MMProgram(omp.dim, list(omp.axes), list(shape), state, levels, arrays)
