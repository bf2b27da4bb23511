"""Evaluation of a parsed Formura program into an orthotope-machine graph.

Semantics follow src/Formura/OrthotopeMachine/Translate.hs:

* values are graph nodes with a type (an element type, or a grid type with
  a rational offset per axis), functions (closures: a lambda captures the
  bindings visible where it is written) and tuples;
* literals are exact rationals (type ``Rational``), emitted later as the
  correctly rounded double;
* binary operators broadcast over tuples (element-wise, or a scalar against
  every element) and lift over functions (``f + g`` is ``fun(x) f x + g x``);
  ``.`` composes functions; grid operands must have the same offset, and an
  element value combines with a grid into a grid (Translate.hs:150-178);
  the result element type is the larger of the two in
  void < bool < int < Rational < float < double < real (Type.hs:15-41);
* ``a[i+k]`` on a grid with offset o gives offset o - k; its integer part
  becomes a ``shift`` node and the fractional part stays in the type
  (Translate.hs:245-270): ``a[i+1/2]`` of an integer grid is ``a`` shifted
  by +1 (``out[n] = a[n+1]``) at offset 1/2;
* statements bind one at a time (a name is visible to the statements after
  it); ``x[i] = e`` binds the index names to the cell coordinates while ``e``
  is evaluated and applies the inverse shift to the result; a type
  declaration casts (an element value becomes a grid), ``manifest`` marks a
  node to be stored, ``extern function :: f`` makes ``f`` a call of the C
  function ``f`` (Translate.hs:385-469);
* ``init`` and ``step`` are evaluated with every top-level statement in
  scope; ``step``'s arguments become ``load`` nodes of the state arrays and
  its results ``store`` nodes into them (Translate.hs:495-584).

Nodes: ``imm`` (Fraction), ``load`` (state name), ``index`` (axis),
``uni`` (op, a), ``bin`` (op, a, b), ``ite`` (c, a, b), ``nary`` (op, [xs]),
``shift`` (offset vector, a), ``store`` (name, a).
"""
from __future__ import annotations

import dataclasses
import math
from fractions import Fraction
from typing import Callable, Dict, List, Optional, Sequence, Tuple, Union

from . import parser as P

ELEM_ORDER = P.ELEMENT_TYPES


class FmrSemanticError(ValueError):
    pass


# ---------------------------------------------------------------------------
# types

@dataclasses.dataclass(frozen=True)
class Elem:
    name: str


@dataclasses.dataclass(frozen=True)
class Grid:
    offset: Tuple[Fraction, ...]
    elem: str


NodeType = Union[Elem, Grid]


def elem_of(t: NodeType) -> str:
    return t.elem if isinstance(t, Grid) else t.name


def meet_elem(a: str, b: str) -> Optional[str]:
    ia = ELEM_ORDER.index(a) if a in ELEM_ORDER else None
    ib = ELEM_ORDER.index(b) if b in ELEM_ORDER else None
    if ia is None or ib is None:
        return None
    return ELEM_ORDER[max(ia, ib)]


def meet(a: NodeType, b: NodeType) -> Optional[NodeType]:
    if a == b:
        return a
    if isinstance(a, Elem) and isinstance(b, Elem):
        e = meet_elem(a.name, b.name)
        return Elem(e) if e else None
    if isinstance(a, Elem) and isinstance(b, Grid):
        e = meet_elem(a.name, b.elem)
        return Grid(b.offset, e) if e else None
    if isinstance(a, Grid) and isinstance(b, Elem):
        return meet(b, a)
    if a.offset == b.offset:
        e = meet_elem(a.elem, b.elem)
        return Grid(a.offset, e) if e else None
    return None


def with_elem(t: NodeType, e: str) -> NodeType:
    return Grid(t.offset, e) if isinstance(t, Grid) else Elem(e)


# ---------------------------------------------------------------------------
# graph and values

@dataclasses.dataclass
class Node:
    kind: str
    args: tuple
    type: NodeType
    manifest: bool = False
    name: Optional[str] = None  # source name (annotation)


@dataclasses.dataclass(frozen=True)
class NodeV:
    id: int
    type: NodeType


@dataclasses.dataclass(frozen=True)
class FunV:
    fn: Callable[["Value"], "Value"]
    doc: str = "fun"


@dataclasses.dataclass(frozen=True)
class TupleV:
    items: Tuple["Value", ...]


Value = Union[NodeV, FunV, TupleV]


class Graph:
    def __init__(self, dim: int):
        self.dim = dim
        self.nodes: List[Node] = []

    def insert(self, kind: str, args: tuple, typ: NodeType) -> NodeV:
        self.nodes.append(Node(kind, args, typ))
        return NodeV(len(self.nodes) - 1, typ)

    def imm_value(self, v: Value) -> Optional[Fraction]:
        if isinstance(v, NodeV) and self.nodes[v.id].kind == "imm":
            return self.nodes[v.id].args[0]
        return None


# ---------------------------------------------------------------------------
# evaluator

class Evaluator:
    def __init__(self, graph: Graph):
        self.g = graph
        self.dim = graph.dim

    # -- helpers -------------------------------------------------------------
    def zero_offset(self) -> Tuple[Fraction, ...]:
        return tuple(Fraction(0) for _ in range(self.dim))

    def norm_offset(self, offs: Sequence[Fraction]) -> Tuple[Fraction, ...]:
        o = [Fraction(x) for x in offs]
        if not o:
            return self.zero_offset()
        if len(o) < self.dim:
            o += [Fraction(0)] * (self.dim - len(o))
        return tuple(o[: self.dim])

    def to_node_type(self, t: P.TypeE) -> NodeType:
        if isinstance(t, P.ElemT):
            return Elem(t.name)
        if isinstance(t, P.GridT):
            inner = self.to_node_type(t.inner)
            return Grid(self.norm_offset(t.offsets), elem_of(inner))
        raise FmrSemanticError("type %r is not a node type" % (t,))

    def cast(self, t: Union[P.TypeE, NodeType], v: Value) -> Value:
        if isinstance(t, (P.TopT, P.FunT)):
            return v
        if isinstance(t, P.TupleT):
            if not isinstance(v, TupleV) or len(v.items) != len(t.items):
                raise FmrSemanticError("tuple type does not match the value")
            return TupleV(tuple(self.cast(ti, vi) for ti, vi in zip(t.items, v.items)))
        if isinstance(t, (P.ElemT, P.GridT)):
            t = self.to_node_type(t)
        if isinstance(v, TupleV):
            return TupleV(tuple(self.cast(t, x) for x in v.items))
        if not isinstance(v, NodeV):
            raise FmrSemanticError("cannot cast a function to %r" % (t,))
        t0 = v.type
        if t == t0:
            return v
        if isinstance(t, Elem) and isinstance(t0, Elem):
            return v
        if isinstance(t, Grid) and isinstance(t0, Elem):
            return NodeV(v.id, t)
        if isinstance(t, Grid) and isinstance(t0, Grid) and t.offset == t0.offset:
            return v
        raise FmrSemanticError("cannot convert type %r to %r" % (t0, t))

    # -- operators -----------------------------------------------------------
    def unop(self, op: str, a: Value) -> Value:
        if isinstance(a, NodeV):
            return self.g.insert("uni", (op, a.id), a.type)
        if isinstance(a, FunV):
            return FunV(lambda x, a=a: self.unop(op, self.apply(a, x)))
        if isinstance(a, TupleV):
            return TupleV(tuple(self.unop(op, x) for x in a.items))
        raise FmrSemanticError("bad operand of unary %s" % op)

    def binop(self, op: str, a: Value, b: Value) -> Value:
        if op == ".":
            return FunV(lambda x, a=a, b=b: self.apply(a, self.apply(b, x)))
        if isinstance(a, NodeV) and isinstance(b, NodeV):
            ct = meet(a.type, b.type)
            if ct is None:
                raise FmrSemanticError("no common type for %r %s %r" % (a.type, op, b.type))
            rt = with_elem(ct, "bool") if op in P.COMPARISON_OPS else ct
            return self.g.insert("bin", (op, a.id, b.id), rt)
        if isinstance(a, FunV) and isinstance(b, FunV):
            return FunV(lambda x, a=a, b=b: self.binop(op, self.apply(a, x), self.apply(b, x)))
        if isinstance(a, FunV) and isinstance(b, NodeV):
            return FunV(lambda x, a=a, b=b: self.binop(op, self.apply(a, x), b))
        if isinstance(a, NodeV) and isinstance(b, FunV):
            return FunV(lambda x, a=a, b=b: self.binop(op, a, self.apply(b, x)))
        if isinstance(a, TupleV) and isinstance(b, TupleV):
            if len(a.items) != len(b.items):
                raise FmrSemanticError("tuple length mismatch")
            return TupleV(tuple(self.binop(op, x, y) for x, y in zip(a.items, b.items)))
        if isinstance(a, NodeV) and isinstance(b, TupleV):
            return TupleV(tuple(self.binop(op, a, y) for y in b.items))
        if isinstance(a, TupleV) and isinstance(b, NodeV):
            return TupleV(tuple(self.binop(op, x, b) for x in a.items))
        raise FmrSemanticError("unexpected operands of %s" % op)

    def _zip_tuples(self, xs: List[Value]):
        """Element-wise over tuples (all of one length), scalars broadcast."""
        lens = {len(x.items) for x in xs if isinstance(x, TupleV)}
        if not lens:
            return None
        if len(lens) > 1:
            raise FmrSemanticError("tuple length mismatch")
        n = lens.pop()
        return [[x.items[i] if isinstance(x, TupleV) else x for x in xs] for i in range(n)]

    def naryop(self, op: str, xs: List[Value]) -> Value:
        z = self._zip_tuples(xs)
        if z is not None:
            return TupleV(tuple(self.naryop(op, row) for row in z))
        if not all(isinstance(x, NodeV) for x in xs):
            raise FmrSemanticError("operands of %s must be values" % op)
        t = xs[0].type
        for x in xs[1:]:
            t = meet(x.type, t)
            if t is None:
                raise FmrSemanticError("no common type in %s" % op)
        return self.g.insert("nary", (op, tuple(x.id for x in xs)), t)

    def ite(self, c: Value, a: Value, b: Value) -> Value:
        z = self._zip_tuples([c, a, b])
        if z is not None:
            return TupleV(tuple(self.ite(*row) for row in z))
        if not all(isinstance(x, NodeV) for x in (c, a, b)):
            raise FmrSemanticError("if-then-else operands must be values")
        if elem_of(c.type) != "bool":
            raise FmrSemanticError("the condition of if-then-else must be of type bool")
        bt = meet(a.type, b.type)
        rt = meet(c.type, bt) if bt is not None else None
        if rt is None:
            raise FmrSemanticError("type mismatch in if-then-else")
        rt = with_elem(rt, elem_of(bt))
        return self.g.insert("ite", (c.id, a.id, b.id), rt)

    def grid_index(self, entries, v: Value) -> Value:
        if isinstance(v, TupleV):
            return TupleV(tuple(self.grid_index(entries, x) for x in v.items))
        if not isinstance(v, NodeV):
            raise FmrSemanticError("grid index applied to a function")
        if isinstance(v.type, Elem):
            return v
        ks = [k for _, k in entries]
        ks = (ks + [Fraction(0)] * self.dim)[: self.dim]
        new_pos = [o - k for o, k in zip(v.type.offset, ks)]
        ints = [math.floor(p) for p in new_pos]
        new_off = tuple(p - i for p, i in zip(new_pos, ints))
        t1 = Grid(new_off, v.type.elem)
        if all(i == 0 for i in ints):
            return NodeV(v.id, t1)
        return self.g.insert("shift", (tuple(-i for i in ints), v.id), t1)

    def apply(self, f: Value, x: Value) -> Value:
        if isinstance(f, FunV):
            return f.fn(x)
        if isinstance(f, TupleV):
            r = self.g.imm_value(x)
            if r is None:
                raise FmrSemanticError("a tuple applied to a non-constant")
            if r.denominator != 1:
                raise FmrSemanticError("non-integer index of a tuple")
            n = int(r)
            if not 0 <= n < len(f.items):
                raise FmrSemanticError("tuple index out of range")
            return f.items[n]
        raise FmrSemanticError("a value that is not a function is applied to an argument")

    # -- patterns ---------------------------------------------------------------
    def names_of(self, lhs: P.Expr):
        if isinstance(lhs, P.Ident):
            return lhs.name
        if isinstance(lhs, (P.GridIdx, P.VecIdx)):
            return self.names_of(lhs.expr)
        if isinstance(lhs, P.TupleE):
            return tuple(self.names_of(x) for x in lhs.items)
        raise FmrSemanticError("bad left-hand side %r" % (lhs,))

    def match(self, names, v) -> List[Tuple[str, object]]:
        if isinstance(names, tuple):
            items = v.items if isinstance(v, TupleV) else (v.items if isinstance(v, P.TupleT) else None)
            if items is None:
                raise FmrSemanticError("the left-hand side expects a tuple")
            if len(items) != len(names):
                raise FmrSemanticError("tuple length mismatch")
            out = []
            for n, x in zip(names, items):
                out += self.match(n, x)
            return out
        return [(names, v)]

    # -- expressions ---------------------------------------------------------------
    def eval(self, e: P.Expr, env: Dict[str, Value]) -> Value:
        if isinstance(e, P.Num):
            return self.g.insert("imm", (e.value,), Elem("Rational"))
        if isinstance(e, P.Ident):
            if e.name not in env:
                raise FmrSemanticError("undefined variable: %s" % e.name)
            return env[e.name]
        if isinstance(e, P.TupleE):
            return TupleV(tuple(self.eval(x, env) for x in e.items))
        if isinstance(e, P.GridIdx):
            return self.grid_index(e.entries, self.eval(e.expr, env))
        if isinstance(e, P.Apply):
            return self.apply(self.eval(e.f, env), self.eval(e.x, env))
        if isinstance(e, P.Lambda):
            names = self.names_of(e.pattern)
            body = e.body

            def fn(x, names=names, body=body, env=env):
                local = dict(env)
                local.update(self.match(names, x))
                return self.eval(body, local)

            return FunV(fn, "lambda")
        if isinstance(e, P.Let):
            return self.with_bindings(e.stmts, env, lambda env2: self.eval(e.body, env2))
        if isinstance(e, P.Unop):
            return self.unop(e.op, self.eval(e.a, env))
        if isinstance(e, P.Binop):
            return self.binop(e.op, self.eval(e.a, env), self.eval(e.b, env))
        if isinstance(e, P.Nary):
            return self.naryop(e.op, [self.eval(x, env) for x in e.items])
        if isinstance(e, P.If):
            return self.ite(self.eval(e.cond, env), self.eval(e.a, env), self.eval(e.b, env))
        raise FmrSemanticError("cannot evaluate %r" % (e,))

    # -- statements -------------------------------------------------------------------
    def with_bindings(self, stmts: List[P.Stmt], env: Dict[str, Value], cont):
        type_of: Dict[str, P.TypeE] = {}
        mods: Dict[str, List[str]] = {}
        for s in stmts:
            if isinstance(s, P.TypeDecl):
                names = self.names_of(s.lhs)
                flat = self._flatten(names)
                if isinstance(s.type, P.TupleT) and isinstance(names, tuple):
                    for n, t in self.match(names, s.type):
                        type_of[n] = t
                else:
                    for n in flat:
                        if not isinstance(s.type, P.TopT):
                            type_of[n] = s.type
                for n in flat:
                    mods.setdefault(n, []).extend(s.modifiers)
        env = dict(env)
        for n, t in type_of.items():
            if isinstance(t, P.FunT) and "extern" in mods.get(n, []):
                env[n] = FunV(lambda x, f=n: self.unop("external-call/" + f, x), "extern " + n)
        for s in stmts:
            if not isinstance(s, P.Subst):
                continue
            local = dict(env)
            if isinstance(s.lhs, P.GridIdx):
                for ax, (name, _) in enumerate(s.lhs.entries):
                    if name:
                        local[name] = self.g.insert("index", (ax,), Elem("Rational"))
            v0 = self.eval(s.rhs, local)
            if isinstance(s.lhs, P.GridIdx):
                pairs = self.match(self.names_of(s.lhs.expr), v0)
                neg = [(None, -k) for _, k in s.lhs.entries]
                pairs = [(n, self.grid_index(neg, v)) for n, v in pairs]
            else:
                pairs = self.match(self.names_of(s.lhs), v0)
            for name, v in pairs:
                if name in type_of:
                    v = self.cast(type_of[name], v)
                self._annotate(v, name, "manifest" in mods.get(name, []))
                env[name] = v
        return cont(env)

    def _flatten(self, names) -> List[str]:
        if isinstance(names, tuple):
            out = []
            for n in names:
                out += self._flatten(n)
            return out
        return [names]

    def _annotate(self, v: Value, name: str, manifest: bool):
        if isinstance(v, NodeV):
            node = self.g.nodes[v.id]
            if manifest:
                node.manifest = True
                node.name = name
            elif node.name is None:
                node.name = name
        elif isinstance(v, TupleV):
            for x in v.items:
                self._annotate(x, name, manifest)


# ---------------------------------------------------------------------------
# programs

@dataclasses.dataclass
class OMProgram:
    dim: int
    axes: List[str]
    state: List[Tuple[str, NodeType]]  # step's arguments and their types
    init: Graph
    step: Graph


def _global_extents(shape: Sequence[int], axes: Sequence[str]) -> List[P.Stmt]:
    return [P.Subst(P.Ident("N" + a.upper()), P.Num(Fraction(int(n)))) for a, n in zip(axes, shape)]


def _lookup(prog: P.Program, name: str) -> P.Expr:
    found = [s.rhs for s in prog.stmts if isinstance(s, P.Subst) and isinstance(s.lhs, P.Ident)
             and s.lhs.name == name]
    if not found:
        raise FmrSemanticError("identifier `%s` not found" % name)
    if len(found) > 1:
        raise FmrSemanticError("multiple declarations of `%s`" % name)
    return found[0]


def _gen_global_function(prog: P.Program, dim: int, axes, global_shape, fn_name: str,
                         input_types: Optional[List[Tuple[str, NodeType]]],
                         out_pattern: P.Expr) -> Tuple[Graph, Value]:
    g = Graph(dim)
    ev = Evaluator(g)
    stmts = _global_extents(global_shape, axes) + list(prog.stmts)
    lam = _lookup(prog, fn_name)
    if not isinstance(lam, P.Lambda):
        raise FmrSemanticError("`%s` is not a function" % fn_name)

    def body(env):
        local = dict(env)
        if input_types is not None:
            for name, t in input_types:
                local[name] = g.insert("load", (name,), t)
        ret = ev.eval(lam.body, local)
        for name, v in ev.match(ev.names_of(out_pattern), ret):
            if not isinstance(v, NodeV):
                raise FmrSemanticError("the result of a global function must be a tuple of grids")
            st = g.insert("store", (name, v.id), Elem("void"))
            g.nodes[st.id].manifest = True
            g.nodes[st.id].name = name + "_next"
        return ret

    return g, ev.with_bindings(stmts, {}, body)


def _types_of(v: Value) -> List[NodeType]:
    if isinstance(v, NodeV):
        return [v.type]
    if isinstance(v, TupleV):
        out = []
        for x in v.items:
            out += _types_of(x)
        return out
    raise FmrSemanticError("a global function must return grids")


def build_om(prog: P.Program, global_shape: Sequence[int]) -> OMProgram:
    """OM graphs of ``init`` and ``step`` for the given global grid shape
    (the extent constants NX, NY, ... of the program)."""
    if prog.dimension is None:
        raise FmrSemanticError("no dimension declaration found")
    if prog.axes is None:
        raise FmrSemanticError("no axes declaration found")
    if len(prog.axes) != prog.dimension:
        raise FmrSemanticError("number of declared axes does not match the declared dimension")
    dim, axes = prog.dimension, list(prog.axes)
    if len(global_shape) != dim:
        raise FmrSemanticError("grid shape has %d axes, the program %d" % (len(global_shape), dim))
    step = _lookup(prog, "step")
    if not isinstance(step, P.Lambda):
        raise FmrSemanticError("`step` is not a function")
    ev0 = Evaluator(Graph(dim))
    state_names = ev0._flatten(ev0.names_of(step.pattern))
    g_init, ret_init = _gen_global_function(prog, dim, axes, global_shape, "init", None,
                                            step.pattern)
    init_types = _types_of(ret_init)
    if len(init_types) != len(state_names):
        raise FmrSemanticError("init returns %d values, step takes %d" %
                               (len(init_types), len(state_names)))
    state = list(zip(state_names, init_types))
    g_step, ret_step = _gen_global_function(prog, dim, axes, global_shape, "step", state,
                                            step.pattern)
    if _types_of(ret_step) != init_types:
        raise FmrSemanticError("the return type of step %r must match the return type of init %r"
                               % (_types_of(ret_step), init_types))
    return OMProgram(dim, axes, state, g_init, g_step)
