"""Parser of the Formura language (.fmr).

Covers the syntax of src/Formura/Parser.hs: special declarations
(``dimension :: n``, ``axes :: x, y, z``), statements (``lhs = rhs``, type
declarations with modifiers ``const``/``extern``/``manifest``, grid types
``double []``, the function sugar ``begin function f(x) returns y ... end
function`` and ``begin function y = f(x) ... end function``), and
expressions with the operator table of Parser.hs:198-208 — from tightest to
loosest: ``.`` (composition, right-assoc), ``**``, ``* /``, prefix ``+ -``,
binary ``+ -``, the n-ary min/max family ``>? <? <%`` (a chain of one operator
is flattened into one n-ary node), comparisons ``<= == != >= < >`` (non-assoc).
Function application is juxtaposition (``f x``, ``e 0``), tighter than any
operator; ``a[i+1/2, j]`` is a grid index with n+k entries (``a[,i-1]`` leaves
an axis unshifted); ``fun (x) body``, ``let ... in e``, ``if c then a else b``
and tuples ``(a, b)`` (a one-element tuple is a parenthesised expression).

Identifiers are alphabetic (a letter, then letters, digits, ``_`` or ``'``)
or symbolic (a run of printable characters that are neither alphanumeric
nor one of ``"#();[\\]{}``, e.g. ``∂``); a run equal to a keyword or operator
is that keyword.  ``#`` starts a comment, a backslash before a newline
continues the line, newlines and ``;`` end statements.

The tree is plain dataclasses; numbers are exact ``fractions.Fraction``.
"""
from __future__ import annotations

import dataclasses
import unicodedata
from fractions import Fraction
from typing import List, Optional, Tuple, Union

KEYWORDS = {"begin", "end", "function", "returns", "let", "in", "fun", "dimension", "axes",
            "if", "then", "else", "const", "extern", "manifest",
            "+", "-", "*", "/", ".", "**", "::", "=", ","}
MINMAX_OPS = {"<?", ">?", "<%"}
COMPARISON_OPS = {"<=", "==", "!=", ">=", "<", ">"}
KEYWORDS |= MINMAX_OPS | COMPARISON_OPS
ELEMENT_TYPES = ["void", "bool", "int", "Rational", "float", "double", "real", "Real"]


class FmrSyntaxError(ValueError):
    pass


# ---------------------------------------------------------------------------
# syntax tree

@dataclasses.dataclass
class Num:
    value: Fraction


@dataclasses.dataclass
class Ident:
    name: str


@dataclasses.dataclass
class TupleE:
    items: List["Expr"]


@dataclasses.dataclass
class GridIdx:
    """``expr[n+k, ...]``: per axis an optional index name and a rational k."""
    entries: List[Tuple[Optional[str], Fraction]]
    expr: "Expr"


@dataclasses.dataclass
class VecIdx:
    name: str
    expr: "Expr"


@dataclasses.dataclass
class Apply:
    f: "Expr"
    x: "Expr"


@dataclasses.dataclass
class Lambda:
    pattern: "Expr"
    body: "Expr"


@dataclasses.dataclass
class Let:
    stmts: List["Stmt"]
    body: "Expr"


@dataclasses.dataclass
class Unop:
    op: str
    a: "Expr"


@dataclasses.dataclass
class Binop:
    op: str
    a: "Expr"
    b: "Expr"


@dataclasses.dataclass
class Nary:
    op: str
    items: List["Expr"]


@dataclasses.dataclass
class If:
    cond: "Expr"
    a: "Expr"
    b: "Expr"


Expr = Union[Num, Ident, TupleE, GridIdx, VecIdx, Apply, Lambda, Let, Unop, Binop, Nary, If]


@dataclasses.dataclass
class ElemT:
    name: str


@dataclasses.dataclass
class GridT:
    offsets: List[Fraction]  # empty: offset 0 on every axis
    inner: "TypeE"


@dataclasses.dataclass
class FunT:
    pass


@dataclasses.dataclass
class TupleT:
    items: List["TypeE"]


@dataclasses.dataclass
class TopT:
    pass


TypeE = Union[ElemT, GridT, FunT, TupleT, TopT]


@dataclasses.dataclass
class TypeDecl:
    type: TypeE
    modifiers: List[str]
    lhs: Expr


@dataclasses.dataclass
class Subst:
    lhs: Expr
    rhs: Expr


Stmt = Union[TypeDecl, Subst]


@dataclasses.dataclass
class Program:
    dimension: Optional[int]
    axes: Optional[List[str]]
    stmts: List[Stmt]


# ---------------------------------------------------------------------------
# lexer

@dataclasses.dataclass
class Tok:
    kind: str  # NUM ID KW LP RP LB RB NL EOF
    text: str
    line: int
    value: Optional[Fraction] = None


def _is_alpha0(c: str) -> bool:
    return c.isalpha()


def _is_alpha1(c: str) -> bool:
    return c.isalnum() or c in "_'"


def _is_symbol(c: str) -> bool:
    if not c.isprintable() or c.isspace() or _is_alpha1(c):
        return False
    return c not in "\"#();[\\]{}"


def tokenize(src: str) -> List[Tok]:
    toks: List[Tok] = []
    i, n, line = 0, len(src), 1
    while i < n:
        c = src[i]
        if c == "\n":
            toks.append(Tok("NL", "\n", line))
            line += 1
            i += 1
        elif c.isspace():
            i += 1
        elif c == "#":
            while i < n and src[i] != "\n":
                i += 1
        elif c == "\\":
            j = i + 1
            while j < n and src[j] in " \t\r":
                j += 1
            if j < n and src[j] == "\n":
                i = j + 1
                line += 1
            else:
                raise FmrSyntaxError("line %d: stray backslash" % line)
        elif c == ";":
            toks.append(Tok("NL", ";", line))
            i += 1
        elif c in "()[]":
            toks.append(Tok({"(": "LP", ")": "RP", "[": "LB", "]": "RB"}[c], c, line))
            i += 1
        elif c.isdigit():
            j = i
            while j < n and src[j].isdigit():
                j += 1
            if j + 1 < n and src[j] == "." and src[j + 1].isdigit():
                j += 1
                while j < n and src[j].isdigit():
                    j += 1
            if j < n and src[j] in "eE":
                k = j + 1
                if k < n and src[k] in "+-":
                    k += 1
                if k < n and src[k].isdigit():
                    while k < n and src[k].isdigit():
                        k += 1
                    j = k
            text = src[i:j]
            toks.append(Tok("NUM", text, line, Fraction(text)))
            i = j
        elif _is_alpha0(c):
            j = i + 1
            while j < n and _is_alpha1(src[j]):
                j += 1
            text = src[i:j]
            toks.append(Tok("KW" if text in KEYWORDS else "ID", text, line))
            i = j
        elif _is_symbol(c):
            j = i + 1
            while j < n and _is_symbol(src[j]):
                j += 1
            text = src[i:j]
            # a comma never glues to other symbols in practice; split it off
            if "," in text and text != ",":
                parts = []
                cur = ""
                for ch in text:
                    if ch == ",":
                        if cur:
                            parts.append(cur)
                        parts.append(",")
                        cur = ""
                    else:
                        cur += ch
                if cur:
                    parts.append(cur)
                for t in parts:
                    toks.append(Tok("KW" if t in KEYWORDS else "ID", t, line))
            else:
                toks.append(Tok("KW" if text in KEYWORDS else "ID", text, line))
            i = j
        else:
            raise FmrSyntaxError("line %d: unexpected character %r (%s)" %
                                 (line, c, unicodedata.name(c, "?")))
    toks.append(Tok("EOF", "", line))
    return toks


# ---------------------------------------------------------------------------
# parser

class Parser:
    def __init__(self, src: str):
        self.toks = tokenize(src)
        self.i = 0
        self.depth = 0  # bracket nesting: newlines inside brackets are ignored

    # -- token helpers ------------------------------------------------------
    def peek(self, k: int = 0) -> Tok:
        j = self.i
        seen = 0
        while True:
            t = self.toks[j]
            if t.kind == "NL" and self.depth > 0:
                j += 1
                continue
            if seen == k:
                return t
            seen += 1
            j += 1

    def next(self) -> Tok:
        while self.toks[self.i].kind == "NL" and self.depth > 0:
            self.i += 1
        t = self.toks[self.i]
        self.i += 1
        return t

    def at(self, kind: str, text: Optional[str] = None) -> bool:
        t = self.peek()
        return t.kind == kind and (text is None or t.text == text)

    def at_kw(self, text: str) -> bool:
        return self.at("KW", text)

    def expect(self, kind: str, text: Optional[str] = None) -> Tok:
        t = self.next()
        if t.kind != kind or (text is not None and t.text != text):
            raise FmrSyntaxError("line %d: expected %s, found %r" % (t.line, text or kind, t.text))
        return t

    def skip_nl(self):
        while self.toks[self.i].kind == "NL":
            self.i += 1

    def open(self, kind: str):
        self.expect(kind)
        self.depth += 1

    def close(self, kind: str):
        self.depth -= 1
        self.expect(kind)

    # -- program --------------------------------------------------------------
    def program(self) -> Program:
        dim, axes, stmts = None, None, []
        self.skip_nl()
        while not self.at("EOF"):
            if self.at_kw("dimension"):
                self.next()
                self.expect("KW", "::")
                dim = int(self.expect("NUM").value)
            elif self.at_kw("axes"):
                self.next()
                self.expect("KW", "::")
                axes = [self.ident_name()]
                while self.at_kw(","):
                    self.next()
                    axes.append(self.ident_name())
            else:
                stmts.extend(self.statement_compound())
            self.end_statement()
        return Program(dim, axes, stmts)

    def end_statement(self):
        if self.at("EOF"):
            return
        t = self.peek()
        if t.kind != "NL":
            raise FmrSyntaxError("line %d: expected end of statement, found %r" % (t.line, t.text))
        self.skip_nl()

    def ident_name(self) -> str:
        t = self.next()
        if t.kind != "ID":
            raise FmrSyntaxError("line %d: expected an identifier, found %r" % (t.line, t.text))
        return t.text

    # -- statements -------------------------------------------------------------
    def statement_compound(self) -> List[Stmt]:
        if self.at_kw("begin"):
            return self.function_sugar()
        return self.type_value_statements()

    def binding(self, terminator: str) -> List[Stmt]:
        stmts: List[Stmt] = []
        self.skip_nl()
        while not self.at_kw(terminator):
            if self.at("EOF"):
                raise FmrSyntaxError("unexpected end of file: missing %r" % terminator)
            stmts.extend(self.statement_compound())
            if not self.at_kw(terminator):
                self.end_statement()
        return stmts

    def function_sugar(self) -> List[Stmt]:
        self.expect("KW", "begin")
        self.expect("KW", "function")
        # returns-form: name ( args ) returns out ; equal-form: out = name ( args )
        if self.at("ID") and self.peek(1).kind == "LP" and self._returns_form_ahead():
            name = self.ident_name()
            pat = self.tuple_of(self.lexpr)
            self.expect("KW", "returns")
            out = self.rexpr()
        else:
            out = self.rexpr()
            self.expect("KW", "=")
            name = self.ident_name()
            pat = self.tuple_of(self.lexpr)
        self.end_statement()
        body = self.binding("end")
        self.expect("KW", "end")
        self.expect("KW", "function")
        return [Subst(Ident(name), Lambda(pat, Let(body, out)))]

    def _returns_form_ahead(self) -> bool:
        # name ( ... ) returns
        j = self.i
        toks = self.toks
        while toks[j].kind == "NL":
            j += 1
        if toks[j].kind != "ID" or toks[j + 1].kind != "LP":
            return False
        depth, k = 0, j + 1
        while True:
            t = toks[k]
            if t.kind == "LP":
                depth += 1
            elif t.kind == "RP":
                depth -= 1
                if depth == 0:
                    break
            elif t.kind == "EOF":
                return False
            k += 1
        k += 1
        while toks[k].kind == "NL":
            k += 1
        return toks[k].kind == "KW" and toks[k].text == "returns"

    def type_value_statements(self) -> List[Stmt]:
        save, save_depth = self.i, self.depth
        typed = self.try_mod_type()
        if typed is not None and self.at_kw("::"):
            self.next()
            mods, typ = typed
            items = []
            while True:
                lhs = self.lexpr()
                rhs = None
                if self.at_kw("="):
                    self.next()
                    rhs = self.rexpr()
                items.append((lhs, rhs))
                if self.at_kw(","):
                    self.next()
                    continue
                break
            out: List[Stmt] = [TypeDecl(typ, mods, lhs) for lhs, _ in items]
            out += [Subst(lhs, rhs) for lhs, rhs in items if rhs is not None]
            return out
        self.i, self.depth = save, save_depth
        lhs = self.lexpr()
        self.expect("KW", "=")
        rhs = self.rexpr()
        return [Subst(lhs, rhs)]

    def try_mod_type(self):
        """modifiers, an optional type expression, modifiers; None if the
        tokens cannot start one."""
        mods: List[str] = []
        while self.at("KW") and self.peek().text in ("const", "extern", "manifest"):
            mods.append(self.next().text)
        save, save_depth = self.i, self.depth
        typ: TypeE = TopT()
        try:
            t = self.type_fexpr()
            if t is not None:
                typ = t
            else:
                self.i, self.depth = save, save_depth
        except FmrSyntaxError:
            self.i, self.depth = save, save_depth
        while self.at("KW") and self.peek().text in ("const", "extern", "manifest"):
            mods.append(self.next().text)
        return mods, typ

    def type_aexpr(self) -> Optional[TypeE]:
        if self.at("LP"):
            self.open("LP")
            items = []
            if not self.at("RP"):
                while True:
                    t = self.type_fexpr()
                    if t is None:
                        raise FmrSyntaxError("bad type")
                    items.append(t)
                    if self.at_kw(","):
                        self.next()
                        continue
                    break
            self.close("RP")
            return items[0] if len(items) == 1 else TupleT(items)
        if self.at("ID") and self.peek().text in ELEMENT_TYPES:
            return ElemT(self.next().text)
        if self.at_kw("function"):
            self.next()
            return FunT()
        return None

    def type_fexpr(self) -> Optional[TypeE]:
        t = self.type_aexpr()
        if t is None:
            return None
        while True:
            if self.at("LB"):
                self.open("LB")
                offs = []
                if not self.at("RB"):
                    while True:
                        offs.append(self.const_rational())
                        if self.at_kw(","):
                            self.next()
                            continue
                        break
                self.close("RB")
                t = GridT(offs, t)
            else:
                return t

    # -- l-expressions ------------------------------------------------------------
    def lexpr(self) -> Expr:
        if self.at("LP"):
            f = self.tuple_of(self.lexpr)
        else:
            f = Ident(self.ident_name())
        while True:
            if self.at("LB"):
                f = GridIdx(self.grid_indices(), f)
            elif self.at("LP") and self.peek(1).kind == "ID" and self.peek(2).kind == "RP":
                self.open("LP")
                name = self.ident_name()
                self.close("RP")
                f = VecIdx(name, f)
            else:
                return f

    def tuple_of(self, item) -> Expr:
        self.open("LP")
        xs = []
        if not self.at("RP"):
            while True:
                xs.append(item())
                if self.at_kw(","):
                    self.next()
                    continue
                break
        self.close("RP")
        return xs[0] if len(xs) == 1 else TupleE(xs)

    def grid_indices(self) -> List[Tuple[Optional[str], Fraction]]:
        self.open("LB")
        entries = []
        while True:
            name = None
            k = Fraction(0)
            if self.at("ID") and self.peek().text[0].isalpha():
                name = self.next().text
            if self.at_kw("+") or self.at_kw("-"):
                sign = self.next().text
                v = self.const_rational()
                k = v if sign == "+" else -v
            if not (self.at_kw(",") or self.at("RB")):
                t = self.peek()
                raise FmrSyntaxError("line %d: bad grid index near %r" % (t.line, t.text))
            entries.append((name, k))
            if self.at_kw(","):
                self.next()
                continue
            break
        self.close("RB")
        return entries

    # -- r-expressions ------------------------------------------------------------
    def rexpr(self) -> Expr:
        return self.level_cmp(self.fexpr)

    def const_rational(self) -> Fraction:
        e = self.level_cmp(self.num_term)
        return _eval_const(e)

    def num_term(self) -> Expr:
        if self.at("NUM"):
            return Num(self.next().value)
        if self.at("LP"):
            self.open("LP")
            e = self.level_cmp(self.num_term)
            self.close("RP")
            return e
        t = self.peek()
        raise FmrSyntaxError("line %d: expected a number, found %r" % (t.line, t.text))

    def level_cmp(self, term) -> Expr:
        a = self.level_minmax(term)
        if self.at("KW") and self.peek().text in COMPARISON_OPS:
            op = self.next().text
            b = self.level_minmax(term)
            a = Binop(op, a, b)
        return a

    def level_minmax(self, term) -> Expr:
        a = self.level_add(term)
        while self.at("KW") and self.peek().text in MINMAX_OPS:
            op = self.next().text
            b = self.level_add(term)
            ap = a.items if isinstance(a, Nary) and a.op == op else [a]
            bp = b.items if isinstance(b, Nary) and b.op == op else [b]
            a = Nary(op, ap + bp)
        return a

    def level_add(self, term) -> Expr:
        a = self.level_unary(term)
        while self.at_kw("+") or self.at_kw("-"):
            op = self.next().text
            b = self.level_unary(term)
            a = Binop(op, a, b)
        return a

    def level_unary(self, term) -> Expr:
        if self.at_kw("+") or self.at_kw("-"):
            op = self.next().text
            return Unop(op, self.level_mul(term))
        return self.level_mul(term)

    def level_mul(self, term) -> Expr:
        a = self.level_pow(term)
        while self.at_kw("*") or self.at_kw("/"):
            op = self.next().text
            b = self.level_pow(term)
            a = Binop(op, a, b)
        return a

    def level_pow(self, term) -> Expr:
        a = self.level_dot(term)
        while self.at_kw("**"):
            self.next()
            b = self.level_dot(term)
            a = Binop("**", a, b)
        return a

    def level_dot(self, term) -> Expr:
        a = term()
        if self.at_kw("."):
            self.next()
            b = self.level_dot(term)
            a = Binop(".", a, b)
        return a

    def starts_aexpr(self) -> bool:
        t = self.peek()
        return t.kind in ("LP", "ID", "NUM") or (t.kind == "KW" and t.text in ("let", "fun", "if"))

    def fexpr(self) -> Expr:
        f = self.aexpr()
        while True:
            if self.at("LB"):
                f = GridIdx(self.grid_indices(), f)
            elif self.starts_aexpr():
                f = Apply(f, self.aexpr())
            else:
                return f

    def aexpr(self) -> Expr:
        t = self.peek()
        if t.kind == "LP":
            return self.tuple_of(self.rexpr)
        if t.kind == "KW" and t.text == "let":
            self.next()
            stmts = self.binding("in")
            self.expect("KW", "in")
            return Let(stmts, self.rexpr())
        if t.kind == "KW" and t.text == "fun":
            self.next()
            pat = self.tuple_of(self.lexpr)
            return Lambda(pat, self.rexpr())
        if t.kind == "KW" and t.text == "if":
            self.next()
            c = self.rexpr()
            self.expect("KW", "then")
            a = self.rexpr()
            self.expect("KW", "else")
            b = self.rexpr()
            return If(c, a, b)
        if t.kind == "ID":
            return Ident(self.next().text)
        if t.kind == "NUM":
            return Num(self.next().value)
        raise FmrSyntaxError("line %d: unexpected %r" % (t.line, t.text))


def _eval_const(e: Expr) -> Fraction:
    if isinstance(e, Num):
        return e.value
    if isinstance(e, Unop):
        v = _eval_const(e.a)
        return v if e.op == "+" else -v
    if isinstance(e, Binop) and e.op in "+-*/":
        a, b = _eval_const(e.a), _eval_const(e.b)
        return {"+": a + b, "-": a - b, "*": a * b, "/": a / b if b else None}[e.op]
    raise FmrSyntaxError("unsupported operator in a constant rational expression")


def parse(src: str) -> Program:
    """Parse the text of a .fmr file."""
    return Parser(src).program()


def parse_file(path) -> Program:
    with open(path, encoding="utf-8") as f:
        return parse(f.read())
