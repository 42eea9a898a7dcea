"""Tokenizer and Pratt parser for the C expressions found in cellML2foam model headers.

The generated ionic-model headers (``src/ionicModels/<Model>/<Model>_<Year>.H``,
emitted by ``applications/scripts/cellML2foam/src/mapping_engine.py:268-437``)
contain straight-line C: array assignments whose right-hand sides use
``+ - * /``, unary minus, comparisons, ``&& ||``, the ternary operator and calls
to ``exp log pow sqrt tanh fabs floor heaviside computeIstim tissueSelect``.
This module turns one such expression into a small immutable AST that the
emitters walk.  Only that subset of C is accepted; anything else raises
``ParseError`` so a new construct in a regenerated header is noticed instead
of being silently mistranslated.
"""
from __future__ import annotations

import re
from dataclasses import dataclass
from typing import Tuple, Union


class ParseError(ValueError):
    pass


@dataclass(frozen=True)
class Num:
    text: str          # literal as written (kept for exact double rounding)

    @property
    def value(self) -> float:
        return float(self.text.rstrip("fF"))

    @property
    def is_int_literal(self) -> bool:
        return re.fullmatch(r"\d+", self.text) is not None


@dataclass(frozen=True)
class Ref:
    """Array element ``STATES[x]``, ``CONSTANTS[x]``, ``ALGEBRAIC[x]`` or ``RATES[x]``."""
    array: str
    name: str


@dataclass(frozen=True)
class Var:
    """Scalar identifier: ``VOI``, ``tissueFlag``, ``solveVmWithinODESolver``, ``stimulus`` ..."""
    name: str


@dataclass(frozen=True)
class Call:
    fn: str
    args: Tuple["Node", ...]


@dataclass(frozen=True)
class Unary:
    op: str
    e: "Node"


@dataclass(frozen=True)
class Bin:
    op: str
    l: "Node"
    r: "Node"


@dataclass(frozen=True)
class Cond:
    c: "Node"
    a: "Node"
    b: "Node"


Node = Union[Num, Ref, Var, Call, Unary, Bin, Cond]

ARRAYS = ("STATES", "CONSTANTS", "ALGEBRAIC", "RATES")

_TOKEN_RE = re.compile(
    r"""
    (?P<ws>\s+)
  | (?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?[fF]?)
  | (?P<id>[A-Za-z_][A-Za-z_0-9]*(?:::[A-Za-z_][A-Za-z_0-9]*)*)
  | (?P<op>&&|\|\||==|!=|<=|>=|[-+*/?:(),<>!\[\]])
    """,
    re.VERBOSE,
)


def tokenize(src: str):
    pos = 0
    out = []
    while pos < len(src):
        m = _TOKEN_RE.match(src, pos)
        if not m:
            raise ParseError(f"bad character {src[pos]!r} in {src!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        out.append((kind, m.group(kind)))
    out.append(("eof", ""))
    return out


# binding powers: higher binds tighter
_BINARY = {
    "||": 3, "&&": 4,
    "==": 7, "!=": 7,
    "<": 8, ">": 8, "<=": 8, ">=": 8,
    "+": 10, "-": 10,
    "*": 11, "/": 11,
}
_TERNARY_BP = 2


class _Parser:
    def __init__(self, src: str):
        self.src = src
        self.toks = tokenize(src)
        self.i = 0

    def peek(self):
        return self.toks[self.i]

    def take(self, want=None):
        tok = self.toks[self.i]
        if want is not None and tok[1] != want:
            raise ParseError(f"expected {want!r}, got {tok[1]!r} in {self.src!r}")
        self.i += 1
        return tok

    def parse(self) -> Node:
        e = self.expr(0)
        if self.peek()[0] != "eof":
            raise ParseError(f"trailing tokens after expression in {self.src!r}")
        return e

    def expr(self, min_bp: int) -> Node:
        lhs = self.prefix()
        while True:
            kind, tok = self.peek()
            if tok == "?" and _TERNARY_BP >= min_bp:
                self.take("?")
                a = self.expr(0)
                self.take(":")
                b = self.expr(_TERNARY_BP)      # right associative
                lhs = Cond(lhs, a, b)
                continue
            bp = _BINARY.get(tok) if kind == "op" else None
            if bp is None or bp < min_bp:
                return lhs
            self.take()
            rhs = self.expr(bp + 1)             # left associative
            lhs = Bin(tok, lhs, rhs)

    def prefix(self) -> Node:
        kind, tok = self.take()
        if kind == "num":
            return Num(tok)
        if kind == "op" and tok in "-+!":
            # unary binds tighter than * and /
            return Unary(tok, self.expr(12))
        if kind == "op" and tok == "(":
            e = self.expr(0)
            self.take(")")
            return e
        if kind == "id":
            name = tok.split("::")[-1]
            nk, nt = self.peek()
            if nt == "[":
                if name not in ARRAYS:
                    raise ParseError(f"unknown array {name} in {self.src!r}")
                self.take("[")
                ik, it = self.take()
                if ik != "id":
                    raise ParseError(f"non-symbolic index in {self.src!r}")
                self.take("]")
                return Ref(name, it)
            if nt == "(":
                self.take("(")
                args = []
                if self.peek()[1] != ")":
                    while True:
                        args.append(self.expr(0))
                        if self.peek()[1] == ",":
                            self.take(",")
                            continue
                        break
                self.take(")")
                return Call(name, tuple(args))
            return Var(name)
        raise ParseError(f"unexpected token {tok!r} in {self.src!r}")


def parse_expr(src: str) -> Node:
    return _Parser(src).parse()


def walk(node: Node):
    """Yield every node of the tree, parents before children."""
    yield node
    if isinstance(node, Call):
        for a in node.args:
            yield from walk(a)
    elif isinstance(node, Unary):
        yield from walk(node.e)
    elif isinstance(node, Bin):
        yield from walk(node.l)
        yield from walk(node.r)
    elif isinstance(node, Cond):
        yield from walk(node.c)
        yield from walk(node.a)
        yield from walk(node.b)


def refs(node: Node, array: str | None = None):
    for n in walk(node):
        if isinstance(n, Ref) and (array is None or n.array == array):
            yield n
