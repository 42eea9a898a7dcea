"""Dynamic operation count of one right-hand-side evaluation.

Evaluates a model's rates body on representative states (resting values
with the membrane potential set to -85, -40, 0 and +30 mV) with an
instrumented interpreter and averages the counts: + - * / as arithmetic
FLOPs, ``pow(x, n)`` with integer n as its multiplies, and exp / log / pow /
sqrt / tanh as transcendental (special-function) operations, reported
separately.  Only the branch a ternary takes is counted.  The part of the
body that depends on the membrane potential and constants alone (evaluated
once per cell and PDE step in tissue mode) is also counted on its own.
"""
from __future__ import annotations

import math
from collections import Counter

from .cexpr import Bin, Call, Cond, Num, Ref, Unary, Var
from .emit import _int_exponent, _is_half, supplement_for
from .model import Assign, If, Model


class _Eval:
    def __init__(self, m: Model, consts, states, tissue: int):
        self.m = m
        self.C = consts
        self.Y = states
        self.A = {}
        self.R = {}
        self.tissue = tissue
        self.n = Counter()

    def ev(self, e):
        n = self.n
        if isinstance(e, Num):
            return int(e.text) if e.is_int_literal else e.value
        if isinstance(e, Ref):
            if e.array == "STATES":
                return self.Y.get(e.name, 0.5)   # states initConsts leaves unset
            if e.array == "CONSTANTS":
                return self.C.get(e.name, 0.0)
            if e.array == "ALGEBRAIC":
                return self.A.get(e.name, 0.0)
            return self.R.get(e.name, 0.0)
        if isinstance(e, Var):
            return {"tissueFlag": self.tissue, "dimension": self.tissue - 10, "VOI": 0.0,
                "solveVmWithinODESolver": 0}[e.name]
        if isinstance(e, Unary):
            v = self.ev(e.e)
            return -v if e.op == "-" else (v if e.op == "+" else float(not v))
        if isinstance(e, Cond):
            return self.ev(e.a) if self.ev(e.c) else self.ev(e.b)
        if isinstance(e, Bin):
            if e.op in ("&&", "||"):
                a = self.ev(e.l)
                if e.op == "&&":
                    return float(bool(a) and bool(self.ev(e.r)))
                return float(bool(a) or bool(self.ev(e.r)))
            a, b = self.ev(e.l), self.ev(e.r)
            if e.op in "+-":
                n["add"] += 1
                return a + b if e.op == "+" else a - b
            if e.op == "*":
                n["mul"] += 1
                return a * b
            if e.op == "/":
                n["div"] += 1
                return a / b if b != 0 else math.copysign(math.inf, a) if a else math.nan
            n["cmp"] += 1
            return float({"<": a < b, ">": a > b, "<=": a <= b, ">=": a >= b, "==": a == b,
                          "!=": a != b}[e.op])
        if isinstance(e, Call):
            if e.fn == "computeIstim":
                return 0.0
            args = [self.ev(x) for x in e.args]
            if e.fn == "pow":
                k = _int_exponent(e.args[1])
                if k is not None:
                    n["mul"] += max(k.bit_length() - 1 + bin(k).count("1") - 1, 0)
                    return args[0] ** k
                if _is_half(e.args[1]):
                    n["sqrt"] += 1
                    return math.sqrt(args[0]) if args[0] >= 0 else math.nan
                n["pow"] += 1
                try:
                    return args[0] ** args[1]
                except (OverflowError, ZeroDivisionError):
                    return math.nan
            if e.fn in ("exp", "log", "sqrt", "tanh"):
                n[e.fn] += 1
                try:
                    return getattr(math, e.fn)(args[0])
                except (OverflowError, ValueError):
                    return math.nan
            if e.fn == "heaviside":
                n["cmp"] += 1
                return 1.0 if args[0] > 0 else 0.0
            if e.fn == "tissueSelect":
                t = args[0]
                return args[1] if t == 3 else args[2] if t == 2 else args[3]
            if e.fn in ("fabs", "floor"):
                return getattr(math, e.fn)(args[0])
            raise ValueError(e.fn)
        raise TypeError(e)

    def run(self, stmts, target):
        for st in stmts:
            if isinstance(st, Assign):
                v = self.ev(st.expr)
                t = st.target
                {"STATES": self.Y, "CONSTANTS": self.C, "ALGEBRAIC": self.A,
                 "RATES": self.R}[t.array][t.name] = v
            elif isinstance(st, If):
                self.run(st.then if self.ev(st.cond) else st.orelse, target)


def count_rhs(m: Model, tissue: int) -> dict:
    init = _Eval(m, {}, {}, tissue)
    init.run(m.init, "init")
    consts = dict(init.C)
    for c, v in supplement_for(m):
        consts[c] = eval(v)   # literal arithmetic of the supplement table
    states = dict(init.Y)
    v0 = m.states[0]
    volts = [-85.0, -40.0, 0.0, 30.0]
    if m.vm_to_state == "aliev":
        volts = [(v + 80) / 100 for v in volts]
    elif m.vm_to_state == "bueno":
        volts = [(v + 84) / 85.7 for v in volts]
    from .hoist import analyse, invariant_statements
    from .emit import tissue_subtrees
    inv_body = invariant_statements(m.rates, analyse(m, m.rates).invariant)
    subtrees = tissue_subtrees(m)
    total, inv = Counter(), Counter()
    for v in volts:
        ev = _Eval(m, dict(consts), dict(states, **{v0: v}), tissue)
        ev.run(m.rates, "rates")
        total.update(ev.n)
        ev = _Eval(m, dict(consts), dict(states, **{v0: v}), tissue)
        ev.run(inv_body, "rates")
        for e in subtrees:
            ev.ev(e)
        inv.update(ev.n)

    def summary(c):
        avg = {k: c[k] / len(volts) for k in c}
        flops = avg.get("add", 0) + avg.get("mul", 0) + avg.get("div", 0)
        sfu = sum(avg.get(k, 0) for k in ("exp", "log", "pow", "sqrt", "tanh"))
        return flops, sfu, avg

    flops, sfu, avg = summary(total)
    iflops, isfu, _ = summary(inv)
    # tissue mode evaluates the membrane-potential-only part once per cell and
    # PDE step (hoist.py): per stage evaluation only the rest runs
    return {"flops": flops, "transcendental": sfu,
            "invariant_flops": iflops, "invariant_transcendental": isfu,
            **{k: round(v, 2) for k, v in avg.items()}}
