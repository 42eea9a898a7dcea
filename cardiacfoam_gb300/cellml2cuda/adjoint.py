"""Reverse-mode derivative (vector-Jacobian product) of a model's right-hand
side in tissue mode, emitted as a CUDA device function.

The body the tissue step evaluates (``rates``: RATES of every state but V, and
``Iion_cm``) is turned into three-address code: every operator node of every
expression gets a named temporary, conditionals (``c ? a : b`` and
``tissueSelect``) become if/else blocks so that only the taken branch is
evaluated and differentiated.  The emitted function first runs that code
forward (the same operations as the forward RHS, in the header's order), then
walks the statements backwards, pushing the adjoint of each statement's target
down its expression tree with the derivative rule of each operator:

    a + b, a - b      (g, g), (g, -g)
    a * b, a / b      (g b, g a), (g / b, -g v / b)      v = the node's value
    -a, exp a, log a  -g, g v, g / a
    sqrt a, tanh a    g / (2 v), g (1 - v^2)
    pow(a, n)         g n a^(n-1) (and g v log a for a non-constant exponent)
    fabs a            g sign(a);  floor, heaviside, comparisons: 0
    exp(x) - 1        evaluated as cfg_expm1(x), adjoint g (v + 1)

Algebraics read before their assignment are the zeroed scratch of
``derivatives()`` (constant 0).  The single-cell stimulus does not exist in
tissue mode (the reference refuses it) and differentiates to 0.

    rhs_vjp<R, KS>(t, y, K, tissue, dbar, ibar, ybar, pbar)

adds to ybar[NS] the product of the transposed Jacobian of (dydt, Iion_cm) with
respect to the states with (dbar, ibar), and to pbar[NSCALE] the same with
respect to the scalable conductances (SCALE_ORDER: GNa, GCaL, GKr, GKs, GK1,
Gto), whose values K(C_x) are the already scaled constants.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

from .cexpr import Bin, Call, Cond, Node, Num, Ref, Unary, Var
from .emit import SCALABLE, SCALE_ORDER, _int_exponent, _is_half, ident
from .model import Assign, Fatal, If, Model, use_before_def

_CMP = ("==", "!=", "<", ">", "<=", ">=", "&&", "||")


def _expm1_arg(e: Node):
    """x of exp(x) - 1 (the GHK flux denominators), else None: evaluated as
    cfg_expm1(x), which in FP32 does not cancel to 0 as x -> 0."""
    if isinstance(e, Bin) and e.op == "-" and isinstance(e.r, Num) and \
            float(e.r.text.rstrip("fF")) == 1.0 and isinstance(e.l, Call) and e.l.fn == "exp":
        return e.l.args[0]
    return None


def tissue_mode_body(stmts) -> List[Assign]:
    """The statements with solveVmWithinODESolver = false resolved."""
    out: List[Assign] = []
    for st in stmts:
        if isinstance(st, Assign):
            out.append(st)
        elif isinstance(st, If):
            c = st.cond
            if isinstance(c, Var) and c.name == "solveVmWithinODESolver":
                out.extend(tissue_mode_body(st.orelse))
            elif isinstance(c, Unary) and c.op == "!" and isinstance(c.e, Var) and \
                    c.e.name == "solveVmWithinODESolver":
                out.extend(tissue_mode_body(st.then))
            else:
                raise ValueError(f"unsupported run-time if ({c}) in the adjoint")
        elif isinstance(st, Fatal):
            continue
    return out


class _Gen:
    """Three-address forward code and the matching reverse sweep."""

    def __init__(self, m: Model, early):
        self.m = m
        self.early = set(early)
        self.params = {v: k for k, v in SCALABLE[m.name].items()}   # constant -> scale key
        self.n = 0
        self.decl: List[str] = []           # hoisted temporaries
        self.defined: Dict[str, str] = {}   # algebraic -> current value name
        self.value: Dict[int, str] = {}     # id(node) -> value name
        self.alg_bar: Dict[str, str] = {}   # algebraic value name -> its adjoint accumulator
        self.states_read = set()

    def tmp(self, prefix="t") -> str:
        self.n += 1
        name = f"{prefix}{self.n}"
        self.decl.append(f"    R {name} = R(0);")
        return name

    # ---------------------------------------------------------------- forward
    def leaf(self, e: Node):
        if isinstance(e, Num):
            return e.text if e.is_int_literal else f"R({e.text})"
        if isinstance(e, Ref):
            if e.array == "STATES":
                self.states_read.add(e.name)
                return f"y_{e.name}"
            if e.array == "CONSTANTS":
                return f"p_{e.name}" if e.name in self.params else f"K(C_{e.name})"
            if e.array == "ALGEBRAIC":
                return self.defined.get(e.name, "R(0)")
            raise ValueError(f"read of {e.array} in the right-hand side")
        if isinstance(e, Var):
            if e.name == "tissueFlag":
                return "tissue"
            if e.name == "dimension":
                return "(tissue - 10)"
            if e.name == "solveVmWithinODESolver":
                return "false"
            if e.name == "VOI":
                return "t"
            raise ValueError(f"unknown variable {e.name}")
        return None

    def cond(self, e: Node, out: List[str], ind: str) -> str:
        """A boolean expression (never differentiated)."""
        if isinstance(e, Bin) and e.op in _CMP:
            return f"({self.cond_or_val(e.l, out, ind)} {e.op} {self.cond_or_val(e.r, out, ind)})"
        if isinstance(e, Unary) and e.op == "!":
            return f"(!{self.cond(e.e, out, ind)})"
        return f"({self.fwd(e, out, ind)} != R(0))"

    def cond_or_val(self, e: Node, out, ind) -> str:
        if isinstance(e, Bin) and e.op in _CMP or isinstance(e, Unary) and e.op == "!":
            return self.cond(e, out, ind)
        return self.fwd(e, out, ind)

    def fwd(self, e: Node, out: List[str], ind: str) -> str:
        lf = self.leaf(e)
        if lf is not None:
            return lf
        x = _expm1_arg(e)
        if x is not None:
            a = self.fwd(x, out, ind)
            v = self.tmp()
            out.append(f"{ind}{v} = cfg_expm1({a});")
            self.value[id(e)] = v
            return v
        if isinstance(e, Unary):
            if e.op == "!":
                raise ValueError("logical not in an arithmetic position")
            a = self.fwd(e.e, out, ind)
            if e.op == "+":
                self.value[id(e)] = a
                return a
            v = self.tmp()
            out.append(f"{ind}{v} = (-{a});")
            self.value[id(e)] = v
            return v
        if isinstance(e, Bin):
            if e.op in _CMP:
                v = self.tmp()
                out.append(f"{ind}{v} = {self.cond(e, out, ind)} ? R(1) : R(0);")
                self.value[id(e)] = v
                return v
            a = self.fwd(e.l, out, ind)
            b = self.fwd(e.r, out, ind)
            v = self.tmp()
            out.append(f"{ind}{v} = ({a} {e.op} {b});")
            self.value[id(e)] = v
            return v
        if isinstance(e, Cond):
            c = self.tmp("c")
            out.append(f"{ind}{c} = {self.cond(e.c, out, ind)} ? R(1) : R(0);")
            v = self.tmp()
            out.append(f"{ind}if ({c} != R(0)) {{")
            a = self.fwd(e.a, out, ind + "    ")
            out.append(f"{ind}    {v} = {a};")
            out.append(f"{ind}}} else {{")
            b = self.fwd(e.b, out, ind + "    ")
            out.append(f"{ind}    {v} = {b};")
            out.append(f"{ind}}}")
            self.value[id(e)] = v
            self.value[("cond", id(e))] = c
            return v
        if isinstance(e, Call):
            if e.fn == "computeIstim":
                return "R(0)"
            if e.fn == "tissueSelect":
                # tissueSelect(flag, endo, m, epi) as nested conditionals on tissue
                sel = Cond(Bin("==", Var("tissueFlag"), Num("3")), e.args[1],
                           Cond(Bin("==", Var("tissueFlag"), Num("2")), e.args[2], e.args[3]))
                v = self.fwd(sel, out, ind)
                self.value[id(e)] = v
                self.value[("alias", id(e))] = sel
                return v
            if e.fn == "heaviside":
                a = self.fwd(e.args[0], out, ind)
                v = self.tmp()
                out.append(f"{ind}{v} = ({a} > R(0)) ? R(1) : R(0);")
                self.value[id(e)] = v
                return v
            args = [self.fwd(x, out, ind) for x in e.args]
            v = self.tmp()
            if e.fn == "pow":
                n = _int_exponent(e.args[1])
                if n is not None:
                    out.append(f"{ind}{v} = cfg_ipow<{n}>({args[0]});")
                elif _is_half(e.args[1]):
                    out.append(f"{ind}{v} = cfg_sqrt({args[0]});")
                else:
                    out.append(f"{ind}{v} = cfg_pow({args[0]}, {args[1]});")
            elif e.fn in ("exp", "log", "sqrt", "tanh", "fabs", "floor"):
                out.append(f"{ind}{v} = cfg_{e.fn}({args[0]});")
            else:
                raise ValueError(f"{self.m.name}: no derivative rule for {e.fn}")
            self.value[id(e)] = v
            return v
        raise TypeError(e)

    # ---------------------------------------------------------------- reverse
    def acc(self, e: Node, g: str, out: List[str], ind: str):
        """Add the adjoint g of node e to its inputs."""
        if isinstance(e, Num) or isinstance(e, Var):
            return
        if isinstance(e, Ref):
            if e.array == "STATES":
                out.append(f"{ind}ybar[S_{e.name}] += {g};")
            elif e.array == "CONSTANTS" and e.name in self.params:
                out.append(f"{ind}pbar[SCALE_{self.params[e.name]}] += {g};")
            elif e.array == "ALGEBRAIC" and id(e) in self.alg_ref:
                out.append(f"{ind}{self.alg_ref[id(e)]} += {g};")
            return
        val = lambda x: self.value.get(id(x)) or self.leaf(x)
        x = _expm1_arg(e)
        if x is not None:
            self.push(x, f"({g} * ({self.value[id(e)]} + R(1)))", out, ind)
            return
        if isinstance(e, Unary):
            if e.op == "+":
                self.acc(e.e, g, out, ind)
            else:
                self.push(e.e, f"(-{g})", out, ind)
            return
        if isinstance(e, Bin):
            if e.op in _CMP:
                return
            a, b, v = val(e.l), val(e.r), self.value[id(e)]
            if e.op == "+":
                self.push(e.l, g, out, ind)
                self.push(e.r, g, out, ind)
            elif e.op == "-":
                self.push(e.l, g, out, ind)
                self.push(e.r, f"(-{g})", out, ind)
            elif e.op == "*":
                self.push(e.l, f"({g} * {b})", out, ind)
                self.push(e.r, f"({g} * {a})", out, ind)
            elif e.op == "/":
                self.push(e.l, f"({g} / {b})", out, ind)
                self.push(e.r, f"(-{g} * {v} / {b})", out, ind)
            return
        if isinstance(e, Cond):
            c = self.value[("cond", id(e))]
            out.append(f"{ind}if ({c} != R(0)) {{")
            self.push(e.a, g, out, ind + "    ")
            out.append(f"{ind}}} else {{")
            self.push(e.b, g, out, ind + "    ")
            out.append(f"{ind}}}")
            return
        if isinstance(e, Call):
            if e.fn in ("computeIstim", "heaviside", "floor"):
                return
            if e.fn == "tissueSelect":
                self.acc(self.value[("alias", id(e))], g, out, ind)
                return
            v = self.value[id(e)]
            a = val(e.args[0])
            if e.fn == "exp":
                self.push(e.args[0], f"({g} * {v})", out, ind)
            elif e.fn == "log":
                self.push(e.args[0], f"({g} / {a})", out, ind)
            elif e.fn == "sqrt":
                self.push(e.args[0], f"({g} / (R(2) * {v}))", out, ind)
            elif e.fn == "tanh":
                self.push(e.args[0], f"({g} * (R(1) - {v} * {v}))", out, ind)
            elif e.fn == "fabs":
                self.push(e.args[0], f"({g} * ({a} >= R(0) ? R(1) : R(-1)))", out, ind)
            elif e.fn == "pow":
                n = _int_exponent(e.args[1])
                if n is not None:
                    d = "R(1)" if n == 1 else (f"R({n}) * {a}" if n == 2 else
                                               f"R({n}) * cfg_ipow<{n - 1}>({a})")
                    self.push(e.args[0], f"({g} * {d})", out, ind)
                elif _is_half(e.args[1]):
                    self.push(e.args[0], f"({g} / (R(2) * {v}))", out, ind)
                else:
                    b = val(e.args[1])
                    self.push(e.args[0], f"({g} * {b} * cfg_pow({a}, {b} - R(1)))", out, ind)
                    if not isinstance(e.args[1], Num):
                        self.push(e.args[1], f"({g} * {v} * cfg_log({a}))", out, ind)
            return
        raise TypeError(e)

    def push(self, e: Node, g: str, out, ind):
        """Adjoint g flows into node e: leaves accumulate, inner nodes get a
        temporary and propagate further."""
        if isinstance(e, (Num, Var)):
            return
        if isinstance(e, Ref):
            self.acc(e, g, out, ind)
            return
        t = self.tmp("g")
        out.append(f"{ind}{t} = {g};")
        self.acc(e, t, out, ind)


def emit_rhs_vjp(m: Model) -> str:
    body = tissue_mode_body(m.rates)
    early = use_before_def(m.rates)
    gen = _Gen(m, early)
    gen.alg_ref = {}
    fwd: List[str] = []
    targets: List[Tuple[Assign, str]] = []
    for st in body:
        t = st.target
        if t.array == "RATES" and t.name == m.states[0]:
            continue                                  # the PDE owns Vm
        # record, for the reverse sweep, which value each algebraic read refers to
        for r in _alg_reads(st.expr):
            if r.name in gen.defined:
                gen.alg_ref[id(r)] = "b" + gen.defined[r.name]
        v = gen.fwd(st.expr, fwd, "    ")
        if t.array == "ALGEBRAIC":
            name = gen.tmp("a")
            fwd.append(f"    {name} = {v};")
            gen.defined[t.name] = name
            gen.decl.append(f"    R b{name} = R(0);")
            targets.append((st, name))
        elif t.array == "RATES":
            targets.append((st, f"dbar[S_{t.name}]"))
        else:
            raise ValueError(f"assignment to {t.array} in the right-hand side")
    iion = gen.defined.get(m.iion_name)
    if iion is None:
        raise ValueError(f"{m.name}: the right-hand side does not compute {m.iion_name}")
    rev: List[str] = [f"    b{iion} += ibar;"]
    for st, name in reversed(targets):
        g = name if name.startswith("dbar") else f"b{name}"
        if name.startswith("dbar"):
            rev.append(f"    {{ const R g0 = {g};")
            gen.push(st.expr, "g0", rev, "      ")
            rev.append("    }")
        else:
            gen.push(st.expr, g, rev, "    ")
    L: List[str] = []
    L.append("// Reverse-mode derivative of rhs<R, false> (tissue mode): adds to ybar the")
    L.append("// transposed Jacobian of (dydt without V, Iion_cm) with respect to the states")
    L.append("// applied to (dbar, ibar), and to pbar the same for the scalable conductances.")
    L.append("template <class R, class KS>")
    L.append("__device__ __noinline__ void rhs_vjp(double t, const R* y, const KS& K, int tissue, "
             "const R* dbar, R ibar, R* ybar, R* pbar)")
    L.append("{")
    L.append("    (void)t; (void)tissue;")
    for s in m.states:
        if s in gen.states_read:
            L.append(f"    const R y_{s} = y[S_{s}];")
    for c, key in gen.params.items():
        L.append(f"    const R p_{c} = K(C_{c});")
    L.extend(gen.decl)
    L.extend(fwd)
    L.extend(rev)
    L.append("}")
    return "\n".join(L) + "\n"


def _alg_reads(e: Node):
    from .cexpr import walk
    for n in walk(e):
        if isinstance(n, Ref) and n.array == "ALGEBRAIC":
            yield n


def emit_adjoint_header(m: Model, src_rel: str) -> str:
    ns = ident(m.name)
    L = [f"// Generated by cardiacfoam_gb300.cellml2cuda from {src_rel}: the reverse-mode",
         "// derivative of the model's tissue-mode right-hand side.  Regenerate with",
         "// `python -m cardiacfoam_gb300.cellml2cuda` instead of editing.",
         "#pragma once",
         "",
         f'#include "{ns}.cuh"',
         "",
         f"namespace cfg {{ namespace {ns} {{",
         ""]
    L.append(emit_rhs_vjp(m))
    L.append(f"}} }}  // namespace cfg::{ns}")
    return "\n".join(L) + "\n"
