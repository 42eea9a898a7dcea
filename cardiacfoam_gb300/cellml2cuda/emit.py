"""Emitters: model IR -> CUDA device functions and -> plain C for the CPU oracle.

Two outputs are produced from one :class:`~.model.Model`:

``emit_cuda``
    ``csrc/models/<model>.cuh``: a namespace with the state layout, a
    ``__host__ __device__`` constants/initial-state function (double), and the
    right-hand side as a template ``rhs<R, SOLVE_VM>(...)`` over the arithmetic
    type ``R`` (``double`` for the plain form, ``float`` for the mixed form).
    Algebraic variables become local values (never an array), so the compiler
    keeps them in registers and drops the ones a caller does not need.
    ``pow`` with an integer exponent is written as a product and ``pow(x, 1/2)``
    as ``sqrt``; everything else keeps the reference's evaluation order.

``emit_c``
    ``oracle/models/<model>.h``: C99 functions with the reference's calling
    convention (STATES/RATES/ALGEBRAIC arrays, ``pow`` kept as written), so the
    CPU oracle evaluates exactly what ``<Model>_<Year>.H`` evaluates.

Reads of an algebraic before its assignment (``ALGEBRAIC[Istim]`` in ORd and
ToRORd_dynCl, e.g. ``ORd_2011.H:962``) see the zeroed scratch array that
``derivatives()`` passes (``ORd.C:167``); both emitters reproduce that.
"""
from __future__ import annotations

import re
from typing import Dict, List

from .cexpr import Bin, Call, Cond, Node, Num, Ref, Unary, Var, walk
from .model import Assign, Fatal, If, Model, iter_assigns, refs, use_before_def

# states stored and accumulated in double precision in the mixed form: the
# membrane potential and every ion concentration / CaMK occupancy (slow states
# whose per-step increments fall below float resolution).  Gates stay float.
WIDE_STATES = {
    "TNNP": ["V", "K_i", "Na_i", "Ca_i", "Ca_SR"],
    "ORd": ["membrane_V", "CaMK_CaMKt", "Na_i", "Na_ss", "K_i", "K_ss", "Ca_ss",
            "Ca_nsr", "Ca_jsr", "Ca_i"],
    "ToRORd_dynCl": ["V", "CaMKt", "Nai", "Nass", "Ki", "Kss", "Cass", "Cansr",
                     "Cajsr", "Cai", "Cli", "Clss"],
    "AlievPanfilov": ["u", "recovery_r"],
    "BuenoOrovio": ["u", "v", "w", "s"],
    "monodomainFDAManufactured": ["V", "u1", "u2", "u3"],
    "bidomainFDAManufactured": ["BidomainV", "BidomainU1", "BidomainU2", "BidomainU3"],
}

# constants a batched run may scale per cell (log-uniform factors); the
# scale multiplies the constant right after initConsts assigns it, before any
# constant derived from it is computed.
SCALABLE = {
    "TNNP": {"GNa": "g_Na", "GCaL": "g_CaL", "GKr": "g_Kr", "GKs": "g_Ks",
             "GK1": "g_K1", "Gto": "g_to"},
    "ORd": {"GNa": "AC_GNa", "GCaL": "AC_PCa_b", "GKr": "AC_GKr_b", "GKs": "AC_GKs_b",
            "GK1": "AC_GK1_b", "Gto": "AC_Gto_b"},
    "ToRORd_dynCl": {"GNa": "AC_GNa", "GCaL": "AC_PCa_b", "GKr": "AC_GKr_b",
                     "GKs": "AC_GKs_b", "GK1": "AC_GK1_b", "Gto": "AC_Gto_b"},
    "AlievPanfilov": {},
    "BuenoOrovio": {},
    "monodomainFDAManufactured": {},
    "bidomainFDAManufactured": {},
}
SCALE_ORDER = ["GNa", "GCaL", "GKr", "GKs", "GK1", "Gto"]

# tissue keys and their flags; the manufactured-solution model selects its
# constants by mesh dimension instead (flags 11-13: dimension = flag - 10)
TISSUE_FLAGS = {"epicardialCells": 1, "mCells": 2, "endocardialCells": 3, "myocyte": 4,
                "1D": 11, "2D": 12, "3D": 13}

# intracellular calcium state of each model (peak Ca of a beat)
CALCIUM_STATE = {"TNNP": "Ca_i", "ORd": "Ca_i", "ToRORd_dynCl": "Cai"}


def scale_dependent_constants(m: "Model") -> List[str]:
    """Constants whose value depends on a per-cell scale (the scaled ones and
    every constant initConsts computes from them) and that the right-hand
    side or the current evaluation reads, in constant-index order."""
    dep = set(SCALABLE[m.name].values())
    changed = True
    while changed:
        changed = False
        for st in iter_assigns(m.init):
            t = st.target
            if t.array == "CONSTANTS" and t.name not in dep and any(
                    r.array == "CONSTANTS" and r.name in dep for r in refs(st.expr)):
                dep.add(t.name)
                changed = True
    used = set()

    def visit(body):
        for st in body:
            exprs = [st.expr] if isinstance(st, Assign) else \
                [st.cond] if isinstance(st, If) else []
            for e in exprs:
                used.update(r.name for r in refs(e) if r.array == "CONSTANTS")
            if isinstance(st, If):
                visit(st.then)
                visit(st.orelse)

    visit(m.rates)
    visit(m.variables)
    return [c for c in m.constants if c in dep and c in used]

# Constants a model's right-hand side reads but its initConsts never assigns.
# The reference zero-fills CONSTANTS, so ORd_2011.H evaluates the Na/K pump
# with zeros and Iion_cm is NaN from the first call.  The supplement assigns
# them: the INaK parameters as ToRORd_dynCl_2023.H:728-753 sets them for the
# same pump formulation (a2 = k2p, a4 = k4p*MgATP/Kmgatp/(1+MgATP/Kmgatp),
# b1 = k1m*MgADP), Pnak = 30 and upScale = 1 (non-epicardial) of the
# published O'Hara-Rudy 2011 model.
SUPPLEMENT = {
    "ORd": [("AC_H", "1e-07"), ("AC_Khp", "1.698e-07"), ("AC_Kki", "0.5"),
            ("AC_Kko", "0.3582"), ("AC_Kmgatp", "1.698e-07"), ("AC_Knai0", "9.073"),
            ("AC_Knao0", "27.78"), ("AC_Knap", "224.0"), ("AC_Kxkur", "292.0"),
            ("AC_MgATP", "9.8"), ("AC_delta", "-0.155"), ("AC_eP", "4.2"),
            ("AC_k1p", "949.5"), ("AC_k2m", "39.4"), ("AC_k3m", "79300.0"),
            ("AC_k3p", "1899.0"), ("AC_k4m", "40.0"), ("AC_Pnak", "30.0"),
            ("AC_upScale", "1.0"), ("AC_a2", "687.2"),
            ("AC_a4", "639.0 * 9.8 / 1.698e-07 / (1.0 + 9.8 / 1.698e-07)"),
            ("AC_b1", "182.4 * 0.05")],
}


def unassigned_constants(m: Model) -> List[str]:
    from .cexpr import refs
    assigned = {a.target.name for a in iter_assigns(m.init) if a.target.array == "CONSTANTS"}
    used = set()
    for body in (m.init, m.rates, m.variables):
        for a in iter_assigns(body):
            used |= {r.name for r in refs(a.expr, "CONSTANTS")}
    return sorted(used - assigned)


def supplement_for(m: Model):
    sup = SUPPLEMENT.get(m.name, [])
    missing = unassigned_constants(m)
    if sorted(c for c, _ in sup) != missing:
        raise ValueError(f"{m.name}: supplement {sorted(c for c, _ in sup)} does not match the "
                         f"unassigned constants {missing}")
    return sup


def ident(model_name: str) -> str:
    return re.sub(r"[^a-z0-9]", "_", model_name.lower())


def _int_exponent(e: Node):
    """Integer value of a pow exponent literal such as 2.0, 3, 8.00000."""
    if isinstance(e, Num):
        v = e.value
        if v == int(v) and 1 <= v <= 16:
            return int(v)
    return None


def _is_half(e: Node) -> bool:
    if isinstance(e, Bin) and e.op == "/" and isinstance(e.l, Num) and isinstance(e.r, Num):
        return e.l.value == 1.0 and e.r.value == 2.0
    return isinstance(e, Num) and e.value == 0.5


def _is_int_expr(e: Node) -> bool:
    if isinstance(e, Num):
        return e.is_int_literal
    if isinstance(e, Var):
        return e.name in ("tissueFlag", "tissue")
    if isinstance(e, Call):
        return e.fn == "heaviside"
    if isinstance(e, Unary):
        return _is_int_expr(e.e) or e.op == "!"
    if isinstance(e, Bin):
        if e.op in ("==", "!=", "<", ">", "<=", ">=", "&&", "||"):
            return True
        return _is_int_expr(e.l) and _is_int_expr(e.r)
    if isinstance(e, Cond):
        return _is_int_expr(e.a) and _is_int_expr(e.b)
    return False


class _Printer:
    """Expression printer; subclasses define how names and calls are spelled."""

    def __init__(self, m: Model):
        self.m = m

    def num(self, n: Num) -> str:
        raise NotImplementedError

    def ref(self, r: Ref) -> str:
        raise NotImplementedError

    def var(self, v: Var) -> str:
        raise NotImplementedError

    def call(self, c: Call) -> str:
        raise NotImplementedError

    def __call__(self, e: Node) -> str:
        if isinstance(e, Num):
            return self.num(e)
        if isinstance(e, Ref):
            return self.ref(e)
        if isinstance(e, Var):
            return self.var(e)
        if isinstance(e, Call):
            return self.call(e)
        if isinstance(e, Unary):
            return f"({e.op}{self(e.e)})"
        if isinstance(e, Bin):
            if e.op == "/" and _is_int_expr(e.l) and _is_int_expr(e.r):
                raise ValueError(f"{self.m.name}: integer division in model expression")
            return f"({self(e.l)} {e.op} {self(e.r)})"
        if isinstance(e, Cond):
            return f"({self(e.c)} ? {self(e.a)} : {self(e.b)})"
        raise TypeError(e)


# --------------------------------------------------------------------------
# CUDA


def _is_one(e) -> bool:
    try:
        return isinstance(e, Num) and float(e.text) == 1.0
    except ValueError:
        return False


class _CudaPrinter(_Printer):
    def __call__(self, e: Node) -> str:
        # exp(x) - 1 (the GHK flux denominators) through cfg_expm1: the FP64
        # overload evaluates exactly exp(x) - 1.0, the FP32 one is expm1f,
        # which does not cancel to 0 as x -> 0 (Vm crossing 0 mV)
        if (self.mode == "rhs" and isinstance(e, Bin) and e.op == "-" and _is_one(e.r)
                and isinstance(e.l, Call) and e.l.fn == "exp"):
            return f"cfg_expm1({self(e.l.args[0])})"
        return super().__call__(e)

    def __init__(self, m: Model, early: List[str], mode: str):
        super().__init__(m)
        self.early = set(early)
        self.mode = mode            # "init" | "rhs"
        self.defined = set()
        self.states_read = set()    # states the body reads (loaded once, up front)

    def num(self, n: Num) -> str:
        if n.is_int_literal:
            return n.text
        if self.mode == "init":
            return n.text if re.search(r"[.eE]", n.text) else n.text + ".0"
        return f"R({n.text})"

    def ref(self, r: Ref) -> str:
        if r.array == "STATES":
            if self.mode == "init":
                return f"y[S_{r.name}]"
            self.states_read.add(r.name)
            return f"y_{r.name}"
        if r.array == "CONSTANTS":
            return f"C[C_{r.name}]" if self.mode == "init" else f"K(C_{r.name})"
        if r.array == "ALGEBRAIC":
            if r.name not in self.defined:
                # zeroed scratch in derivatives(): read as 0
                return "R(0)"
            return f"a_{r.name}"
        if r.array == "RATES":
            return f"dydt[S_{r.name}]"
        raise TypeError(r)

    def var(self, v: Var) -> str:
        if v.name == "tissueFlag":
            return "tissue"
        if v.name == "dimension":
            return "(tissue - 10)"
        if v.name == "solveVmWithinODESolver":
            return "SOLVE_VM"
        if v.name == "VOI":
            return "t"
        raise ValueError(f"unknown variable {v.name}")

    def call(self, c: Call) -> str:
        a = c.args
        if c.fn == "pow":
            n = _int_exponent(a[1])
            if n is not None:
                return f"cfg_ipow<{n}>({self(a[0])})"
            if _is_half(a[1]):
                return f"cfg_sqrt({self(a[0])})"
            return f"cfg_pow({self(a[0])}, {self(a[1])})"
        if c.fn in ("exp", "log", "sqrt", "tanh", "fabs", "floor"):
            return f"cfg_{c.fn}({self(a[0])})"
        if c.fn == "heaviside":
            return f"(({self(a[0])}) > R(0) ? 1 : 0)" if self.mode != "init" \
                else f"(({self(a[0])}) > 0.0 ? 1 : 0)"
        if c.fn == "computeIstim":
            # stimulus timing stays in double in every precision; tissue runs
            # (SOLVE_VM false) have no single-cell stimulus: the reference
            # refuses an active one (myocardiumDomain.C:377-394)
            return "(SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0))"
        if c.fn == "tissueSelect":
            return (f"((tissue == 3) ? {self(a[1])} : (tissue == 2) ? {self(a[2])} "
                    f": {self(a[3])})")
        raise ValueError(f"{self.m.name}: unsupported function {c.fn}")


def _cuda_body(m: Model, stmts, pr: _CudaPrinter, indent: str, out: List[str]):
    for st in stmts:
        if isinstance(st, Assign):
            rhs = pr(st.expr)
            t = st.target
            if t.array == "ALGEBRAIC":
                if t.name in pr.defined:
                    out.append(f"{indent}a_{t.name} = {rhs};")
                else:
                    out.append(f"{indent}R a_{t.name} = {rhs};")
                    pr.defined.add(t.name)
            elif t.array == "RATES":
                out.append(f"{indent}dydt[S_{t.name}] = {rhs};")
            elif t.array == "CONSTANTS":
                out.append(f"{indent}C[C_{t.name}] = {rhs};")
            elif t.array == "STATES":
                out.append(f"{indent}y[S_{t.name}] = {rhs};")
        elif isinstance(st, If):
            out.append(f"{indent}if ({pr(st.cond)}) {{")
            _cuda_body(m, st.then, pr, indent + "    ", out)
            if st.orelse:
                out.append(f"{indent}}} else {{")
                _cuda_body(m, st.orelse, pr, indent + "    ", out)
            out.append(f"{indent}}}")
        elif isinstance(st, Fatal):
            out.append(f"{indent}/* unsupported configuration in the reference */")


class _TissuePrinter(_CudaPrinter):
    """The right-hand side of tissue mode with the membrane-potential-only
    algebraics read from the per-cell values H (see hoist.py); a read before
    such an algebraic's assignment is the zeroed scratch, as in the body."""

    def __init__(self, m: Model, early: List[str], invariant, needed, recip=frozenset()):
        super().__init__(m, early, "rhs")
        self.invariant = set(invariant)
        self.needed = list(needed)
        self.hoisted_defined = set()
        self.subtrees: Dict[Node, int] = {}   # expression -> its slot after `needed`
        # slots read only as divisors hold their reciprocal (cfg_hrcp) and
        # are read through cfg_hdiv; the first pass counts the uses
        self.recip = set(recip)
        self.div_uses: Dict[str, int] = {}
        self.other_uses: Dict[str, int] = {}

    def _slot(self, e: Node):
        """The H slot an expression reads, or None."""
        if isinstance(e, Ref) and e.array == "ALGEBRAIC" and e.name in self.invariant:
            return f"H_{e.name}" if e.name in self.hoisted_defined else None
        if self._extractable(e):
            k = self.subtrees.setdefault(e, len(self.subtrees))
            return str(len(self.needed) + k)
        return None

    def _extractable(self, e: Node) -> bool:
        """A subexpression of a statement that depends on the membrane
        potential and constants alone and holds a special function: its
        value is the same at every stage, so H keeps it too."""
        if isinstance(e, (Num, Ref, Var)):
            return False
        special = False
        for n in walk(e):
            if isinstance(n, Var) and n.name not in ("tissueFlag", "dimension"):
                return False
            if isinstance(n, Call):
                if n.fn == "computeIstim":
                    return False
                if n.fn in ("exp", "log", "sqrt", "tanh") or (
                        n.fn == "pow" and _int_exponent(n.args[1]) is None):
                    special = True
            if isinstance(n, Ref):
                if n.array == "STATES" and n.name != self.m.states[0]:
                    return False
                if n.array == "RATES":
                    return False
                if n.array == "ALGEBRAIC" and (n.name not in self.invariant or
                                               n.name not in self.hoisted_defined):
                    return False
        return special

    def __call__(self, e: Node) -> str:
        if isinstance(e, Bin) and e.op == "/":
            slot = self._slot(e.r)
            if slot is not None:
                self.div_uses[slot] = self.div_uses.get(slot, 0) + 1
                if slot in self.recip:
                    return f"cfg_hdiv({self(e.l)}, H({slot}))"
                return f"({self(e.l)} / H({slot}))"
        slot = self._slot(e) if not isinstance(e, Ref) else None
        if slot is not None:
            self.other_uses[slot] = self.other_uses.get(slot, 0) + 1
            return f"H({slot})"
        return super().__call__(e)

    def ref(self, r: Ref) -> str:
        if r.array == "ALGEBRAIC" and r.name in self.invariant:
            if r.name not in self.hoisted_defined:
                return "R(0)"
            slot = f"H_{r.name}"
            self.other_uses[slot] = self.other_uses.get(slot, 0) + 1
            return f"H({slot})"
        return super().ref(r)


def _cuda_body_tissue(m: Model, stmts, pr: _TissuePrinter, indent: str, out: List[str]):
    """The body without the invariant assignments (whose values H holds)."""
    inv = pr.invariant
    for st in stmts:
        if isinstance(st, Assign):
            if st.target.array == "ALGEBRAIC" and st.target.name in inv:
                pr.hoisted_defined.add(st.target.name)
                continue
            _cuda_body(m, [st], pr, indent, out)
        elif isinstance(st, If):
            assigns = list(iter_assigns([st]))
            if all(a.target.array == "ALGEBRAIC" and a.target.name in inv for a in assigns):
                pr.hoisted_defined.update(a.target.name for a in assigns)
                continue
            out.append(f"{indent}if ({pr(st.cond)}) {{")
            _cuda_body_tissue(m, st.then, pr, indent + "    ", out)
            if st.orelse:
                out.append(f"{indent}}} else {{")
                _cuda_body_tissue(m, st.orelse, pr, indent + "    ", out)
            out.append(f"{indent}}}")
        elif isinstance(st, Fatal):
            out.append(f"{indent}/* unsupported configuration in the reference */")


def tissue_subtrees(m: Model) -> List[Node]:
    """The special-function subexpressions rhs_tissue() reads from H."""
    from .hoist import analyse
    h = analyse(m, m.rates)
    if not h.needed:
        return []
    pr = _TissuePrinter(m, use_before_def(m.rates), h.invariant, h.needed)
    _cuda_body_tissue(m, m.rates, pr, "    ", [])
    return [e for e, _ in sorted(pr.subtrees.items(), key=lambda kv: kv[1])]


def _emit_tissue_rhs(m: Model, L: List[str]):
    """hoist() and rhs_tissue(): the right-hand side of tissue mode split into
    its membrane-potential-only part, evaluated once per cell and PDE step,
    and the rest, evaluated at every RKF45 stage."""
    from .hoist import analyse, invariant_statements
    h = analyse(m, m.rates)
    vm = m.states[0]
    # the rest of the body first: it finds the subexpressions H also keeps
    rest: List[str] = []
    subtrees: Dict[Node, int] = {}
    recip: set = set()

    def print_rest(recip_slots):
        pr = _TissuePrinter(m, use_before_def(m.rates), h.invariant, h.needed, recip_slots)
        body = []
        for name in _predeclare_conditional_algebraics(m, m.rates, body, "    "):
            if name in h.invariant:
                continue
            body.append(f"    R a_{name} = R(0);")
            pr.defined.add(name)
        _cuda_body_tissue(m, m.rates, pr, "    ", body)
        return pr, body

    if h.needed:
        # pass 1 finds the slots read only as divisors, pass 2 prints
        pr, _ = print_rest(frozenset())
        recip = {k for k in pr.div_uses if k not in pr.other_uses}
        recip.discard(f"H_{m.iion_name}")
        pr, body = print_rest(frozenset(recip))
        rest.extend(_state_loads(m, pr))
        rest.extend(body)
        if m.iion_name in h.invariant:
            rest.append(f"    return H(H_{m.iion_name});")
        else:
            rest.append(f"    return a_{m.iion_name};")
        subtrees = pr.subtrees
    nh = len(h.needed) + len(subtrees)
    L.append("// Tissue mode (solveVmWithinODESolver false): the PDE owns the membrane")
    L.append("// potential, so state 0 is the same at every RKF45 stage of a PDE step and")
    L.append("// the algebraics computed from it and constants alone are too.  hoist()")
    L.append("// evaluates the ones the rest of the body reads, and the special-function")
    L.append("// subexpressions of the rest that depend on state 0 and constants alone,")
    L.append("// once per cell and step into H[NH]; rhs_tissue() is the body without them,")
    L.append("// reading H (the same expressions in the same order: bitwise the values")
    L.append("// of rhs() in FP64).")
    L.append(f"constexpr int NH = {nh};")
    if h.needed:
        L.append("enum Hoisted { " + ", ".join(f"H_{a}" for a in h.needed) + " };")
    L.append("template <class R, class KS>")
    L.append(f"__device__ __forceinline__ void hoist(R y_{vm}, const KS& K, int tissue, R* H)")
    L.append("{")
    L.append(f"    (void)tissue; (void)K; (void)H; (void)y_{vm};")
    if h.needed:
        stmts = invariant_statements(m.rates, h.invariant)
        pr = _CudaPrinter(m, [], "rhs")
        body = []
        for name in _predeclare_conditional_algebraics(m, stmts, body, "    "):
            body.append(f"    R a_{name} = R(0);")
            pr.defined.add(name)
        _cuda_body(m, stmts, pr, "    ", body)
        for a in h.needed:
            v = f"cfg_hrcp(a_{a})" if f"H_{a}" in recip else f"a_{a}"
            body.append(f"    H[H_{a}] = {v};")
        for e, k in sorted(subtrees.items(), key=lambda kv: kv[1]):
            slot = str(len(h.needed) + k)
            v = f"cfg_hrcp({pr(e)})" if slot in recip else pr(e)
            body.append(f"    H[{slot}] = {v};")
        if set(pr.states_read) - {vm}:
            raise ValueError(f"{m.name}: hoisted statements read {pr.states_read}")
        L.extend(body)
    L.append("}")
    L.append("template <class R, class YS, class KS, class HS>")
    L.append("__device__ __forceinline__ R rhs_tissue(double t, const YS& Y, const KS& K, "
             "const HS& H, R* dydt, int tissue, const CfgStimulus& stim)")
    L.append("{")
    if not h.needed:
        L.append("    (void)H;")
        L.append("    return rhs<R, false>(t, Y, K, dydt, tissue, stim);")
        L.append("}")
        return h
    L.append("    constexpr bool SOLVE_VM = false;")
    L.append("    (void)tissue; (void)stim; (void)t; (void)H;")
    L.extend(rest)
    L.append("}")
    return h


def _state_loads(m: Model, pr: "_CudaPrinter") -> List[str]:
    """Every state the body reads, loaded once before any derivative is
    written: the stores to dydt then cannot force reloads (the compiler must
    assume dydt may alias the state array), and the loads can be scheduled
    early."""
    return [f"    const R y_{s} = Y(S_{s});" for s in m.states if s in pr.states_read]


def _predeclare_conditional_algebraics(m: Model, stmts, out, indent):
    """Algebraics first assigned inside an if-block need a declaration outside."""
    inside = set()
    def visit(body, depth):
        for st in body:
            if isinstance(st, If):
                visit(st.then, depth + 1)
                visit(st.orelse, depth + 1)
            elif isinstance(st, Assign) and depth > 0 and st.target.array == "ALGEBRAIC":
                inside.add(st.target.name)
    visit(stmts, 0)
    return sorted(inside)


def constant_values(m: Model, tissue: int) -> List[float]:
    """initConsts (plus the supplement) evaluated with IEEE double arithmetic
    for one tissue flag; the order of operations is the header's, and exp/log/
    pow/sqrt come from the C library as in the reference."""
    from .opcount import _Eval
    ev = _Eval(m, {}, {}, tissue)
    ev.run(m.init, "init")
    out = []
    for c in m.constants:
        v = ev.C.get(c, 0.0)
        out.append(float(v))
    for c, expr in supplement_for(m):
        out[m.constants.index(c)] = float(eval(expr))
    return out


def _cxx_double(v: float) -> str:
    if v != v:
        return "__builtin_nan(\"\")"
    if v in (float("inf"), float("-inf")):
        return ("-" if v < 0 else "") + "__builtin_huge_val()"
    r = repr(float(v))
    return r if ("e" in r or "." in r or "inf" in r) else r + ".0"


def emit_cuda(m: Model, src_rel: str) -> str:
    ns = ident(m.name)
    L: List[str] = []
    L.append(f"// Generated by cardiacfoam_gb300.cellml2cuda from {src_rel}.")
    L.append("// The equations are the published cell model as cellML2foam wrote them;")
    L.append("// regenerate with `python -m cardiacfoam_gb300.cellml2cuda` instead of editing.")
    L.append("#pragma once")
    L.append('#include "../ionic_common.cuh"')
    L.append("")
    L.append(f"namespace cfg {{ namespace {ns} {{")
    L.append("")
    L.append(f"constexpr int NS = {len(m.states)};")
    L.append(f"constexpr int NC = {len(m.constants)};")
    L.append(f"constexpr int NA = {len(m.algebraic)};")
    L.append("enum State { " + ", ".join(f"S_{s}" for s in m.states) + " };")
    L.append("enum Constant { " + ", ".join(f"C_{c}" for c in m.constants) + " };")
    wide = WIDE_STATES[m.name]
    mask = 0
    for s in wide:
        mask |= 1 << m.states.index(s)
    L.append(f"// states kept in double in the mixed form (bit i = state i)")
    L.append(f"constexpr unsigned long long WIDE_MASK = 0x{mask:x}ull;")
    L.append(f"constexpr double IION_SCALE = {m.iion_scale!r};")
    L.append(f"constexpr double TIME_SCALE = {m.time_scale!r};")
    L.append(f'constexpr int VM_MAP = CFG_VM_{m.vm_to_state.upper()};')
    tis = [TISSUE_FLAGS[t] for t in m.tissues]
    L.append("constexpr int N_TISSUES = %d;" % len(tis))
    L.append("static const int TISSUES[] = {" + ", ".join(str(t) for t in tis) + ", 0};")
    L.append("using TissueSet = TissueList<" + ", ".join(str(t) for t in tis) + ">;")
    L.append("static const char* const STATE_NAMES[NS] = {" +
             ", ".join(f'"{s}"' for s in m.states) + "};")
    L.append("CFG_HD inline bool tissue_supported(int t) { return " +
             " || ".join(f"t == {t}" for t in tis) + "; }")
    L.append("")
    # scalable constants
    sc = SCALABLE[m.name]
    L.append("// per-cell conductance scales: index into the scale vector, or -1")
    for k in SCALE_ORDER:
        L.append(f"constexpr int SCALE_{k} = {SCALE_ORDER.index(k) if k in sc else -1};")
    L.append("")
    # constants that depend on the scales
    sd = scale_dependent_constants(m)
    L.append("// Constants that depend on the per-cell conductance scales and that the")
    L.append("// right-hand side reads: the scaled conductances and every constant")
    L.append("// initConsts derives from them.  sd_slot(i) is constant i's index in a")
    L.append("// cell's vector of them, or -1 (then the constant is the tissue's).")
    L.append(f"constexpr int NSD = {len(sd)};")
    L.append("CFG_HD constexpr int sd_const(int k)")
    L.append("{")
    L.append("    switch (k) {")
    for k, c in enumerate(sd):
        L.append(f"    case {k}: return C_{c};")
    L.append("    default: return -1;")
    L.append("    }")
    L.append("}")
    L.append("CFG_HD constexpr int sd_slot(int i)")
    L.append("{")
    L.append("    switch (i) {")
    for k, c in enumerate(sd):
        L.append(f"    case C_{c}: return {k};")
    L.append("    default: return -1;")
    L.append("    }")
    L.append("}")
    ca = CALCIUM_STATE.get(m.name)
    L.append("// intracellular calcium state (peak Ca of a beat), or -1")
    L.append(f"constexpr int CA_STATE = {('S_' + ca) if ca else -1};")
    L.append("")
    # init
    L.append("// Constants and initial states (initConsts).  `scale` may be null;")
    L.append("// otherwise scale[SCALE_x] multiplies the named conductance right after")
    L.append("// it is assigned, before constants derived from it are computed.")
    L.append("CFG_HD __forceinline__ void init_consts(double* C, double* y, int tissue, "
             "const double* scale)")
    L.append("{")
    L.append("    (void)tissue; (void)scale;")
    pr = _CudaPrinter(m, [], "init")
    inv = {v: k for k, v in sc.items()}
    body: List[str] = []
    for st in m.init:
        _cuda_body(m, [st], pr, "    ", body)
        if isinstance(st, Assign) and st.target.array == "CONSTANTS" and st.target.name in inv:
            body.append(f"    if (scale) C[C_{st.target.name}] *= "
                        f"scale[SCALE_{inv[st.target.name]}];")
    L.extend(body)
    sup = supplement_for(m)
    if sup:
        L.append("    // constants the generated initConsts leaves unset (see the emitter's")
        L.append("    // SUPPLEMENT table for their source)")
        for c, v in sup:
            L.append(f"    C[C_{c}] = {v};")
    L.append("}")
    L.append("")
    # per-tissue constant tables, folded into the kernels as immediates
    L.append("// initConsts evaluated per tissue flag (IEEE double, the header's order of")
    L.append("// operations): cval<T>(i) is constant i for tissue T.  Kernels for one uniform")
    L.append("// tissue without per-cell scales read constants from here, so the compiler")
    L.append("// folds them into the instructions.")
    L.append("template <int T> CFG_HD constexpr double cval(int i);")
    for t in tis:
        vals = constant_values(m, t)
        L.append(f"template <> CFG_HD constexpr double cval<{t}>(int i)")
        L.append("{")
        L.append("    switch (i) {")
        for k, v in enumerate(vals):
            L.append(f"    case {k}: return {_cxx_double(v)};")
        L.append("    default: return 0.0;")
        L.append("    }")
        L.append("}")
    L.append("")
    # rhs
    early = use_before_def(m.rates)
    L.append("// Right-hand side as used by derivatives(): dydt for every state that the")
    L.append("// reference assigns (RATES of V only when SOLVE_VM).  Returns Iion.")
    L.append("// Y(i) reads state i as R (each state once, before any dydt store),")
    L.append("// K(i) reads constant i as R.")
    L.append("template <class R, bool SOLVE_VM, class YS, class KS>")
    L.append("__device__ __forceinline__ R rhs(double t, const YS& Y, const KS& K, R* dydt, "
             "int tissue, const CfgStimulus& stim)")
    L.append("{")
    L.append("    (void)tissue; (void)stim; (void)t;")
    pr = _CudaPrinter(m, early, "rhs")
    body = []
    for name in _predeclare_conditional_algebraics(m, m.rates, body, "    "):
        body.append(f"    R a_{name} = R(0);")
        pr.defined.add(name)
    _cuda_body(m, m.rates, pr, "    ", body)
    L.extend(_state_loads(m, pr))
    L.extend(body)
    L.append(f"    return a_{m.iion_name};")
    L.append("}")
    L.append("")
    _emit_tissue_rhs(m, L)
    L.append("")
    # iion at end of step (the variables body); last Iion assignment wins
    L.append("// Ionic current after the step (computeVariables at tEnd).")
    L.append("template <class R, bool SOLVE_VM, class YS, class KS>")
    L.append("__device__ __forceinline__ R iion(double t, const YS& Y, const KS& K, int tissue, "
             "const CfgStimulus& stim)")
    L.append("{")
    L.append("    (void)tissue; (void)stim; (void)t;")
    L.append("    R dydt[NS];")
    pr = _CudaPrinter(m, use_before_def(m.variables), "rhs")
    body = []
    for name in _predeclare_conditional_algebraics(m, m.variables, body, "    "):
        body.append(f"    R a_{name} = R(0);")
        pr.defined.add(name)
    _cuda_body(m, m.variables, pr, "    ", body)
    L.extend(_state_loads(m, pr))
    L.extend(body)
    L.append("    (void)dydt;")
    L.append(f"    return a_{m.iion_name};")
    L.append("}")
    L.append("")
    # every algebraic of the sweep body (sweepCurrent)
    L.append("// computeVariables with every algebraic stored: A[k] is ALGEBRAIC[k] (0 for")
    L.append("// the ones the body does not assign), dydt the RATES it assigns.")
    L.append("template <class R, bool SOLVE_VM, class YS, class KS>")
    L.append("__device__ __forceinline__ void variables_all(double t, const YS& Y, const KS& K, "
             "R* A, R* dydt, int tissue, const CfgStimulus& stim)")
    L.append("{")
    L.append("    (void)tissue; (void)stim; (void)t;")
    pr = _CudaPrinter(m, use_before_def(m.sweep_body), "rhs")
    body = []
    for name in _predeclare_conditional_algebraics(m, m.sweep_body, body, "    "):
        body.append(f"    R a_{name} = R(0);")
        pr.defined.add(name)
    _cuda_body(m, m.sweep_body, pr, "    ", body)
    L.extend(_state_loads(m, pr))
    L.extend(body)
    for k, a in enumerate(m.algebraic):
        if a in pr.defined:
            L.append(f"    A[{k}] = a_{a};")
    L.append("}")
    L.append("")
    # the reference's name tables and sweepCurrent dependency map
    def strtab(name, items, n):
        items = list(items) + [""] * max(0, n - len(items))
        L.append(f"static const char* const {name}[{max(1, n)}] = {{" +
                 (", ".join(f'"{x}"' for x in items[:n]) if n else '""') + "};")
    L.append("// STATES_NAMES / ALGEBRAIC_NAMES as the header spells them; matched by")
    L.append("// position, entries the header leaves out are empty")
    strtab("STATE_STRINGS", m.state_strings, len(m.states))
    strtab("ALG_STRINGS", m.alg_strings, len(m.algebraic))
    L.append("// <Model>DependencyMap(): current -> comma-separated variables, null-ended")
    L.append("static const char* const SWEEP_CURRENTS[] = {" +
             "".join(f'"{k}", ' for k, _ in m.sweep_deps) + "nullptr};")
    L.append("static const char* const SWEEP_DEPS[] = {" +
             "".join('"' + ",".join(v) + '", ' for _, v in m.sweep_deps) + "nullptr};")
    L.append("")
    L.append("// traits bundle used by the kernel templates")
    L.append("struct Model {")
    L.append("    static constexpr int NS = " + ns + "::NS, NC = " + ns + "::NC;")
    L.append("    static constexpr unsigned long long WIDE_MASK = " + ns + "::WIDE_MASK;")
    L.append("    static constexpr double IION_SCALE = " + ns + "::IION_SCALE;")
    L.append("    static constexpr double TIME_SCALE = " + ns + "::TIME_SCALE;")
    L.append("    static constexpr int VM_MAP = " + ns + "::VM_MAP;")
    L.append("    CFG_HD static __forceinline__ void init(double* C, double* y, int tissue, "
             "const double* scale) { init_consts(C, y, tissue, scale); }")
    L.append("    template <int T> CFG_HD static constexpr double constant(int i) "
             "{ return cval<T>(i); }")
    L.append("    static constexpr int NSD = " + ns + "::NSD, CA_STATE = " + ns + "::CA_STATE;")
    L.append("    static constexpr int NH = " + ns + "::NH;")
    L.append("    template <class R, class KS>")
    L.append("    __device__ static __forceinline__ void hoist_vm(R v, const KS& K, int tissue, "
             "R* H) { hoist<R>(v, K, tissue, H); }")
    L.append("    template <class R, class YS, class KS, class HS>")
    L.append("    __device__ static __forceinline__ R rates_tissue(double t, const YS& Y, "
             "const KS& K, const HS& H, R* dydt, int tissue, const CfgStimulus& st) "
             "{ return rhs_tissue<R>(t, Y, K, H, dydt, tissue, st); }")
    L.append("    CFG_HD static constexpr int sd_slot(int i) { return " + ns + "::sd_slot(i); }")
    L.append("    static constexpr int NA = " + ns + "::NA;")
    L.append("    template <class R, bool SV, class YS, class KS>")
    L.append("    __device__ static __forceinline__ void all_variables(double t, const YS& Y, "
             "const KS& K, R* A, R* dydt, int tissue, const CfgStimulus& st) "
             "{ variables_all<R, SV>(t, Y, K, A, dydt, tissue, st); }")
    L.append("    CFG_HD static constexpr int sd_const(int k) { return " + ns + "::sd_const(k); }")
    L.append("    template <class R, bool SV, class YS, class KS>")
    L.append("    __device__ static __forceinline__ R rates(double t, const YS& Y, const KS& K, "
             "R* dydt, int tissue, const CfgStimulus& st) { return rhs<R, SV>(t, Y, K, dydt, "
             "tissue, st); }")
    L.append("    template <class R, bool SV, class YS, class KS>")
    L.append("    __device__ static __forceinline__ R current(double t, const YS& Y, const KS& K, "
             "int tissue, const CfgStimulus& st) { return iion<R, SV>(t, Y, K, tissue, st); }")
    L.append("};")
    L.append("")
    L.append(f"}} }}  // namespace cfg::{ns}")
    return "\n".join(L) + "\n"


# --------------------------------------------------------------------------
# plain C for the oracle


class _CPrinter(_Printer):
    def __init__(self, m: Model, pre: str):
        super().__init__(m)
        self.pre = pre

    def num(self, n: Num) -> str:
        return n.text

    def ref(self, r: Ref) -> str:
        arr = {"STATES": "STATES", "CONSTANTS": "CONSTANTS", "ALGEBRAIC": "ALGEBRAIC",
               "RATES": "RATES"}[r.array]
        kind = {"STATES": "S", "CONSTANTS": "C", "ALGEBRAIC": "A", "RATES": "S"}[r.array]
        return f"{arr}[{self.pre}_{kind}_{r.name}]"

    def var(self, v: Var) -> str:
        return {"tissueFlag": "tissueFlag", "VOI": "VOI", "dimension": "(tissueFlag - 10)",
                "solveVmWithinODESolver": "solveVm"}[v.name]

    def call(self, c: Call) -> str:
        if c.fn == "computeIstim":
            return "oracle_stimulus_current(VOI, stim)"
        args = ", ".join(self(x) for x in c.args)
        if c.fn == "heaviside":
            return f"oracle_heaviside({args})"
        if c.fn == "tissueSelect":
            return f"oracle_tissue_select({args})"
        if c.fn in ("exp", "log", "pow", "sqrt", "tanh", "fabs", "floor"):
            return f"{c.fn}({args})"
        raise ValueError(c.fn)


def _c_body(stmts, pr: _CPrinter, indent, out):
    for st in stmts:
        if isinstance(st, Assign):
            out.append(f"{indent}{pr.ref(st.target)} = {pr(st.expr)};")
        elif isinstance(st, If):
            out.append(f"{indent}if ({pr(st.cond)}) {{")
            _c_body(st.then, pr, indent + "    ", out)
            if st.orelse:
                out.append(f"{indent}}} else {{")
                _c_body(st.orelse, pr, indent + "    ", out)
            out.append(f"{indent}}}")
        elif isinstance(st, Fatal):
            out.append(f"{indent}oracle_fatal(\"unsupported configuration\");")


def emit_c(m: Model, src_rel: str) -> str:
    pre = ident(m.name).upper()
    fn = ident(m.name)
    L: List[str] = []
    L.append(f"/* Generated by cardiacfoam_gb300.cellml2cuda from {src_rel}.")
    L.append(" * Oracle form: reference calling convention and evaluation order, pow kept")
    L.append(" * as written.  Test infrastructure only; the product uses the CUDA form. */")
    L.append(f"#ifndef ORACLE_MODEL_{pre}_H")
    L.append(f"#define ORACLE_MODEL_{pre}_H")
    L.append('#include "../oracle_common.h"')
    L.append("")
    L.append(f"enum {{ {pre}_NS = {len(m.states)}, {pre}_NA = {len(m.algebraic)}, "
             f"{pre}_NC = {len(m.constants)} }};")
    L.append("enum { " + ", ".join(f"{pre}_S_{s}" for s in m.states) + " };")
    L.append("enum { " + ", ".join(f"{pre}_A_{s}" for s in m.algebraic) + " };")
    L.append("enum { " + ", ".join(f"{pre}_C_{s}" for s in m.constants) + " };")
    L.append(f"static const char* const {pre}_STATE_NAMES[] = {{ " +
             ", ".join(f'"{s}"' for s in m.states) + " };")
    L.append("")
    sc = SCALABLE[m.name]
    inv = {v: k for k, v in sc.items()}
    L.append(f"static void {fn}_init(double* CONSTANTS, double* STATES, int tissueFlag, "
             "const double* scale)")
    L.append("{")
    L.append("    (void)tissueFlag; (void)scale;")
    pr = _CPrinter(m, pre)
    for st in m.init:
        body: List[str] = []
        _c_body([st], pr, "    ", body)
        L.extend(body)
        if isinstance(st, Assign) and st.target.array == "CONSTANTS" and st.target.name in inv:
            L.append(f"    if (scale) CONSTANTS[{pre}_C_{st.target.name}] *= "
                     f"scale[{SCALE_ORDER.index(inv[st.target.name])}];")
    L.append("}")
    L.append("")
    sup = supplement_for(m)
    L.append(f"/* constants {fn}_init leaves unset; NULL-equivalent when none */")
    L.append(f"static void {fn}_supplement(double* CONSTANTS)")
    L.append("{")
    L.append("    (void)CONSTANTS;")
    for c, v in sup:
        L.append(f"    CONSTANTS[{pre}_C_{c}] = {v};")
    L.append("}")
    L.append("")
    for tag, stmts in (("rates", m.rates), ("variables", m.variables)):
        L.append(f"static void {fn}_{tag}(double VOI, const double* CONSTANTS, double* RATES, "
                 "const double* STATES, double* ALGEBRAIC, int tissueFlag, int solveVm, "
                 "const oracle_stimulus* stim)")
        L.append("{")
        L.append("    (void)tissueFlag; (void)solveVm; (void)stim;")
        body = []
        _c_body(stmts, pr, "    ", body)
        L.extend(body)
        L.append("}")
        L.append("")
    L.append(f"#define {pre}_IION_INDEX {pre}_A_{m.iion_name}")
    L.append(f"#define {pre}_IION_SCALE {m.iion_scale!r}")
    L.append(f"#define {pre}_TIME_SCALE {m.time_scale!r}")
    L.append("#endif")
    return "\n".join(L) + "\n"
