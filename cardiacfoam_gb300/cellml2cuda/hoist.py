"""Membrane-potential-only algebraics of a right-hand side (tissue mode).

In a tissue run the PDE owns Vm: ``solveODE`` sets ``STATES[V] = 1000 Vm``
and the rates body leaves ``RATES[V]`` at zero unless
``solveVmWithinODESolver`` (e.g. ``TNNP_2004.H:493-497``,
``ORd_2011.H:984-987``), so V is the same at every RKF45 stage of the PDE
step.  Every algebraic computed from V and constants alone (gate steady
states and time constants, the GHK factors of V, ...) is then the same at all
six stages of every substep: it can be evaluated once per cell and PDE step
and read back in the stage loop.  With the same expressions evaluated in the
same order the values are bitwise those of the loop (FP64 without FMA
contraction).

:func:`analyse` returns the statement classes the emitter needs:

* ``invariant`` - algebraics all of whose assignments read only state 0,
  constants, the tissue flag and other invariant algebraics, under
  conditions of the same kind, assigned once (or once per branch of one
  if/else) and never read between assignments;
* ``needed`` - the invariant algebraics that the rest of the body (or its
  returned current) reads: the values a kernel keeps per cell.

A model whose body writes ``RATES[V]`` outside an ``if
(solveVmWithinODESolver)`` (other than a literal 0) gets no invariants.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Dict, List, Set

from .cexpr import Call, Num, Var, refs, walk
from .model import Assign, Fatal, If, Model, iter_assigns

_ALLOWED_VARS = {"tissueFlag", "dimension"}


@dataclass
class Hoisting:
    vm: str                                       # name of state 0
    invariant: Set[str] = field(default_factory=set)
    needed: List[str] = field(default_factory=list)


def _rates_v_zero_in_tissue(body, vm: str) -> bool:
    """RATES[vm] is 0 unless solveVmWithinODESolver."""
    def visit(stmts, guarded):
        for st in stmts:
            if isinstance(st, Assign):
                if st.target.array == "RATES" and st.target.name == vm:
                    if not guarded and not (isinstance(st.expr, Num) and st.expr.value == 0.0):
                        return False
            elif isinstance(st, If):
                g = guarded or (isinstance(st.cond, Var) and
                                st.cond.name == "solveVmWithinODESolver")
                if not visit(st.then, g) or not visit(st.orelse, guarded):
                    return False
        return True
    return visit(body, False)


def _expr_invariant(e, vm: str, inv: Set[str], defined: Set[str]) -> bool:
    for n in walk(e):
        if isinstance(n, Var) and n.name not in _ALLOWED_VARS:
            return False
        if isinstance(n, Call) and n.fn == "computeIstim":
            return False
    for r in refs(e):
        if r.array == "STATES" and r.name != vm:
            return False
        if r.array == "RATES":
            return False
        if r.array == "ALGEBRAIC" and (r.name not in inv or r.name not in defined):
            return False
    return True


def analyse(m: Model, body) -> Hoisting:
    vm = m.states[0]
    h = Hoisting(vm=vm)
    if not _rates_v_zero_in_tissue(body, vm):
        return h
    # assignments per algebraic, with the top-level statement they sit in
    sites: Dict[str, List[int]] = {}
    for k, st in enumerate(body):
        for a in ([st] if isinstance(st, Assign) else list(iter_assigns([st])) if
                  isinstance(st, If) else []):
            if a.target.array == "ALGEBRAIC":
                sites.setdefault(a.target.name, []).append(k)
    # one assignment, or several inside one top-level if/else
    cand = {a for a, ks in sites.items() if len(set(ks)) == 1}

    # fixed point: drop every candidate with a non-invariant assignment
    while True:
        bad = set()
        defined: Set[str] = set()

        def visit(stmts, cond_ok):
            for st in stmts:
                if isinstance(st, Assign):
                    t = st.target
                    if t.array == "ALGEBRAIC" and t.name in cand:
                        if not (cond_ok and _expr_invariant(st.expr, vm, cand, defined)):
                            bad.add(t.name)
                    if t.array == "ALGEBRAIC":
                        defined.add(t.name)
                elif isinstance(st, If):
                    ok = cond_ok and _expr_invariant(st.cond, vm, cand, defined)
                    # a name assigned in one branch is not defined in the other
                    before = set(defined)
                    visit(st.then, ok)
                    then_defined = set(defined)
                    defined.clear()
                    defined.update(before)
                    visit(st.orelse, ok)
                    defined.update(then_defined)
                elif isinstance(st, Fatal):
                    pass
        visit(body, True)
        if not bad:
            break
        cand -= bad
    # a name assigned inside an if must not be read inside that same if
    for a in list(cand):
        k = sites[a][0]
        st = body[k]
        if isinstance(st, If):
            inner = [r.name for s in iter_assigns([st]) for r in refs(s.expr, "ALGEBRAIC")]
            if a in inner:
                cand.discard(a)
    h.invariant = cand
    # invariant values read by the rest of the body or returned
    needed: List[str] = []

    def use(e):
        for r in refs(e, "ALGEBRAIC"):
            if r.name in cand and r.name not in needed:
                needed.append(r.name)

    def visit_rest(stmts, cond_inv):
        for st in stmts:
            if isinstance(st, Assign):
                if st.target.array == "ALGEBRAIC" and st.target.name in cand:
                    continue
                use(st.expr)
            elif isinstance(st, If):
                has_rest = any(not (a.target.array == "ALGEBRAIC" and a.target.name in cand)
                               for a in iter_assigns([st]))
                if has_rest:
                    use(st.cond)
                visit_rest(st.then, cond_inv)
                visit_rest(st.orelse, cond_inv)
    visit_rest(body, True)
    if m.iion_name in cand and m.iion_name not in needed:
        needed.append(m.iion_name)
    h.needed = needed
    return h


def invariant_statements(body, inv: Set[str]):
    """The statements that compute the invariant algebraics, with the if
    statements around them (and only those)."""
    out = []
    for st in body:
        if isinstance(st, Assign):
            if st.target.array == "ALGEBRAIC" and st.target.name in inv:
                out.append(st)
        elif isinstance(st, If):
            then = invariant_statements(st.then, inv)
            orelse = invariant_statements(st.orelse, inv)
            if then or orelse:
                out.append(If(st.cond, then, orelse, st.line))
    return out
