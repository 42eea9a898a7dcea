"""Read a cellML2foam-generated ionic model header into an intermediate form.

Input: the pair ``<Model>_<Year>.H`` / ``<Model>_<Year>Names.H`` that
``applications/scripts/cellML2foam`` writes for each model under
``src/ionicModels/<Model>/``.  The header holds three kinds of functions:

* ``<Model>initConsts(CONSTANTS, RATES, STATES, tissueFlag, dict)`` - constants
  and initial states (``TNNP_2004.H:310-383``, ``ORd_2011.H:494-692``,
  ``ToRORd_dynCl_2023.H:571-846``, ``AlievPanfilov_1996.H:73-92``);
* ``<Model>computeRates(...)`` (TNNP only, ``TNNP_2004.H:386-509``) - the RHS
  used by ``TNNP::derivatives`` (``TNNP.C:181-203``);
* ``<Model>computeVariables(...)`` - algebraics incl. ``Iion_cm`` (and, for all
  models except TNNP, the RATES as well).

The result is a :class:`Model` holding ordered statement lists whose
expressions are :mod:`cexpr` trees.  The emitters in :mod:`emit` turn those
into CUDA device functions (templated on precision) and into the plain-C
functions the CPU oracle uses.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from pathlib import Path
from typing import List, Optional, Union

from .cexpr import Node, Ref, Var, parse_expr, refs, ParseError


@dataclass
class Assign:
    target: Ref
    expr: Node
    line: int = 0          # 1-based line in the source header


@dataclass
class If:
    cond: Node
    then: List["Stmt"]
    orelse: List["Stmt"] = field(default_factory=list)
    line: int = 0


@dataclass
class Fatal:
    line: int = 0


Stmt = Union[Assign, If, Fatal]


@dataclass
class Model:
    name: str                       # class name, e.g. "TNNP"
    header: str                     # header file name, e.g. "TNNP_2004.H"
    states: List[str]
    algebraic: List[str]
    constants: List[str]
    init: List[Stmt]
    rates: List[Stmt]               # body used by derivatives()
    variables: List[Stmt]           # body(ies) used after the ODE solve, in call order
    tissues: List[str]              # supportedTissueTypes()
    vm_to_state: str = "mV"         # how the PDE Vm [V] maps to STATES[0]
    iion_name: str = "Iion_cm"
    iion_scale: float = 1.0         # Im = scale * ALGEBRAIC[iion]
    time_scale: float = 1.0         # model time = t[s] * 1000 / time_scale
    extra_args: List[str] = field(default_factory=list)
    # the header's string tables (ALGEBRAIC_NAMES may differ from the enum:
    # entries are matched by position, as ionicModelIO does) and the
    # <Model>DependencyMap() of sweepCurrent: (current, [variable names])
    state_strings: List[str] = field(default_factory=list)
    alg_strings: List[str] = field(default_factory=list)
    sweep_deps: List = field(default_factory=list)
    # the body sweepCurrent evaluates (the first variables function only,
    # e.g. TNNP.C:250-261 calls TNNPcomputeVariables without computeRates)
    sweep_body: List[Stmt] = field(default_factory=list)

    def state_index(self, n: str) -> int:
        return self.states.index(n)


# --------------------------------------------------------------------------
# source scanning helpers

def _strip_comments(src: str) -> str:
    """Blank out // and /* */ comments, keeping line structure and offsets."""
    out = []
    i, n = 0, len(src)
    in_str = False
    while i < n:
        c = src[i]
        if in_str:
            out.append(c)
            if c == "\\" and i + 1 < n:
                out.append(src[i + 1])
                i += 2
                continue
            if c == '"':
                in_str = False
            i += 1
            continue
        if c == '"':
            in_str = True
            out.append(c)
            i += 1
            continue
        if src.startswith("//", i):
            j = src.find("\n", i)
            j = n if j < 0 else j
            out.append(" " * (j - i))
            i = j
            continue
        if src.startswith("/*", i):
            j = src.find("*/", i + 2)
            j = n if j < 0 else j + 2
            out.append("".join(ch if ch == "\n" else " " for ch in src[i:j]))
            i = j
            continue
        out.append(c)
        i += 1
    return "".join(out)


def _enum_names(text: str, *enum_names: str) -> List[str]:
    for en in enum_names:
        m = re.search(r"enum\s+(?:\w+_)?" + en + r"\s*\{(.*?)\}", text, re.S)
        if m:
            names = []
            for item in m.group(1).split(","):
                item = item.strip()
                if not item:
                    continue
                nm = item.split("=")[0].strip()
                if nm.startswith("NUM_") or "_NUM_" in nm:
                    continue
                names.append(nm)
            return names
    raise ParseError(f"enum {enum_names} not found")


def _function_body(text: str, fname: str):
    """Return (body_text, body_start_offset) of the function named fname."""
    m = re.search(r"\b" + re.escape(fname) + r"\s*\(", text)
    if not m:
        return None, -1
    # skip the parameter list
    depth, i = 0, m.end() - 1
    while True:
        if text[i] == "(":
            depth += 1
        elif text[i] == ")":
            depth -= 1
            if depth == 0:
                break
        i += 1
    j = text.index("{", i)
    depth, k = 0, j
    while True:
        if text[k] == "{":
            depth += 1
        elif text[k] == "}":
            depth -= 1
            if depth == 0:
                break
        k += 1
    return text[j + 1:k], j + 1


class _StmtParser:
    """Statement-level parser for the function bodies (assignments and ifs)."""

    def __init__(self, body: str, base_line: int):
        self.s = body
        self.i = 0
        self.base_line = base_line

    def line(self) -> int:
        return self.base_line + self.s.count("\n", 0, self.i)

    def ws(self):
        while self.i < len(self.s) and self.s[self.i] in " \t\r\n":
            self.i += 1

    def at_end(self) -> bool:
        self.ws()
        return self.i >= len(self.s)

    def _balanced(self, open_c: str, close_c: str) -> str:
        assert self.s[self.i] == open_c
        depth, j = 0, self.i
        while True:
            if self.s[j] == open_c:
                depth += 1
            elif self.s[j] == close_c:
                depth -= 1
                if depth == 0:
                    break
            j += 1
        inner = self.s[self.i + 1:j]
        self.i = j + 1
        return inner

    def block(self) -> List[Stmt]:
        self.ws()
        if self.s[self.i] == "{":
            start_line = self.line()
            inner = self._balanced("{", "}")
            return _StmtParser(inner, start_line).stmts()
        return [self.stmt()]

    def stmt(self) -> Optional[Stmt]:
        self.ws()
        ln = self.line()
        if re.match(r"if\b", self.s[self.i:]):
            self.i += 2
            self.ws()
            cond = parse_expr(self._balanced("(", ")"))
            then = self.block()
            self.ws()
            orelse: List[Stmt] = []
            if re.match(r"else\b", self.s[self.i:]):
                self.i += 4
                orelse = self.block()
            return If(cond, then, orelse, ln)
        j = self.s.index(";", self.i)
        text = self.s[self.i:j].strip()
        self.i = j + 1
        if not text or text.startswith("using "):
            return None
        if text.startswith("FatalError"):
            return Fatal(ln)
        m = re.fullmatch(r"(\w+)\s*\[\s*(\w+)\s*\]\s*=(.*)", text, re.S)
        if not m:
            raise ParseError(f"unsupported statement at line {ln}: {text[:80]!r}")
        return Assign(Ref(m.group(1), m.group(2)), parse_expr(m.group(3)), ln)

    def stmts(self) -> List[Stmt]:
        out = []
        while not self.at_end():
            if self.s[self.i] == ";":
                self.i += 1
                continue
            st = self.stmt()
            if st is not None:
                out.append(st)
        return out


def _parse_function(clean: str, fname: str) -> Optional[List[Stmt]]:
    body, off = _function_body(clean, fname)
    if body is None:
        return None
    base_line = clean.count("\n", 0, off) + 1
    return _StmtParser(body, base_line).stmts()


# --------------------------------------------------------------------------
# per-model facts that live in the hand-written wrappers (<Model>.C), not in
# the generated header.  Each entry cites the wrapper lines it restates.

WRAPPERS = {
    # TNNP.C:90-94 (tissues), 114-179 (solveODE: Vm*1000, Im = Iion_cm,
    # computeVariables then computeRates at tEnd), 181-203 (derivatives ->
    # computeRates)
    "TNNP": dict(dir="TNNP", header="TNNP_2004.H", names="TNNP_2004Names.H",
                 prefix="TNNP", rates_fn="TNNPcomputeRates",
                 variables_fns=["TNNPcomputeVariables", "TNNPcomputeRates"],
                 tissues=["endocardialCells", "mCells", "epicardialCells"],
                 vm_to_state="mV", iion_name="Iion_cm", iion_scale=1.0, time_scale=1.0),
    # ORd.C:93-96 (tissue myocyte only), 102-155 (solveODE), 157-180 (derivatives)
    "ORd": dict(dir="ORd", header="ORd_2011.H", names="ORd_2011Names.H",
                prefix="ORd", rates_fn="ORdcomputeVariables",
                variables_fns=["ORdcomputeVariables"],
                tissues=["myocyte"],
                vm_to_state="mV", iion_name="Iion_cm", iion_scale=1.0, time_scale=1.0),
    # ToRORd_dynCl.C:93-96 (tissues), 102-155 (solveODE)
    "ToRORd_dynCl": dict(dir="ToRORd_dynCl", header="ToRORd_dynCl_2023.H",
                         names="ToRORd_dynCl_2023Names.H", prefix="ToRORd_dynCl",
                         rates_fn="ToRORd_dynClcomputeVariables",
                         variables_fns=["ToRORd_dynClcomputeVariables"],
                         tissues=["endocardialCells", "mCells", "epicardialCells"],
                         vm_to_state="mV", iion_name="Iion_cm", iion_scale=1.0,
                         time_scale=1.0),
    # AlievPanfilov.C:95-97 (myocyte), 99-153 (u = (1000 Vm + 80)/100,
    # model time = t_ms/12.9, Im = 100 Iion_cm)
    "AlievPanfilov": dict(dir="AlievPanfilov", header="AlievPanfilov_1996.H",
                          names="AlievPanfilov_1996Names.H", prefix="AlievPanfilov",
                          rates_fn="AlievPanfilovcomputeVariables",
                          variables_fns=["AlievPanfilovcomputeVariables"],
                          tissues=["myocyte"],
                          vm_to_state="aliev", iion_name="Iion_cm", iion_scale=100.0,
                          time_scale=12.9),
    # BuenoOrovio.C:90-93 (tissues), 99-152 (u = (1000 Vm + 84)/85.7,
    # Im = 85.7 Jion).  Kept as the model the reference's regression tests pin.
    "BuenoOrovio": dict(dir="BuenoOrovio", header="BuenoOrovio_2008.H",
                        names="BuenoOrovio_2008Names.H", prefix="BuenoOrovio",
                        rates_fn="BuenoOroviocomputeVariables",
                        variables_fns=["BuenoOroviocomputeVariables"],
                        tissues=["endocardialCells", "mCells", "epicardialCells"],
                        vm_to_state="bueno", iion_name="Jion", iion_scale=85.7,
                        time_scale=1.0),
    # monodomainFDAManufactured.C:54-72 (dimension selects the constants),
    # 88-132 (solveODE: S[V] = Vm, model time = t [s], h = min(h, deltaT),
    # Im = Iion / Cm with Cm = 2).  The verification model of the
    # manufactured-solution convergence study.
    "monodomainFDAManufactured": dict(
        dir="monodomainFDAManufactured", header="monodomainFDAManufactured_2014.H",
        names="monodomainFDAManufactured_2014Names.H", prefix="monodomainFDAManufactured",
        init_fn="monodomainFDAManufacturedInitConsts",
        rates_fn="monodomainFDAManufacturedComputeVariables",
        variables_fns=["monodomainFDAManufacturedComputeVariables"],
        tissues=["1D", "2D", "3D"],
        vm_to_state="identity", iion_name="Iion", iion_scale=0.5, time_scale=1000.0),
    # bidomainFDAManufactured.C:47-60 (k from manufacturedBidomain.k, default
    # 1/sqrt(2); the tutorial's value is compiled in), 77 (initConsts with k),
    # solveODE as monodomainFDAManufactured.  initConsts keeps the dimension's
    # Beta in a local before scaling it by (1 - k); the rewrite keeps it in
    # the Beta constant instead, with the same arithmetic (and the casts to
    # void that mark unused parameters go).
    "bidomainFDAManufactured": dict(
        dir="bidomainFDAManufactured", header="bidomainFDAManufactured_2014.H",
        names="bidomainFDAManufactured_2014Names.H", prefix="bidomainFDAManufactured",
        init_fn="bidomainFDAManufacturedInitConsts",
        rates_fn="bidomainFDAManufacturedComputeVariables",
        variables_fns=["bidomainFDAManufacturedComputeVariables"],
        tissues=["1D", "2D", "3D"],
        vm_to_state="identity", iion_name="BidomainIion", iion_scale=0.5, time_scale=1000.0,
        rewrite=[("CONSTANTS[BidomainBeta] = betaBase*(1.0 - k);",
                  "CONSTANTS[BidomainBeta] = CONSTANTS[BidomainBeta]*(1.0 - 0.7071067811865476);"),
                 ("double betaBase = 0.0;", "CONSTANTS[BidomainBeta] = 0.0;"),
                 ("betaBase = ", "CONSTANTS[BidomainBeta] = "),
                 ("(void)VOI;", ""), ("(void)dimension;", ""),
                 ("(void)solveVmWithinODESolver;", "")]),
}
BIDOMAIN_K = 0.7071067811865476   # manufacturedBidomain.k of the bidomain tutorial


def _string_table(text: str, table: str) -> List[str]:
    m = re.search(r"(\w*)" + table + r"\s*\[[^\]]*\]\s*=\s*\{(.*?)\};", text, re.S)
    return re.findall(r'"([^"]*)"', m.group(2)) if m else []


def _dependency_map(text: str):
    """Entries of <Model>DependencyMap(): {"INa", wordList({"i_Na", ...})}."""
    body, _ = _function_body(text, next(iter(re.findall(r"\b(\w+DependencyMap)\s*\(\s*\)",
                                                         text)), "NoDependencyMap"))
    if body is None:
        return []
    out = []
    for key, items in re.findall(r'\{\s*"(\w+)"\s*,\s*Foam::wordList\s*\(\s*\{([^}]*)\}\s*\)\s*\}',
                                 body):
        out.append((key, re.findall(r'"([^"]*)"', items)))
    return out


def load_model(ionic_models_dir: Union[str, Path], name: str) -> Model:
    w = WRAPPERS[name]
    d = Path(ionic_models_dir) / w["dir"]
    names_txt = _strip_comments((d / w["names"]).read_text())
    hdr_txt = _strip_comments((d / w["header"]).read_text())
    for a, b in w.get("rewrite", []):
        if a not in hdr_txt:
            raise ParseError(f"{name}: rewrite target {a!r} not found")
        hdr_txt = hdr_txt.replace(a, b)
    states = _enum_names(names_txt, "STATES_INDEX", "STATE_INDEX")
    algebraic = _enum_names(names_txt, "ALGEBRAIC_INDEX")
    constants = _enum_names(names_txt, "CONSTANTS_INDEX", "CONSTANT_INDEX")
    init = _parse_function(hdr_txt, w.get("init_fn", w["prefix"] + "initConsts"))
    rates = _parse_function(hdr_txt, w["rates_fn"])
    variables = []
    for fn in w["variables_fns"]:
        variables.extend(_parse_function(hdr_txt, fn))
    if init is None or rates is None:
        raise ParseError(f"{name}: model functions not found in {w['header']}")
    m = Model(name=name, header=w["header"], states=states, algebraic=algebraic,
              constants=constants, init=init, rates=rates, variables=variables,
              tissues=list(w["tissues"]), vm_to_state=w["vm_to_state"],
              iion_name=w["iion_name"], iion_scale=w["iion_scale"],
              time_scale=w["time_scale"])
    raw = (d / w["header"]).read_text()
    m.state_strings = _string_table(raw, "STATES_NAMES")
    m.alg_strings = _string_table(raw, "ALGEBRAIC_NAMES")
    m.sweep_deps = _dependency_map(_strip_comments(raw))
    m.sweep_body = _parse_function(hdr_txt, w["variables_fns"][0])
    _check_names(m)
    return m


def iter_assigns(stmts: List[Stmt]):
    for st in stmts:
        if isinstance(st, Assign):
            yield st
        elif isinstance(st, If):
            yield from iter_assigns(st.then)
            yield from iter_assigns(st.orelse)


def _check_names(m: Model):
    known = {"STATES": set(m.states), "CONSTANTS": set(m.constants),
             "ALGEBRAIC": set(m.algebraic), "RATES": set(m.states)}
    for body in (m.init, m.rates, m.variables):
        for a in iter_assigns(body):
            for r in [a.target, *refs(a.expr)]:
                if r.name not in known[r.array]:
                    raise ParseError(f"{m.name}: {r.array}[{r.name}] is not declared "
                                     f"(line {a.line})")


def use_before_def(stmts: List[Stmt], array: str = "ALGEBRAIC"):
    """Names of ``array`` read before their first assignment in ``stmts``.

    In ``derivatives()`` the reference passes a freshly zeroed ALGEBRAIC array
    (e.g. ``ORd.C:167``), so such reads see 0; the emitters reproduce that.
    """
    defined, early = set(), []
    def visit(body):
        for st in body:
            if isinstance(st, Assign):
                for r in refs(st.expr, array):
                    if r.name not in defined and r.name not in early:
                        early.append(r.name)
                if st.target.array == array:
                    defined.add(st.target.name)
            elif isinstance(st, If):
                for r in refs(st.cond, array):
                    if r.name not in defined and r.name not in early:
                        early.append(r.name)
                visit(st.then)
                visit(st.orelse)
    visit(stmts)
    return early
