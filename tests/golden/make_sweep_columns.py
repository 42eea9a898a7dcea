"""Resolve every sweepCurrent dependency name of the compiled models the way
the reference does (ionicVariableCompatibility::resolveVariable,
src/genericWriter/ionicVariableCompatibility.C:37-59 and 215-275) and write
tests/golden/sweep_columns.json: model -> current -> [[source, index], ...]
with source "state", "alg" or "rate".  Reads the reference's model headers
(their STATES_NAMES / ALGEBRAIC_NAMES tables and DependencyMap); the GPU
tests read only the JSON.

    python tests/golden/make_sweep_columns.py <cardiacFoam>/src/ionicModels
"""
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from cardiacfoam_gb300.cellml2cuda.model import WRAPPERS, load_model  # noqa: E402


def canonical(raw: str) -> str:
    out = "".join(c.lower() for c in raw if c not in "_- ")
    return out[2:] if len(out) > 2 and out.startswith("av") else out


def same(a: str, b: str) -> bool:
    return a == b or canonical(a) == canonical(b)


def resolve(name, states, algs):
    if name == "Vm" or canonical(name) == "vm":
        return ["state", 0]
    for i, s in enumerate(states):
        if same(name, s):
            return ["state", i]
    for i, a in enumerate(algs):
        if a and same(name, a):
            return ["alg", i]
    if len(name) > 6 and name[:6].lower() == "rates_":
        for i, s in enumerate(states):
            if same(name[6:], s):
                return ["rate", i]
    raise KeyError(name)


def main(models_dir):
    out = {}
    for name in WRAPPERS:
        m = load_model(models_dir, name)
        states = m.state_strings + [""] * (len(m.states) - len(m.state_strings))
        algs = m.alg_strings + [""] * (len(m.algebraic) - len(m.alg_strings))
        out[name] = {cur: [resolve(d, states, algs) for d in deps] for cur, deps in m.sweep_deps}
    p = Path(__file__).parent / "sweep_columns.json"
    p.write_text(json.dumps(out, indent=0, sort_keys=True) + "\n")
    print(p, sum(len(v) for v in out.values()), "currents")


if __name__ == "__main__":
    main(sys.argv[1])
