"""Generate the golden fixtures in this directory from the reference.

Run where a cardiacFoam checkout is available ($CARDIACFOAM_REFERENCE, or the
location oracle/build.py knows):

    python tests/golden/make_golden.py

* ionic_rhs_<model>.npz - right-hand sides and algebraics of the reference's
  own generated model headers (src/ionicModels/<Model>/<Model>_<Year>.H,
  compiled verbatim by oracle/ref/build_ref.sh) at seeded random states, for
  every supported tissue, with and without solveVmWithinODESolver and with an
  active single-cell stimulus.
* aliev_panfilov_singlecell.npz - the reference's single-cell trace
  tutorials/manufacturedSolutions/singleCellBidomain/postProcessing/
  AlievPanfilov_myocyte_S1_1000.txt (Vm [mV] every 5e-5 s, 7 decimals),
  stored as integers of 1e-7 mV.
* regression_pins.json - the values the reference's regression tests assert:
  tutorials/regressionTests/singleCell/singleCell.reference:2-6 and
  tutorials/regressionTests/NiedererEtAl2012/NiedererEtAl2012.reference:8-13.
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import pyoracle as po  # noqa: E402

from oracle.build import reference_dir  # noqa: E402

REF = reference_dir()
if REF is None:
    sys.exit("no cardiacFoam checkout found: set CARDIACFOAM_REFERENCE")
KEYS = {"TNNP": "tnnp", "ORd": "ord", "ToRORd_dynCl": "torord_dyncl",
        "AlievPanfilov": "alievpanfilov", "BuenoOrovio": "buenoorovio"}
TISSUES = {"TNNP": [1, 2, 3], "ORd": [4], "ToRORd_dynCl": [1, 2, 3], "AlievPanfilov": [4],
           "BuenoOrovio": [1, 2, 3]}
STIM = np.array([0.0, 10.0, 1.0, 50.0, 5.0, 0.0, 0.0])   # start, S1, dur, amp, n1, S2, n2


def random_states(model, y0, rng, n):
    ns = y0.size
    if model in ("AlievPanfilov", "BuenoOrovio"):
        return rng.uniform(0.0, 1.2, (n, ns))
    y = y0[None, :] * (1.0 + 0.2 * rng.standard_normal((n, ns)))
    y[:, 0] = rng.uniform(-95.0, 50.0, n)
    return y


def make_rhs(R, model, n=24, seed=1234):
    key = KEYS[model]
    ns, na, nc = po.sizes(model)
    rng = np.random.default_rng(seed)
    out = {}
    for tissue in TISSUES[model]:
        Cc = np.zeros(nc); Rr = np.zeros(ns); S0 = np.zeros(ns)
        getattr(R, f"ref_{key}_init")(po.ptr(Cc), po.ptr(Rr), po.ptr(S0), tissue)
        ys = random_states(model, S0, rng, n)
        ts = rng.uniform(0.0, 60.0, n)
        for sv in (0, 1):
            rates = np.zeros((n, ns)); alg = np.zeros((n, na))
            vrates = np.zeros((n, ns)); valg = np.zeros((n, na))
            for i in range(n):
                y = ys[i].copy()
                getattr(R, f"ref_{key}_rates")(ts[i], po.ptr(Cc), po.ptr(rates[i]), po.ptr(y),
                                               po.ptr(alg[i]), tissue, sv, po.ptr(STIM))
                y = ys[i].copy()
                getattr(R, f"ref_{key}_variables")(ts[i], po.ptr(Cc), po.ptr(vrates[i]),
                                                   po.ptr(y), po.ptr(valg[i]), tissue, sv,
                                                   po.ptr(STIM))
            out[f"t{tissue}_sv{sv}_rates"] = rates
            out[f"t{tissue}_sv{sv}_alg"] = alg
            out[f"t{tissue}_sv{sv}_vrates"] = vrates
            out[f"t{tissue}_sv{sv}_valg"] = valg
        out[f"t{tissue}_consts"] = Cc
        out[f"t{tissue}_init"] = S0
        out[f"t{tissue}_states"] = ys
        out[f"t{tissue}_times"] = ts
    out["stim"] = STIM
    np.savez_compressed(HERE / f"ionic_rhs_{key}.npz", **out)


def make_trace():
    src = (REF / "tutorials/manufacturedSolutions/singleCellBidomain/postProcessing/"
           "AlievPanfilov_myocyte_S1_1000.txt")
    g = np.loadtxt(src, skiprows=1)
    vm = np.rint(g[:, 1] * 1e7).astype(np.int64)
    np.savez_compressed(HERE / "aliev_panfilov_singlecell.npz", vm_1e7=vm,
                        t_first=g[0, 0], dt=g[1, 0] - g[0, 0])


def parse_table(path):
    rows = []
    for line in Path(path).read_text().splitlines():
        if not line.strip() or line.lstrip().startswith("#"):
            continue
        rows.append(line.split())
    return rows


def make_pins():
    sc = parse_table(REF / "tutorials/regressionTests/singleCell/singleCell.reference")
    nd = parse_table(REF / "tutorials/regressionTests/NiedererEtAl2012/NiedererEtAl2012.reference")
    pins = {
        "singleCell": {"model": "BuenoOrovio", "tissue": "endocardialCells",
                       "points": [{"time": float(r[1]), "vm": float(r[2]), "tol": float(r[3])}
                                  for r in sc]},
        "NiedererEtAl2012": {"model": "BuenoOrovio", "tissue": "epicardialCells",
                             "points": [{"time": float(r[1]), "column": int(r[2]),
                                         "activation": float(r[3]), "tol": float(r[4])}
                                        for r in nd]},
    }
    (HERE / "regression_pins.json").write_text(json.dumps(pins, indent=1))


def main():
    R = po.ref_lib()
    if R is None:
        raise SystemExit(f"reference not found at {REF}")
    for m in KEYS:
        make_rhs(R, m)
    make_trace()
    make_pins()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
