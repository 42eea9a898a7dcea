"""sweepCurrent on the GPU (cfg_ionic_sweep_current) against the oracle's
computeVariables at the same clamped states, for every current of the
dependency maps of the four tissue models, with the dependency columns
resolved independently (tests/golden/sweep_columns.json)."""
import json
from pathlib import Path

import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib

GOLDEN = Path(__file__).parent / "golden"
CASES = [("TNNP", "epicardialCells", 1, (-90.0, 60.0)), ("ORd", "myocyte", 4, (-90.0, 60.0)),
         ("ToRORd_dynCl", "endocardialCells", 3, (-90.0, 60.0)),
         ("BuenoOrovio", "endocardialCells", 3, (0.0, 1.5))]


@pytest.mark.gpu
@pytest.mark.parametrize("model,tissue,flag,vrange", CASES, ids=[c[0] for c in CASES])
def test_sweep_matches_oracle_variables(gpu_lib, oracle, model, tissue, flag, vrange):
    cols = json.loads((GOLDEN / "sweep_columns.json").read_text())[model]
    n, dt = 4, 1e-5
    ion = api.IonicModel(model, tissue, n, dt, ode=api.ode_desc(max_steps=10 ** 6))
    vm, im = np.full(n, -0.08), np.zeros(n)
    for s in range(5):                      # states away from the initial ones
        ion.solveODE(s * dt, dt, vm, im)
    y0 = ion.states()[:, 0].copy()
    consts, _ = oracle.model_init(model, flag, supplement=True)
    currents = ion.sweep_currents()
    assert set(currents) == set(cols)
    npts = 33
    for cur in currents:
        header, table = ion.sweep_current(cur, vrange[0], vrange[1], npts)
        assert header[0] == "V" and len(header) == 1 + len(cols[cur])
        for i in range(npts):
            y = y0.copy()
            y[0] = vrange[0] + (vrange[1] - vrange[0]) * float(i) / (npts - 1)
            assert table[i, 0] == y[0]
            rates, alg = oracle.model_variables(model, 0.0, consts, y.copy(), flag, False)
            src = {"state": y, "alg": alg, "rate": rates}
            want = np.array([src[s][k] for s, k in cols[cur]])
            got = table[i, 1:]
            # FP64 on both sides; last-ulp exp/log differences only
            assert np.allclose(got, want, rtol=1e-11, atol=1e-300, equal_nan=True), (cur, i)


@pytest.mark.gpu
def test_sweep_unknown_current(gpu_lib):
    ion = api.IonicModel("TNNP", "epicardialCells", 1, 1e-5)
    with pytest.raises(lib.CfgError) as e:
        ion.sweep_current("NoSuchCurrent", -90, 60, 10)
    assert "Unknown current: NoSuchCurrent" in str(e.value)
    assert "INa" in str(e.value)
