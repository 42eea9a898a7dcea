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


@pytest.mark.gpu
def test_single_cell_trace_against_reference_file(gpu_lib, tmp_path):
    """SingleCellSolver's trace of AlievPanfilov written through
    cfg_ionic_trace_row equals the reference's own trace file (time and Vm,
    7 decimals) within one unit of the last printed digit."""
    from cardiacfoam_gb300 import io
    g = np.load(GOLDEN / "aliev_panfilov_singlecell.npz")
    ref = g["vm_1e7"][:400] * 1e-7
    dt = 5e-5
    stim = api.stimulus_desc(20, 1000, 1, 0.4, 3)
    m = api.IonicModel("AlievPanfilov", "myocyte", 1, dt, solve_vm_within_ode=True,
                       ode=api.ode_desc(abs_tol=1e-6, rel_tol=1e-4, max_steps=10 ** 6),
                       stimulus=stim)
    path = tmp_path / io.trace_file_name("AlievPanfilov", "myocyte", stim)
    tr = io.SingleCellTrace(m, path, columns=["Vm"])
    im = np.zeros(1)
    t = 0.0
    for k in range(ref.size):
        t = t + dt                       # runTime accumulates deltaT
        m.solveODE(t - dt, dt, None, im)
        tr.write(t)
    tr.close()
    lines = path.read_text().splitlines()
    assert lines[0] == "time Vm"
    rows = np.array([[float(x) for x in l.split()] for l in lines[1:]])
    assert np.allclose(rows[:, 0], (np.arange(ref.size) + 1) * dt, atol=5e-8)
    assert np.max(np.abs(rows[:, 1] - ref)) <= 2.01e-7
    # every variable: Vm, the other states, the algebraics, RATES_<state>
    header = m.trace_header()
    names = header.split()
    assert names[0] == "time" and names[1] == "Vm" and names[-1].startswith("RATES_")
    row = m.trace_row(0, t).split()
    assert len(row) == len(names)
    m.close()
