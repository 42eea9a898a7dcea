"""The CPU oracle against the reference's own numbers (no GPU needed).

* model right-hand sides vs the reference's generated headers compiled
  verbatim (golden vectors from tests/golden/make_golden.py), bit for bit;
* RKF45 + single-cell driver vs the reference's regression values
  (singleCell.reference) and its Aliev-Panfilov golden trace;
* explicit tissue path vs the NiedererEtAl2012 regression probes.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import niederer_case as nc

GOLDEN = Path(__file__).parent / "golden"
MODELS = {"TNNP": "tnnp", "ORd": "ord", "ToRORd_dynCl": "torord_dyncl",
          "AlievPanfilov": "alievpanfilov", "BuenoOrovio": "buenoorovio"}


@pytest.mark.parametrize("model", list(MODELS))
def test_rhs_matches_reference_headers(oracle, model):
    g = np.load(GOLDEN / f"ionic_rhs_{MODELS[model]}.npz")
    s = g["stim"]
    stim = oracle.make_stimulus(s[0], s[1], s[2], s[3], int(s[4]), s[5], int(s[6]))
    tissues = sorted({int(k.split("_")[0][1:]) for k in g.files if k.startswith("t")})
    for tissue in tissues:
        consts, y0 = oracle.model_init(model, tissue)
        assert np.array_equal(consts, g[f"t{tissue}_consts"])
        assert np.array_equal(y0, g[f"t{tissue}_init"])
        ys, ts = g[f"t{tissue}_states"], g[f"t{tissue}_times"]
        for sv in (0, 1):
            for i in range(ys.shape[0]):
                d, a = oracle.model_rates(model, ts[i], consts, ys[i].copy(), tissue, sv, stim)
                np.testing.assert_array_equal(d, g[f"t{tissue}_sv{sv}_rates"][i])
                np.testing.assert_array_equal(a, g[f"t{tissue}_sv{sv}_alg"][i])
                r, a = oracle.model_variables(model, ts[i], consts, ys[i].copy(), tissue, sv, stim)
                np.testing.assert_array_equal(r, g[f"t{tissue}_sv{sv}_vrates"][i])
                np.testing.assert_array_equal(a, g[f"t{tissue}_sv{sv}_valg"][i])


def test_bueno_orovio_single_cell_regression(oracle):
    pins = json.loads((GOLDEN / "regression_pins.json").read_text())["singleCell"]
    ode = oracle.ode_settings(abs_tol=1e-6, rel_tol=1e-4, max_steps=1000000000)
    stim = oracle.make_stimulus(20, 1000, 1, 0.4, 3)
    dt = 5e-5
    trace, _, _ = oracle.single_cell("BuenoOrovio", 3, dt, 10000, ode, stim)
    for p in pins["points"]:
        i = int(round(p["time"] / dt)) - 1
        assert abs(trace[i] - p["vm"]) <= p["tol"]
        # the pins are printed with 7 decimals: agreement is at that resolution
        assert abs(trace[i] - p["vm"]) < 1e-7


def test_aliev_panfilov_golden_trace(oracle):
    g = np.load(GOLDEN / "aliev_panfilov_singlecell.npz")
    ref = g["vm_1e7"]
    ode = oracle.ode_settings(abs_tol=1e-6, rel_tol=1e-4, max_steps=1000000000)
    stim = oracle.make_stimulus(20, 1000, 1, 0.4, 3)
    trace, _, _ = oracle.single_cell("AlievPanfilov", 4, 5e-5, ref.size, ode, stim)
    got = np.rint(trace * 1e7).astype(np.int64)
    assert np.array_equal(got, ref)


def niederer_run(oracle, contract=None, nthreads=8):
    """Activation times of the NiedererEtAl2012 case on the oracle: contract
    None runs the box with exact centres (i + 1/2) h, an integer the cell
    centres as OpenFOAM's geometry code rounds them."""
    b = nc.BLOCK
    if contract is None:
        mesh = oracle.Mesh(b["ni"], b["nj"], b["nk"], *nc.LENGTHS)
    else:
        mesh = oracle.Mesh.general(nc.openfoam_mesh(oracle, contract))
    desc = oracle.tissue_desc("BuenoOrovio", 1, nc.SIGMA, implicit=False, ddt_backward=True,
                              boxes=[(*nc.BOX, *nc.STIMULUS)])
    T = oracle.Tissue(desc, mesh)
    dt = nc.explicit_dt()
    while T.time() < nc.END_TIME - 1e-12:
        T.step(dt, nthreads)
    return T.activation()


@pytest.mark.parametrize("contract", [0, 15], ids=["no-fma", "fma"])
def test_niederer_explicit_regression(oracle, contract):
    """All six probes within the reference's own tolerances
    (NiedererEtAl2012.reference:8-13), on the cell centres OpenFOAM computes
    for the case's mesh: built without fma contraction (gcc on x86-64) and
    with it everywhere an expression allows (clang's default on arm64, the
    host of the regression log).  The stimulus box's faces pass through cell
    centres, and the inclusive box test takes the part of those layers that
    rounding leaves inside: that set decides the transverse probe."""
    act = niederer_run(oracle, contract)
    for probe, expect, tol in nc.pins():
        got = act[nc.probe_cell(nc.PROBES[probe])]
        assert abs(got - expect) <= tol, (probe, got, expect)


def test_niederer_stimulus_layers_are_split_by_rounding(oracle):
    """The stimulus box (0..1.5, 0..1.5, 5.5..7 mm) has its three inner faces
    on planes of cell centres.  Exact centres put all 8 x 8 x 8 cells in;
    OpenFOAM's rounding of the centres leaves part of each face layer out."""
    lo, hi = (np.array(v) for v in nc.BOX)
    b = nc.BLOCK
    exact = oracle.Mesh(b["ni"], b["nj"], b["nk"], *nc.LENGTHS).centres()
    assert np.all((exact >= lo) & (exact <= hi), axis=1).sum() == 512
    for contract in (0, 15):
        c = nc.openfoam_mesh(oracle, contract).centres
        # a few units in the last place of the block's extent on each axis
        assert np.all(np.abs(c - exact) <= 8 * np.spacing(np.array(nc.LENGTHS)))
        inside = np.all((c >= lo) & (c <= hi), axis=1)
        near = np.all((c >= lo - 1e-9) & (c <= hi + 1e-9), axis=1)
        assert near.sum() == 512 and 440 < inside.sum() < 512


def test_ord_reference_constants_gap(oracle):
    """ORd_2011.H never assigns the Na/K-pump constants and upScale: the
    reference (zero-filled CONSTANTS) yields NaN; with the supplement the
    current is finite and the cell fires."""
    consts, y = oracle.model_init("ORd", 4)
    _, alg = oracle.model_rates("ORd", 0.0, consts, y.copy(), 4, 0)
    assert np.isnan(alg[oracle.lib().oracle_model_iion_index(1)])
    consts, y = oracle.model_init("ORd", 4, supplement=True)
    _, alg = oracle.model_rates("ORd", 0.0, consts, y.copy(), 4, 0)
    assert np.all(np.isfinite(alg))
    trace, _, _ = oracle.single_cell("ORd", 4, 1e-5, 3000,
                                     oracle.ode_settings(abs_tol=1e-6, max_steps=10 ** 7),
                                     oracle.make_stimulus(10, 1000, 0.5, 80, 1))
    assert trace[900] < -85 and trace.max() > 30
