"""GPU ionic update (cfg_ionic_* through the C ABI) against the CPU oracle."""
import json
from pathlib import Path

import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib

GOLDEN = Path(__file__).parent / "golden"
CASES = [("TNNP", "epicardialCells"), ("TNNP", "mCells"), ("ORd", "myocyte"),
         ("ToRORd_dynCl", "endocardialCells"), ("AlievPanfilov", "myocyte"),
         ("BuenoOrovio", "epicardialCells")]


def vm_history(n, t):
    """A smooth upstroke per cell at staggered times (V)."""
    tc = np.linspace(0.2e-3, 1.5e-3, n)
    return -0.084 + 0.12 / (1.0 + np.exp(-(t - tc) / 5e-5))


@pytest.mark.gpu
@pytest.mark.parametrize("model,tissue", CASES)
def test_tissue_mode_fp64_matches_oracle(gpu_lib, oracle, model, tissue):
    n, dt, steps = 64, 1e-5, 200
    flag = api.TISSUE_FLAGS[tissue]
    gpu = api.IonicModel(model, tissue, n, dt, precision=lib.PRECISION_FP64,
                         ode=api.ode_desc(max_steps=10 ** 6))
    ora = oracle.Ionic(model, n, flag, dt, ode=oracle.ode_settings(max_steps=10 ** 6))
    im_g, im_o = np.zeros(n), np.zeros(n)
    t = 0.0
    for s in range(steps):
        t = t + dt
        vm = vm_history(n, t - dt)
        gpu.solveODE(t - dt, dt, vm, im_g)
        ora.solve(t - dt, dt, vm, im_o)
        scale = max(np.abs(im_o).max(), 1e-30)
        assert np.max(np.abs(im_g - im_o)) <= 1e-9 * scale, (s, np.max(np.abs(im_g - im_o)))
    yg = gpu.states().T
    yo = ora.states()
    rel = np.abs(yg - yo) / np.maximum(np.abs(yo), 1e-12)
    assert np.max(rel[:, 1:]) < 1e-9
    assert np.allclose(gpu.steps(), ora.steps(), rtol=1e-9, atol=0)
    # same work up to rare accept/reject flips at err ~ 1 (last-ulp exp differences)
    assert abs(gpu.rhs_evaluations() - (ora.rhs_evals() + steps * n)) <= 0.005 * ora.rhs_evals()


@pytest.mark.gpu
@pytest.mark.parametrize("model,tissue", [("TNNP", "epicardialCells"), ("ORd", "myocyte"),
                                          ("ToRORd_dynCl", "endocardialCells")])
def test_tissue_mode_mixed_close_to_fp64(gpu_lib, model, tissue):
    n, dt, steps = 64, 1e-5, 200
    a = api.IonicModel(model, tissue, n, dt, precision=lib.PRECISION_FP64,
                       ode=api.ode_desc(max_steps=10 ** 6))
    b = api.IonicModel(model, tissue, n, dt, precision=lib.PRECISION_MIXED,
                       ode=api.ode_desc(max_steps=10 ** 6))
    ia, ib = np.zeros(n), np.zeros(n)
    t = 0.0
    for s in range(steps):
        t = t + dt
        vm = vm_history(n, t - dt)
        a.solveODE(t - dt, dt, vm, ia)
        b.solveODE(t - dt, dt, vm, ib)
    # mixed form: FP32 currents; compare relative to the current's range
    assert np.max(np.abs(ia - ib)) < 2e-3 * np.max(np.abs(ia)) + 1e-3


@pytest.mark.gpu
def test_single_cell_aliev_panfilov_golden_trace(gpu_lib):
    g = np.load(GOLDEN / "aliev_panfilov_singlecell.npz")
    ref = g["vm_1e7"] * 1e-7
    dt = 5e-5
    stim = api.stimulus_desc(20, 1000, 1, 0.4, 3)
    cell = api.IonicModel("AlievPanfilov", "myocyte", 1, dt, solve_vm_within_ode=True,
                          ode=api.ode_desc(abs_tol=1e-6, rel_tol=1e-4, max_steps=10 ** 6),
                          stimulus=stim)
    im = np.zeros(1)
    out = np.zeros(ref.size)
    t = 0.0
    for s in range(ref.size):
        t = t + dt
        cell.solveODE(t - dt, dt, None, im)
        out[s] = cell.states()[0, 0] * 100 - 80      # AlievPanfilov::transformedVm
    assert np.max(np.abs(out - ref)) < 2e-7


@pytest.mark.gpu
def test_single_cell_bueno_orovio_regression(gpu_lib):
    pins = json.loads((GOLDEN / "regression_pins.json").read_text())["singleCell"]["points"]
    dt = 5e-5
    stim = api.stimulus_desc(20, 1000, 1, 0.4, 3)
    cell = api.IonicModel("BuenoOrovio", "endocardialCells", 1, dt, solve_vm_within_ode=True,
                          ode=api.ode_desc(abs_tol=1e-6, rel_tol=1e-4, max_steps=10 ** 6),
                          stimulus=stim)
    im = np.zeros(1)
    want = {int(round(p["time"] / dt)): p for p in pins}
    t = 0.0
    for s in range(1, max(want) + 1):
        t = t + dt
        cell.solveODE(t - dt, dt, None, im)
        if s in want:
            vm = cell.states()[0, 0] * 85.7 - 84.0          # BuenoOrovio::transformedVm
            assert abs(vm - want[s]["vm"]) <= want[s]["tol"]
            assert abs(vm - want[s]["vm"]) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [lib.PRECISION_FP64, lib.PRECISION_MIXED],
                         ids=["fp64", "mixed"])
def test_per_cell_tissue_equals_uniform_models(gpu_lib, precision):
    """Per-cell tissue flags: the cells run grouped by tissue through the
    kernels specialised for each tissue, so every cell equals, bit for bit,
    the same cell in a model of its tissue alone; states, steps and the
    import of states come back in cell order."""
    rng = np.random.default_rng(17)
    n, dt = 3000, 1e-5
    flags = rng.integers(1, 4, n).astype(np.uint8)
    names = {1: "epicardialCells", 2: "mCells", 3: "endocardialCells"}
    vm = -0.084 + 0.12 * rng.random(n)
    mixed = api.IonicModel("TNNP", "epicardialCells", n, dt, precision=precision,
                           tissue_per_cell=flags)
    im = np.zeros(n)
    for k in range(5):
        mixed.solveODE(k * dt, dt, vm, im)
    states = mixed.states()
    steps = mixed.steps()
    for t, name in names.items():
        uni = api.IonicModel("TNNP", name, n, dt, precision=precision)
        im_u = np.zeros(n)
        for k in range(5):
            uni.solveODE(k * dt, dt, vm, im_u)
        sel = flags == t
        assert np.array_equal(im[sel], im_u[sel])
        assert np.array_equal(states[:, sel], uni.states()[:, sel])
        assert np.array_equal(steps[sel], uni.steps()[sel])
        uni.close()
    # import: a round trip through set_states leaves the cells where they are
    mixed.set_states(states)
    assert np.array_equal(mixed.states(), states)
    mixed.close()
