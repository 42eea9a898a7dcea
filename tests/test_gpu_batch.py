"""Batched single cells (cfg_batch_*): the persistent work-stealing kernels
against the CPU oracle's single cells, the device-side beat detector against
the restated restitution post-processing on the same trace, the reference's
AlievPanfilov golden trace through the batch path, and chunking invariance.

A lone FP64 thread runs ToRORd_dynCl at GB300's FP64 rate (tens of
microseconds per right-hand side), so the FP64 cases use a 0.1 ms solver
step and one beat."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from cardiacfoam_gb300 import api, lib
from oracle import apd as oapd

GOLDEN = Path(__file__).parent / "golden"
TORORD_CA = 9          # index of Cai among ToRORd_dynCl's states


def _protocols(n, seed, cl_range=(0.3, 0.45), beats=(2, 3)):
    """S1 trains from 10 ms (an upstroke at t = 0 has no baseline sample),
    and 250 ms after the last stimulus so the last beat repolarises."""
    rng = np.random.default_rng(seed)
    cl = rng.uniform(*cl_range, n)                       # s
    nb = rng.integers(beats[0], beats[1] + 1, n)
    stimuli = [api.stimulus_desc(10.0, cl[c] * 1000.0, 1.0, 53.0, int(nb[c])) for c in range(n)]
    end = 0.01 + cl * nb + 0.25
    scales = np.exp(rng.uniform(np.log(0.5), np.log(2.0), (6, n)))
    return stimuli, end, scales


def _times(steps, dt):
    t = np.zeros(steps + 1)
    t[1:] = np.cumsum(np.full(steps, dt))      # runTime accumulates deltaT
    return t


def _oracle_cell(oracle, c, stimuli, end, scales, dt):
    st = stimuli[c]
    stim = oracle.Stimulus(st.stim_start, st.stim_period_s1, st.stim_duration,
                           st.stim_amplitude, st.nstim1, st.stim_period_s2, st.nstim2)
    n_steps = int(round(end[c] / dt))
    ode = oracle.ode_settings(max_steps=10 ** 6)
    vm, ca, _, _ = oracle.single_cell_traces("ToRORd_dynCl", 3, dt, n_steps, TORORD_CA,
                                             ode=ode, stim=stim, scales=scales[:, c].copy())
    return vm, ca


@pytest.mark.gpu
def test_batch_fp64_matches_oracle_single_cells(gpu_lib, oracle):
    dt, n = 1e-4, 2
    stimuli, end, scales = _protocols(n, seed=7, cl_range=(0.3, 0.35), beats=(1, 1))
    steps = np.round(end / dt).astype(int)
    b = api.BatchCells("ToRORd_dynCl", "endocardialCells", dt, stimuli, end,
                       precision=lib.PRECISION_FP64, scales=scales,
                       ode=api.ode_desc(max_steps=10 ** 6), trace_cells=n,
                       trace_samples=int(steps.max()) + 1, chunk=1000)
    b.run()
    tr = b.trace()
    nb, apd_ms, tup, ca = b.results()
    quiet = int(0.009 / dt)          # before the first stimulus at 10 ms
    for c in range(n):
        vm_o, ca_o = _oracle_cell(oracle, c, stimuli, end, scales, dt)
        vm_g = tr[c, 0, 1:steps[c] + 1]
        # the same arithmetic: equal to round-off until the upstroke, where
        # last-ulp exp/log differences (device vs host libm) shift the
        # adaptive steps by a fraction of a microsecond
        assert np.max(np.abs(vm_g[:quiet] - vm_o[:quiet])) < 1e-9 * np.max(np.abs(vm_o[:quiet]))
        t = _times(steps[c], dt)
        nbo, apdo, tupo, cao = oapd.last_beat(t, np.concatenate([[tr[c, 0, 0]], vm_o]),
                                              np.concatenate([[tr[c, 1, 0]], ca_o]))
        assert nb[c] == nbo == stimuli[c].nstim1
        assert abs(apd_ms[c] - apdo) < 1e-2, (apd_ms[c], apdo)     # ms
        assert abs(tup[c] - tupo) < 1e-6
        assert abs(ca[c] - cao) < 1e-3 * abs(cao)
        # the device's beat detector equals the post-processing of its trace
        got = oapd.last_beat(t, tr[c, 0, :steps[c] + 1], tr[c, 1, :steps[c] + 1])
        assert (nb[c], apd_ms[c], tup[c], ca[c]) == got
    b.close()


@pytest.mark.gpu
def test_batch_mixed_beat_detector_equals_trace_postprocessing(gpu_lib):
    """The streaming detector on the device gives what the restated
    post-processing gives on the full trace the device recorded."""
    dt, n = 1e-5, 8
    stimuli, end, scales = _protocols(n, seed=11, beats=(2, 4))
    steps = np.round(end / dt).astype(int)
    b = api.BatchCells("ToRORd_dynCl", "endocardialCells", dt, stimuli, end,
                       precision=lib.PRECISION_MIXED, scales=scales,
                       ode=api.ode_desc(max_steps=10 ** 6), trace_cells=n,
                       trace_samples=int(steps.max()) + 1)
    b.run()
    tr = b.trace()
    nb, apd_ms, tup, ca = b.results()
    for c in range(n):
        t = _times(steps[c], dt)
        got = oapd.last_beat(t, tr[c, 0, :steps[c] + 1], tr[c, 1, :steps[c] + 1])
        assert nb[c] == got[0] == stimuli[c].nstim1
        assert not np.isnan(apd_ms[c])
        assert (nb[c], apd_ms[c], tup[c], ca[c]) == got
    b.close()


@pytest.mark.gpu
def test_batch_mixed_close_to_fp64(gpu_lib):
    """APD90 and peak Ca of the mixed form against the FP64 form."""
    dt, n = 1e-4, 32
    stimuli, end, scales = _protocols(n, seed=3, cl_range=(0.3, 0.35), beats=(1, 1))
    runs = []
    for precision in (lib.PRECISION_FP64, lib.PRECISION_MIXED):
        b = api.BatchCells("ToRORd_dynCl", "endocardialCells", dt, stimuli, end,
                           precision=precision, scales=scales, ode=api.ode_desc(max_steps=10 ** 6))
        b.run()
        runs.append(b.results())
        b.close()
    (nb0, apd0, _, ca0), (nb1, apd1, _, ca1) = runs
    assert np.array_equal(nb0, nb1) and np.all(nb0 == 1)
    assert not np.any(np.isnan(apd0)) and not np.any(np.isnan(apd1))
    assert np.max(np.abs(apd0 - apd1)) < 0.05                   # ms
    assert np.max(np.abs(ca0 - ca1) / np.abs(ca0)) < 1e-3


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [lib.PRECISION_FP64, lib.PRECISION_MIXED],
                         ids=["fp64", "mixed"])
def test_batch_chunking_and_uneven_lengths(gpu_lib, precision):
    """Work stealing over uneven run lengths (including empty ones) with a
    small chunk gives bitwise the same cells as one long chunk."""
    dt, n = 1e-4, 40
    stimuli, _, scales = _protocols(n, seed=5, beats=(1, 1))
    end = np.random.default_rng(1).uniform(0.0, 0.04, n)
    end[::7] = 0.0
    out = []
    for chunk in (37, 10 ** 6):
        b = api.BatchCells("ToRORd_dynCl", "endocardialCells", dt, stimuli, end,
                           precision=precision, scales=scales,
                           ode=api.ode_desc(max_steps=10 ** 6), chunk=chunk)
        b.run()
        out.append((b.results(), b.states(), b.stats()))
        b.close()
    (r0, s0, st0), (r1, s1, st1) = out
    for a, bb in zip(r0, r1):
        assert np.array_equal(a, bb, equal_nan=True)
    assert np.array_equal(s0, s1)
    assert st0[1] == st1[1] == int(np.round(end / dt).sum())
    assert st0[2] > st1[2]                                       # more launches


@pytest.mark.gpu
def test_batch_aliev_panfilov_golden_trace(gpu_lib):
    """The reference's AlievPanfilov single-cell trace through the batch path."""
    g = np.load(GOLDEN / "aliev_panfilov_singlecell.npz")
    ref = g["vm_1e7"] * 1e-7
    dt = 5e-5
    stim = api.stimulus_desc(20, 1000, 1, 0.4, 3)
    b = api.BatchCells("AlievPanfilov", "myocyte", dt, [stim], np.array([ref.size * dt]),
                       ode=api.ode_desc(abs_tol=1e-6, rel_tol=1e-4, max_steps=10 ** 6),
                       trace_cells=1, trace_samples=ref.size + 1)
    b.run()
    vm = b.trace()[0, 0, 1:]
    assert np.max(np.abs(vm - ref)) < 2e-7
    b.close()


def test_batch_rejects_unknown_model(gpu_lib):
    """Selection errors come before any device work (runs without a GPU)."""
    stim = (lib.StimulusDesc * 1)(api.stimulus_desc())
    end = np.array([0.1])
    d = lib.BatchDesc()
    d.ionic_model = b"NoSuchModel"
    d.tissue = b"myocyte"
    d.n_cells = 1
    d.delta_t = 1e-5
    d.ode = api.ode_desc()
    d.stimulus = C.cast(stim, C.c_void_p)
    d.end_time = end.ctypes.data
    h = C.c_void_p()
    assert gpu_lib.cfg_batch_create(C.byref(d), C.byref(h)) == lib.CFG_ERR_INVALID
    assert b"NoSuchModel" in gpu_lib.cfg_last_error()


def test_apd_restatement_on_a_synthetic_trace():
    """The restated post-processing on a trace whose answer is known: two
    trapezoidal action potentials (rise 1 ms, plateau, linear decay)."""
    dt = 1e-5
    t = np.arange(0, 1.0, dt)
    vm = np.full_like(t, -85.0)
    for t0 in (0.1, 0.6):
        up = (t >= t0) & (t < t0 + 1e-3)
        vm[up] = -85.0 + 125.0 * (t[up] - t0) / 1e-3
        pl = (t >= t0 + 1e-3) & (t < t0 + 0.2)
        vm[pl] = 40.0
        dn = (t >= t0 + 0.2) & (t < t0 + 0.3)
        vm[dn] = 40.0 - 125.0 * (t[dn] - t0 - 0.2) / 0.1
    beats = oapd.detect_beats(t, vm)
    assert len(beats) == 2
    for b, t0 in zip(beats, (0.1, 0.6)):
        assert b["v_base"] == -85.0 and b["v_peak"] == 40.0
        # v90 = -72.5 is reached 0.09 s into the decay
        assert abs(b["t_repol90"] - (t0 + 0.29)) < 2 * dt
        assert abs(b["t_up"] - t0) < 2 * dt
