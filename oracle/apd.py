"""APD90 and beat detection of a single-cell trace, as the reference's
restitution post-processing computes them (test infrastructure: the checker
of the device-side beat detector, never used by the library).

Restates ``detect_beats`` of
tutorials/singleCellprotocols/restitutionCurves_s1s2Protocol/
setupRestitutionCurves_s1s2Protocol/postProcessing_restCurves.py (the second
definition, which replaces the first) with its parameters at
lines 14-16:

* dV/dt by central differences, the end points copying their neighbours
  (``safe_dvdt``, lines 53-58);
* an upstroke wherever dV/dt crosses the threshold upwards, its time linearly
  interpolated (lines 123-128);
* baseline = minimum of Vm over [t_up - 2 ms, t_up); the beat is skipped if
  that window holds no sample (lines 146-150);
* peak = maximum over [t_up, min(t_up + 2 s, next upstroke)] (lines 152-163);
* v90 = baseline + 0.1 (peak - baseline), and the first downward crossing of
  v90 after the (first) peak, linearly interpolated, is the 90 %
  repolarisation time (lines 166-186).

The peak Ca of a beat is the maximum of the Ca trace over the same window
(the reference reports APD only; Ca is sampled where Vm is).
"""
from __future__ import annotations

import numpy as np

DVDT_THRESHOLD = 5000.0   # mV/s
BASELINE = 0.002          # s
PEAK_SEARCH = 2.0         # s


def safe_dvdt(vm: np.ndarray, time: np.ndarray) -> np.ndarray:
    d = np.zeros_like(vm)
    d[1:-1] = (vm[2:] - vm[:-2]) / (time[2:] - time[:-2])
    d[0] = d[1]
    d[-1] = d[-2]
    return d


def detect_beats(time: np.ndarray, vm: np.ndarray, ca: np.ndarray | None = None) -> list:
    """Beats of a trace (time [s], Vm [mV]); each a dict with t_up, v_base,
    v_peak, v90, t_repol90 (NaN when not found) and ca_peak."""
    dvdt = safe_dvdt(vm, time)
    cands = []
    for i in range(1, len(dvdt)):
        if dvdt[i - 1] < DVDT_THRESHOLD <= dvdt[i]:
            frac = (DVDT_THRESHOLD - dvdt[i - 1]) / (dvdt[i] - dvdt[i - 1])
            if 0.0 <= frac <= 1.0:
                cands.append(time[i - 1] + frac * (time[i] - time[i - 1]))
    beats = []
    for k, t_up in enumerate(cands):
        base = (time >= t_up - BASELINE) & (time < t_up)
        if not np.any(base):
            continue
        v_base = float(np.min(vm[base]))
        t_end = t_up + PEAK_SEARCH
        if k < len(cands) - 1:
            t_end = min(t_end, cands[k + 1])
        win = (time >= t_up) & (time <= t_end)
        if not np.any(win):
            continue
        seg_t, seg_v = time[win], vm[win]
        v_peak = float(np.max(seg_v))
        v90 = v_base + 0.1 * (v_peak - v_base)
        j_peak = int(np.argmax(seg_v))
        t_rep = float("nan")
        for j in range(j_peak + 1, len(seg_v)):
            if seg_v[j - 1] > v90 >= seg_v[j]:
                frac = (v90 - seg_v[j - 1]) / (seg_v[j] - seg_v[j - 1])
                t_rep = float(seg_t[j - 1] + frac * (seg_t[j] - seg_t[j - 1]))
                break
            if k < len(cands) - 1 and seg_t[j] >= cands[k + 1]:
                break
        beats.append({"t_up": float(t_up), "v_base": v_base, "v_peak": v_peak, "v90": v90,
                      "t_repol90": t_rep,
                      "ca_peak": float(np.max(ca[win])) if ca is not None else float("nan")})
    return beats


def last_beat(time: np.ndarray, vm: np.ndarray, ca: np.ndarray | None = None):
    """(beats, last-beat APD90 [ms] (NaN if not repolarised), its upstroke
    time [s], its peak Ca)."""
    beats = detect_beats(time, vm, ca)
    if not beats:
        return 0, float("nan"), float("nan"), float("nan")
    b = beats[-1]
    return len(beats), (b["t_repol90"] - b["t_up"]) * 1000.0, b["t_up"], b["ca_peak"]
