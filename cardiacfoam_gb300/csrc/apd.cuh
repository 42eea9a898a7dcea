// Streaming beat detector (APD90, peak Ca) restating the reference's
// restitution post-processing (postProcessing_restCurves.py), fed one sample
// (time, Vm [mV], Ca) at a time; used by the batched single cells and by the
// tissue step's per-cell APD tracking.
#pragma once

#include <cuda_runtime.h>

#include "ionic_common.cuh"

namespace cfg {

// Beat detection settings (postProcessing_restCurves.py:14-17): upstroke at
// dV/dt = 5000 mV/s, baseline = minimum over the 2 ms before it, peak and
// repolarisation searched up to 2 s after it or to the next upstroke.
struct ApdParams {
    double dvdt_threshold;   // mV/s
    double baseline;         // s
    double peak_search;      // s
    int ring;                // samples kept for the baseline window
};

// Streaming state of the beat detector of one cell.  Samples are the
// solver's trace (time [s], Vm [mV], Ca); sample m is processed into the beat
// windows when sample m+1 arrives, because the central dV/dt at m needs it.
struct ApdTracker {
    long long m;             // samples seen
    double t1, v1, ca1;      // sample m-1
    double t2, v2;           // sample m-2
    double d1;               // dV/dt at sample m-2
    int open;                // a beat window is open
    int crossed;             // repolarisation found after the current peak
    double t_up, v_base, v_peak, t_rep, ca_peak;
    double tw, vw;           // previous sample inside the window
    int n_beats;
    double last_t_up, last_apd, last_ca;   // last finished beat (apd [s], NaN if none)
};

CFG_HD inline ApdParams apd_defaults(double dt)
{
    ApdParams p;
    p.dvdt_threshold = 5000.0;
    p.baseline = 0.002;
    p.peak_search = 2.0;
    p.ring = int(p.baseline / dt) + 3;
    return p;
}

CFG_D __forceinline__ double cfg_nan() { return __longlong_as_double(0x7ff8000000000000ll); }
CFG_D __forceinline__ double cfg_neg_inf() { return __longlong_as_double(0xfff0000000000000ll); }

// One sample of the open window: peak, first downward crossing of v90 after
// the peak (linear interpolation), peak Ca.
CFG_D __forceinline__ void apd_include(ApdTracker& a, double t, double v, double ca)
{
    if (v > a.v_peak) {
        a.v_peak = v;
        a.t_rep = cfg_nan();
        a.crossed = 0;
    } else if (!a.crossed) {
        const double v90 = a.v_base + 0.1 * (a.v_peak - a.v_base);
        if (a.vw > v90 && v90 >= v) {
            const double frac = (v90 - a.vw) / (v - a.vw);
            a.t_rep = a.tw + frac * (t - a.tw);
            a.crossed = 1;
        }
    }
    if (ca > a.ca_peak) a.ca_peak = ca;
    a.tw = t;
    a.vw = v;
}

CFG_D __forceinline__ void apd_finish(ApdTracker& a)
{
    a.n_beats += 1;
    a.last_t_up = a.t_up;
    a.last_apd = a.crossed ? a.t_rep - a.t_up : cfg_nan();
    a.last_ca = a.ca_peak;
    a.open = 0;
}

// Sample m (t, v, ca).  ring_t/ring_v: this cell's ring of the last
// `ring` samples, stride `rs` between entries.
CFG_D inline void apd_sample(ApdTracker& a, const ApdParams& P, double t, double v, double ca,
                             double* ring_t, double* ring_v, long long rs)
{
    const long long slot = (a.m % P.ring) * rs;
    ring_t[slot] = t;
    ring_v[slot] = v;
    if (a.m >= 2) {
        const double d = (v - a.v2) / (t - a.t2);          // dV/dt at sample m-1
        const double dprev = a.m == 2 ? d : a.d1;           // sample 0 copies sample 1
        const double thr = P.dvdt_threshold;
        bool cand = dprev < thr && thr <= d;
        double tup = 0.0;
        if (cand) {
            const double frac = (thr - dprev) / (d - dprev);
            cand = frac >= 0.0 && frac <= 1.0;
            tup = a.t2 + frac * (a.t1 - a.t2);
        }
        if (cand) {
            if (a.open) {
                if (a.t1 <= tup) apd_include(a, a.t1, a.v1, a.ca1);
                apd_finish(a);
            }
            // baseline: minimum over tup - baseline <= t < tup
            double vb = 0.0;
            bool any = false;
            const long long k0 = a.m + 1 > P.ring ? a.m + 1 - P.ring : 0;
            for (long long k = k0; k <= a.m; ++k) {
                const long long s = (k % P.ring) * rs;
                const double tk = ring_t[s];
                if (tk >= tup - P.baseline && tk < tup) {
                    const double vk = ring_v[s];
                    if (!any || vk < vb) vb = vk;
                    any = true;
                }
            }
            if (any) {
                a.open = 1;
                a.t_up = tup;
                a.v_base = vb;
                a.v_peak = cfg_neg_inf();
                a.t_rep = cfg_nan();
                a.crossed = 0;
                a.ca_peak = cfg_neg_inf();
                apd_include(a, a.t1, a.v1, a.ca1);
            }
        } else if (a.open) {
            if (a.t1 <= a.t_up + P.peak_search) apd_include(a, a.t1, a.v1, a.ca1);
            else apd_finish(a);
        }
        a.d1 = d;
    }
    a.t2 = a.t1;
    a.v2 = a.v1;
    a.t1 = t;
    a.v1 = v;
    a.ca1 = ca;
    a.m += 1;
}

// End of the trace: the last sample (no upstroke can start there, dV/dt at
// the end copies its neighbour) and the open beat.
CFG_D inline void apd_end(ApdTracker& a, const ApdParams& P)
{
    if (a.m >= 2 && a.open) {
        if (a.t1 <= a.t_up + P.peak_search) apd_include(a, a.t1, a.v1, a.ca1);
        else apd_finish(a);
    }
    if (a.open) apd_finish(a);
}

}  // namespace cfg
