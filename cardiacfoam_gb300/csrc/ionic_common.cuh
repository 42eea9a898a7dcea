// Device-side building blocks shared by the generated ionic models and the
// ionic kernels: precision-overloaded math, the single-cell stimulus
// protocol, and the Fehlberg 4(5) tableau that OpenFOAM's RKF45 uses.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define CFG_HD __host__ __device__
#define CFG_D __device__
#else
#define CFG_HD
#define CFG_D
#endif

// how the PDE membrane potential [V] maps onto state 0 of a model
#define CFG_VM_MV 0      // mV (TNNP.C:137, ORd.C:125, ToRORd_dynCl.C:125)
#define CFG_VM_ALIEV 1   // (1000 Vm + 80) / 100 (AlievPanfilov.C:121)
#define CFG_VM_BUENO 2   // (1000 Vm + 84) / 85.7 (BuenoOrovio.C:120)
#define CFG_VM_IDENTITY 3  // Vm itself (monodomainFDAManufactured.C:108)

namespace cfg {

// compile-time list of tissue flags
template <int... T>
struct TissueList {};

// ---------------------------------------------------------------- math
// double: IEEE functions (the plain form); float: single-precision
// functions (the mixed form).  Integer powers are products, so pow(x, 2.0)
// rounds exactly like a correctly rounded pow.
CFG_HD __forceinline__ double cfg_exp(double x) { return exp(x); }
CFG_HD __forceinline__ float cfg_exp(float x) { return expf(x); }
CFG_HD __forceinline__ double cfg_log(double x) { return log(x); }
CFG_HD __forceinline__ float cfg_log(float x) { return logf(x); }
CFG_HD __forceinline__ double cfg_sqrt(double x) { return sqrt(x); }
CFG_HD __forceinline__ float cfg_sqrt(float x) { return sqrtf(x); }
CFG_HD __forceinline__ double cfg_tanh(double x) { return tanh(x); }
CFG_HD __forceinline__ float cfg_tanh(float x) { return tanhf(x); }
CFG_HD __forceinline__ double cfg_fabs(double x) { return fabs(x); }
CFG_HD __forceinline__ float cfg_fabs(float x) { return fabsf(x); }
CFG_HD __forceinline__ double cfg_floor(double x) { return floor(x); }
CFG_HD __forceinline__ float cfg_floor(float x) { return floorf(x); }
CFG_HD __forceinline__ double cfg_pow(double x, double y) { return pow(x, y); }
// exp(x) - 1 of the generated GHK fluxes: in double exactly the reference's
// two operations; in float expm1f, which keeps its relative accuracy as
// x -> 0 where expf(x) - 1 cancels to 0 (and the flux to 0/0)
CFG_HD __forceinline__ double cfg_expm1(double x) { return exp(x) - 1.0; }
CFG_HD __forceinline__ float cfg_expm1(float x) { return expm1f(x); }
CFG_HD __forceinline__ float cfg_pow(float x, float y) { return powf(x, y); }

// Division by a value the tissue form keeps per cell and step (a rate
// constant or time constant of the membrane potential alone): the hoisted
// slot holds cfg_hrcp(v) and each stage evaluates cfg_hdiv(a, slot).  In
// double that is exactly a / v; in float (the mixed form, where a division
// is already a reciprocal and a product) the reciprocal is formed once per
// step instead of at every stage.
CFG_HD __forceinline__ double cfg_hrcp(double v) { return v; }
CFG_HD __forceinline__ float cfg_hrcp(float v) { return 1.0f / v; }
CFG_HD __forceinline__ double cfg_hdiv(double a, double h) { return a / h; }
CFG_HD __forceinline__ float cfg_hdiv(float a, float h) { return a * h; }

template <int N, class R>
CFG_HD __forceinline__ R cfg_ipow(R x)
{
    static_assert(N >= 1 && N <= 16, "integer power out of range");
    if constexpr (N == 1) return x;
    else if constexpr (N == 2) return x * x;
    else if constexpr (N == 3) return x * x * x;
    else if constexpr (N % 2 == 0) { R h = cfg_ipow<N / 2>(x); return h * h; }
    else { R h = cfg_ipow<N / 2>(x); return h * h * x; }
}

// ---------------------------------------------------------------- stimulus
// Single-cell S1/S2 protocol (StimulusProtocol, stimulusIO.H:32-53).
struct CfgStimulus {
    double start, period_s1, duration, amplitude;
    int n1;
    double period_s2;
    int n2;
};

// stimulusIO::computeStimulus (stimulusIO.C:238-286) in type R
template <class R>
CFG_D __forceinline__ R cfg_stimulus_current(R t, const CfgStimulus& s)
{
    R I = R(0);
    if (s.period_s1 > 0.0 && s.n1 > 0) {
        R per = R(s.period_s1);
        R tp = t - R(s.start);
        if (tp >= R(0) && tp <= per * R(s.n1)) {
            R phase = tp - cfg_floor(tp / per) * per;
            if (phase >= R(0) && phase <= R(s.duration)) I = -R(s.amplitude);
        }
    }
    if (I == R(0) && s.period_s2 > 0.0 && s.n2 > 0) {
        R per = R(s.period_s2);
        R t1 = R(s.start) + R(s.period_s1) * R(s.n1);
        R tp = t - t1;
        if (tp >= R(0) && tp <= per * R(s.n2)) {
            R phase = tp - cfg_floor(tp / per) * per;
            if (phase >= R(0) && phase <= R(s.duration)) I = -R(s.amplitude);
        }
    }
    return I;
}

// ---------------------------------------------------------------- RKF45
// Fehlberg 4(5) coefficients as OpenFOAM's RKF45 defines them; the
// divisions are evaluated in double exactly as the host does.
namespace rkf {
constexpr double c2 = 1.0 / 4.0, c3 = 3.0 / 8.0, c4 = 12.0 / 13.0, c5 = 1.0, c6 = 1.0 / 2.0;
constexpr double a21 = 1.0 / 4.0;
constexpr double a31 = 3.0 / 32.0, a32 = 9.0 / 32.0;
constexpr double a41 = 1932.0 / 2197.0, a42 = -7200.0 / 2197.0, a43 = 7296.0 / 2197.0;
constexpr double a51 = 439.0 / 216.0, a52 = -8.0, a53 = 3680.0 / 513.0, a54 = -845.0 / 4104.0;
constexpr double a61 = -8.0 / 27.0, a62 = 2.0, a63 = -3544.0 / 2565.0, a64 = 1859.0 / 4104.0,
                 a65 = -11.0 / 40.0;
constexpr double b1 = 16.0 / 135.0, b3 = 6656.0 / 12825.0, b4 = 28561.0 / 56430.0,
                 b5 = -9.0 / 50.0, b6 = 2.0 / 55.0;
constexpr double e1 = 25.0 / 216.0 - b1, e3 = 1408.0 / 2565.0 - b3, e4 = 2197.0 / 4104.0 - b4,
                 e5 = -1.0 / 5.0 - b5, e6 = -b6;
}  // namespace rkf

// adaptive controller settings (ODESolver / adaptiveSolver dictionary keys)
struct OdeSettings {
    double abs_tol, rel_tol;
    long long max_steps;
    double safe_scale, min_scale, max_scale, alpha_inc, alpha_dec;
    double inc_threshold;   // pow(max_scale/safe_scale, -1/alpha_inc), computed on the host
};

}  // namespace cfg
