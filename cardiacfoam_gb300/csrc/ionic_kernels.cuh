// Ionic update kernels: one thread per cell, state in SoA arrays, the whole
// per-cell ODE solve of a PDE step held in registers / thread-local memory.
//
// Reference behaviour reproduced (per cell, <Model>::solveODE, e.g.
// src/ionicModels/TNNP/TNNP.C:114-179):
//   STATES[0] <- Vm mapped to model units; step <- min(step, dt_model);
//   ODESolver::solve(tStart, tEnd, STATES, step) with RKF45;
//   computeVariables(tEnd); Im = scale * ALGEBRAIC[Iion].
// The RKF45 step control restates OpenFOAM's ODESolver/adaptiveSolver
// (truncated last step, persistent per-cell step, safeScale/minScale/
// maxScale/alphaInc/alphaDec); the tableau is Fehlberg's.
//
// Precision forms:
//   R = double : every operation in FP64 with the reference's evaluation order
//                (compiled without FMA contraction) - the plain form.
//   R = float  : right-hand side, stage states, gates and the error norm in
//                FP32; the membrane potential, ion concentrations and CaMK
//                (Model::WIDE_MASK) are stored and accumulated in FP64 - the
//                mixed form.  Time and step control stay FP64.
#pragma once

#include <type_traits>

#include "ionic_common.cuh"
#include "../../include/cardiac_gpu.h"

// resident 128-thread blocks per SM the ionic kernels are compiled for
// (register budget 65536 / (128 * blocks))
#ifndef CFG_IONIC_MIN_BLOCKS
#define CFG_IONIC_MIN_BLOCKS 2
#endif
// unroll factor of the per-state loops around the right-hand side (stage
// sums, 5th-order update, error norm); 1 keeps the kernel's instruction
// footprint close to one copy of the model body
#ifndef CFG_IONIC_STATE_UNROLL
#define CFG_IONIC_STATE_UNROLL 1
#endif


namespace cfg {

constexpr int kStateUnroll = CFG_IONIC_STATE_UNROLL;

struct IonicLaunch {
    long long n;                     // cells (and the stride of the state arrays)
    long long first, count;          // state slots [first, first + count) of this launch
    const int* perm;                 // [n] cell of each state slot, or null (slot = cell)
    int cells_per_thread;            // slots per thread (grid-stride), chosen by the launcher
    double t0, dt;                   // PDE step [s] (used when t_dev is null)
    const double* t_dev;             // device time of the step start [s], or null
    int tissue;                      // uniform tissue flag (when tissue_cell is null)
    const unsigned char* tissue_cell;
    const double* scales;            // [6][scale_stride] conductance scales, or null
    long long scale_stride;
    CfgStimulus stim;                // single-cell protocol (tissue runs: none)
    OdeSettings ode;
    const double* vm;                // [n] membrane potential [V] (tissue mode)
    double* im;                      // [n] ionic current [V/s]
    double* yw;                      // wide states  [NW][n] (all states in the plain form)
    float* yn;                       // narrow states [NN][n] (mixed form only)
    double* step;                    // [n] persistent ODE step [model time units]
    int* status;                     // CFG_ERR_* bits, OR-ed
    unsigned long long* rhs_evals;   // optional counter of RHS evaluations
    double* fail_record;             // optional [8]: first failing cell (see IonicFailure)
};

// Record of the first cell whose ODE solve failed: [0] cell, [1] reason
// (1 = maxSteps, 2 = step underflow), [2] x, [3] dx, [4] worst state,
// [5] its normalised error, [6] that state's value, [7] substeps taken.
struct IonicFailure {
    int reason = 0;
    double x = 0, dx = 0, err = 0, value = 0;
    int worst = -1;
    long long steps = 0;
};

template <class R>
struct ArrayView {
    const R* a;
    CFG_D __forceinline__ R operator()(int i) const { return a[i]; }
};

// constants computed at run time (per-cell tissue or conductance scales)
template <class R>
struct ConstView {
    const double* c;
    CFG_D __forceinline__ R operator()(int i) const { return R(c[i]); }
};

// constants of one uniform tissue, known at compile time
template <class R, class M, int T>
struct ConstFold {
    CFG_D __forceinline__ R operator()(int i) const { return R(M::template constant<T>(i)); }
};

template <unsigned long long MASK>
CFG_D __forceinline__ constexpr bool is_wide(int i) { return (MASK >> i) & 1ull; }

template <class M, bool FP64>
struct Layout {
    // index of state i inside the wide or the narrow array
    static CFG_HD constexpr int slot(int i)
    {
        int k = 0;
        for (int j = 0; j < i; ++j)
            if (FP64 || ((M::WIDE_MASK >> j) & 1ull) == ((M::WIDE_MASK >> i) & 1ull)) ++k;
        return k;
    }
    static CFG_HD constexpr int n_wide()
    {
        int k = 0;
        for (int j = 0; j < M::NS; ++j)
            if (FP64 || ((M::WIDE_MASK >> j) & 1ull)) ++k;
        return k;
    }
    static CFG_HD constexpr int n_narrow() { return M::NS - n_wide(); }
};

template <int MAP>
CFG_D __forceinline__ double vm_to_state0(double vm)
{
    if constexpr (MAP == CFG_VM_ALIEV) return (vm * 1000.0 + 80) / 100;
    else if constexpr (MAP == CFG_VM_BUENO) return (vm * 1000.0 + 84) / 85.7;
    else if constexpr (MAP == CFG_VM_IDENTITY) return vm;
    else return vm * 1000.0;
}

// model time of the step: TNNP.C:122-123 (t*1000), AlievPanfilov.C:107-108
template <class M>
CFG_D __forceinline__ void model_times(double t0, double dt, double& ts, double& te, double& dtm)
{
    if constexpr (M::TIME_SCALE == 1000.0) {
        // model time in seconds (monodomainFDAManufactured.C:96-97)
        ts = t0;
        te = t0 + dt;
        dtm = dt;
    } else if constexpr (M::TIME_SCALE == 1.0) {
        ts = t0 * 1000;
        te = (t0 + dt) * 1000;
        dtm = dt * 1000.0;
    } else {
        ts = t0 * 1000.0 / M::TIME_SCALE;
        te = (t0 + dt) * 1000.0 / M::TIME_SCALE;
        dtm = dt * 1000.0 / M::TIME_SCALE;
    }
}

// Step-control arithmetic that must round exactly as written (no FMA
// contraction, which the mixed-form build enables): the end-of-interval test
// relies on x - xEnd being exactly zero when x has landed on xEnd.
CFG_D __forceinline__ double exact_add(double a, double b) { return __dadd_rn(a, b); }
CFG_D __forceinline__ double exact_sub(double a, double b) { return __dsub_rn(a, b); }
CFG_D __forceinline__ double exact_mul(double a, double b) { return __dmul_rn(a, b); }

// Stage table of the Fehlberg tableau for the stage loop (row s: a_s,j),
// in double for the plain form and float for the mixed form.
static __constant__ double kRkfA[6][5] = {
    {0, 0, 0, 0, 0},
    {rkf::a21, 0, 0, 0, 0},
    {rkf::a31, rkf::a32, 0, 0, 0},
    {rkf::a41, rkf::a42, rkf::a43, 0, 0},
    {rkf::a51, rkf::a52, rkf::a53, rkf::a54, 0},
    {rkf::a61, rkf::a62, rkf::a63, rkf::a64, rkf::a65},
};
static __constant__ float kRkfAf[6][5] = {
    {0, 0, 0, 0, 0},
    {float(rkf::a21), 0, 0, 0, 0},
    {float(rkf::a31), float(rkf::a32), 0, 0, 0},
    {float(rkf::a41), float(rkf::a42), float(rkf::a43), 0, 0},
    {float(rkf::a51), float(rkf::a52), float(rkf::a53), float(rkf::a54), 0},
    {float(rkf::a61), float(rkf::a62), float(rkf::a63), float(rkf::a64), float(rkf::a65)},
};
static __constant__ double kRkfC[6] = {0.0, rkf::c2, rkf::c3, rkf::c4, rkf::c5, rkf::c6};

template <class R>
CFG_D __forceinline__ R tableau_a(int s, int j)
{
    if constexpr (sizeof(R) == sizeof(double)) return kRkfA[s][j];
    else return kRkfAf[s][j];
}

// Mixed form: multiple of the FP32 unit round-off charged to each stage
// derivative in the error test (model right-hand sides lose a few tens of
// ulps through exp/log/division chains).
constexpr double kFp32NoiseUlps = 64.0;


// One right-hand-side evaluation.  Not inlined: the stage loop and the final
// current evaluation share one copy of the (large) model body, which keeps
// the kernel's instruction footprint to a single model instance.  In tissue
// mode (SV false) the model's membrane-potential-only values come from H,
// evaluated once per cell and PDE step by M::hoist_vm.
template <class M, bool SV, class R, class KS>
__device__ __noinline__ R rhs_eval(double t, const R* y, const KS* K, const R* H, R* dydt,
                                   int tissue, const CfgStimulus* st)
{
    if constexpr (!SV && M::NH > 0)
        return M::template rates_tissue<R>(t, ArrayView<R>{y}, *K, ArrayView<R>{H}, dydt, tissue,
                                           *st);
    else
        return M::template rates<R, SV>(t, ArrayView<R>{y}, *K, dydt, tissue, *st);
}

// Storage of the per-cell membrane-potential-only values (at least one
// element, so that models without any still compile).
template <class M, class R>
struct Hoisted {
    R v[M::NH > 0 ? M::NH : 1];
};

// Per-cell solver state: y holds every state in double (the plain form) or
// only the slow (WIDE_MASK) states in double; yf holds every state in the
// arithmetic type R, which is what the right-hand side reads.
template <class M, class R>
struct CellState {
    double y[M::NS] = {};   // states initConsts leaves unset are zero
    R yf[M::NS];
};

// ODESolver::solve(xStart, xEnd, y, dxTry) with adaptiveSolver::solve and
// RKF45::solve inside.  The six right-hand-side evaluations of a trial step
// (dydx0 and stages 2..6) run through one loop, so the model body is
// instantiated once.  FP64 stage sums are accumulated left to right exactly
// as the host code writes them.  Returns accepted substeps, or -1 on
// maxSteps overflow / step underflow.
template <class M, bool SV, class R, class KS>
CFG_D __forceinline__ long long rkf45_solve(double xs, double xe, CellState<M, R>& cs,
                                            double& dx_try, R (*k)[M::NS], const KS& K,
                                            int tissue, const CfgStimulus& st,
                                            const OdeSettings& s, unsigned& evals,
                                            IonicFailure* why = nullptr,
                                            const R* H = nullptr)
{
    using namespace rkf;
    constexpr int NS = M::NS;
    constexpr bool D = sizeof(R) == sizeof(double);
    double* y = cs.y;
    R* yf = cs.yf;
    double step_dx = dx_try;
    bool last = false;
    double x = xs;
    R yt[NS];
    R y5f[NS];
    double y5w[NS];
    for (long long n = 0; n < s.max_steps; ++n) {
        const double dx_try0 = step_dx;
        {
            const double xn = exact_add(x, step_dx);
            if (exact_mul(exact_sub(xn, xe), exact_sub(xn, xs)) > 0) {
                last = true;
                step_dx = exact_sub(xe, x);
            }
        }
        // --- adaptiveSolver::solve(odes, x, y, dxTry)
        double dx = step_dx;
        double err;
        int worst = -1;
        int s0 = 0;   // dydx0 is evaluated once per adaptive step
        for (;;) {
            const R h = R(dx);
#pragma unroll 1
            for (int sg = s0; sg < 6; ++sg) {
                if (sg == 0) {
#pragma unroll kStateUnroll
                    for (int i = 0; i < NS; ++i) yt[i] = yf[i];
                } else if (sg == 1) {
#pragma unroll kStateUnroll
                    for (int i = 0; i < NS; ++i) {
                        if constexpr (D) yt[i] = y[i] + a21 * dx * k[0][i];
                        else yt[i] = yf[i] + R(a21) * h * k[0][i];
                    }
                } else {
#pragma unroll kStateUnroll
                    for (int i = 0; i < NS; ++i) {
                        R acc = tableau_a<R>(sg, 0) * k[0][i];
                        for (int j = 1; j < sg; ++j) acc += tableau_a<R>(sg, j) * k[j][i];
                        if constexpr (D) yt[i] = y[i] + dx * acc;
                        else yt[i] = yf[i] + h * acc;
                    }
                }
                rhs_eval<M, SV, R, KS>(x + kRkfC[sg] * dx, yt, &K, H, k[sg], tissue, &st);
                evals += 1;
            }
            s0 = 1;
            // 5th-order solution and the embedded error (RKF45::solve), then
            // ODESolver::normalizeError
            double maxerr = 0.0;
            R maxerr_r = R(0);
            worst = -1;
#pragma unroll kStateUnroll
            for (int i = 0; i < NS; ++i) {
                if constexpr (D) {
                    y5w[i] = y[i] + dx * (b1 * k[0][i] + b3 * k[2][i] + b4 * k[3][i]
                                          + b5 * k[4][i] + b6 * k[5][i]);
                    y5f[i] = y5w[i];
                } else {
                    R incr = h * (R(b1) * k[0][i] + R(b3) * k[2][i] + R(b4) * k[3][i]
                                  + R(b5) * k[4][i] + R(b6) * k[5][i]);
                    // slow states accumulate in FP64, gates in FP32
                    if (is_wide<M::WIDE_MASK>(i)) {
                        y5w[i] = y[i] + double(incr);
                        y5f[i] = R(y5w[i]);
                    } else {
                        y5f[i] = yf[i] + incr;
                    }
                }
            }
#pragma unroll kStateUnroll
            for (int i = 0; i < NS; ++i) {
                if constexpr (D) {
                    double e_i = dx * (e1 * k[0][i] + e3 * k[2][i] + e4 * k[3][i]
                                       + e5 * k[4][i] + e6 * k[5][i]);
                    double a = fabs(y[i]), b = fabs(y5w[i]);
                    double tol = s.abs_tol + s.rel_tol * (a > b ? a : b);
                    double e = fabs(e_i) / tol;
                    if (e > maxerr) { maxerr = e; worst = i; }
                } else {
                    R e_i = h * (R(e1) * k[0][i] + R(e3) * k[2][i] + R(e4) * k[3][i]
                                 + R(e5) * k[4][i] + R(e6) * k[5][i]);
                    // FP32 round-off of the embedded difference (and of the
                    // stage derivatives feeding it) is not error the step
                    // size can remove: count it as tolerance, otherwise a
                    // tiny absTol drives dx towards zero
                    R noise = R(kFp32NoiseUlps * 1.1920929e-07) * h
                              * (fabsf(R(e1) * k[0][i]) + fabsf(R(e3) * k[2][i])
                                 + fabsf(R(e4) * k[3][i]) + fabsf(R(e5) * k[4][i])
                                 + fabsf(R(e6) * k[5][i]));
                    R a = fabsf(yf[i]), b = fabsf(y5f[i]);
                    R tol = R(s.abs_tol) + R(s.rel_tol) * (a > b ? a : b) + noise;
                    R e = fabsf(e_i) / tol;
                    if (e > maxerr_r) { maxerr_r = e; worst = i; }
                }
            }
            err = D ? maxerr : double(maxerr_r);
            if (!(err > 1)) break;
            double scale;
            if constexpr (D) scale = s.safe_scale * pow(err, -s.alpha_dec);
            else scale = double(float(s.safe_scale) * powf(float(err), -float(s.alpha_dec)));
            if (scale < s.min_scale) scale = s.min_scale;
            dx *= scale;
            if (dx < 1e-300) {
                if (why) *why = IonicFailure{2, x, dx, err, worst >= 0 ? y[worst] : 0.0, worst, n};
                return -1;
            }
        }
        if (why) { why->x = x; why->dx = dx; why->err = err; why->worst = worst; why->steps = n; }
        x = exact_add(x, dx);
#pragma unroll kStateUnroll
        for (int i = 0; i < NS; ++i) {
            yf[i] = y5f[i];
            if (D || is_wide<M::WIDE_MASK>(i)) y[i] = y5w[i];
        }
        if (err > s.inc_threshold) {
            double scale;
            if constexpr (D) scale = s.safe_scale * pow(err, -s.alpha_inc);
            else scale = double(float(s.safe_scale) * powf(float(err), -float(s.alpha_inc)));
            if (scale > s.max_scale) scale = s.max_scale;
            step_dx = scale * dx;
        } else {
            step_dx = s.safe_scale * s.max_scale * dx;
        }
        // --- back in ODESolver::solve
        if (exact_mul(exact_sub(x, xe), exact_sub(xe, xs)) >= 0) {
            if (n > 0 && last) step_dx = dx_try0;
            dx_try = step_dx;
            return n + 1;
        }
    }
    if (why) {
        why->reason = 1;
        why->value = why->worst >= 0 ? y[why->worst] : 0.0;
    }
    return -1;
}

// Tissue / single-cell ionic update of one PDE step for all cells (the plain
// FP64 form; the mixed form runs ionic_mixed_kernel).
// TISSUE > 0: every cell has that tissue flag and no per-cell scales, and the
// constants are compile-time values; TISSUE == 0: constants are evaluated per
// cell (per-cell tissue flags or conductance scales).
template <class M, bool FP64, bool SV, int TISSUE>
__global__ void __launch_bounds__(128, CFG_IONIC_MIN_BLOCKS) ionic_step_kernel(IonicLaunch p)
{
    using R = typename std::conditional<FP64, double, float>::type;
    using L = Layout<M, FP64>;
    constexpr int NS = M::NS;
    unsigned evals = 0;
    const long long end = p.first + p.count;
    for (long long c = p.first + (long long)blockIdx.x * blockDim.x + threadIdx.x; c < end;
         c += (long long)gridDim.x * blockDim.x) {
        const long long cell = p.perm ? p.perm[c] : c;
        const double t0 = p.t_dev ? p.t_dev[0] : p.t0;
        double ts, te, dtm;
        model_times<M>(t0, p.dt, ts, te, dtm);

        CellState<M, R> cs;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            if (FP64 || is_wide<M::WIDE_MASK>(i)) {
                cs.y[i] = p.yw[(long long)L::slot(i) * p.n + c];
                cs.yf[i] = R(cs.y[i]);
            } else {
                cs.yf[i] = p.yn[(long long)L::slot(i) * p.n + c];
            }
        }
        if (!SV) {
            cs.y[0] = vm_to_state0<M::VM_MAP>(p.vm[cell]);
            cs.yf[0] = R(cs.y[0]);
        }
        double step = p.step[c];
        if (dtm < step) step = dtm;   // step = min(step, dt_model)

        R k[6][NS];
#pragma unroll
        for (int j = 0; j < 6; ++j)
#pragma unroll
            for (int i = 0; i < NS; ++i) k[j][i] = R(0);

        IonicFailure why;
        long long nsub;
        R iion;
        int tissue = TISSUE;
        Hoisted<M, R> H;
        if constexpr (TISSUE > 0) {
            const ConstFold<R, M, TISSUE> K{};
            if constexpr (!SV) M::template hoist_vm<R>(cs.yf[0], K, TISSUE, H.v);
            nsub = rkf45_solve<M, SV, R>(ts, te, cs, step, k, K, TISSUE, p.stim, p.ode, evals,
                                         &why, H.v);
            // computeVariables at tEnd: the rates body computes the same Iion
            iion = rhs_eval<M, SV, R, ConstFold<R, M, TISSUE>>(te, cs.yf, &K, H.v, k[0], TISSUE,
                                                               &p.stim);
        } else {
            tissue = p.tissue_cell ? int(p.tissue_cell[c]) : p.tissue;
            double C[M::NC] = {};   // the reference zero-fills CONSTANTS
            double yinit[NS] = {};
            double sc[6];
            const double* scp = nullptr;
            if (p.scales) {
#pragma unroll
                for (int j = 0; j < 6; ++j) sc[j] = p.scales[j * p.scale_stride + c];
                scp = sc;
            }
            M::init(C, yinit, tissue, scp);
            const ConstView<R> K{C};
            if constexpr (!SV) M::template hoist_vm<R>(cs.yf[0], K, tissue, H.v);
            nsub = rkf45_solve<M, SV, R>(ts, te, cs, step, k, K, tissue, p.stim, p.ode, evals,
                                         &why, H.v);
            iion = rhs_eval<M, SV, R, ConstView<R>>(te, cs.yf, &K, H.v, k[0], tissue, &p.stim);
        }
        (void)tissue;
        evals += 1;
        if (nsub < 0) {
            const int prev = atomicOr(p.status, CFG_ERR_ODE_STEPS);
            if (p.fail_record && !(prev & CFG_ERR_ODE_STEPS)) {
                // the thread that raised the flag first writes the record
                double* r = p.fail_record;
                r[0] = double(cell); r[1] = why.reason; r[2] = why.x; r[3] = why.dx;
                r[4] = why.worst; r[5] = why.err; r[6] = why.value; r[7] = double(why.steps);
            }
        }
        const double im = double(iion) * M::IION_SCALE;
        if (!isfinite(im)) atomicOr(p.status, CFG_ERR_NONFINITE);
        if (p.im) p.im[cell] = im;

#pragma unroll
        for (int i = 0; i < NS; ++i) {
            if (FP64 || is_wide<M::WIDE_MASK>(i)) p.yw[(long long)L::slot(i) * p.n + c] = cs.y[i];
            else p.yn[(long long)L::slot(i) * p.n + c] = cs.yf[i];
        }
        p.step[c] = step;
    }
    if (p.rhs_evals) {
        unsigned long long v = evals;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(p.rhs_evals, v);
    }
}

// Initial states and constants for n cells (initConsts per cell).
template <class M, bool FP64>
__global__ void ionic_init_kernel(long long n, int tissue, const unsigned char* tissue_cell,
                                  const double* scales, long long scale_stride, double init_step,
                                  double* yw, float* yn, double* step)
{
    using L = Layout<M, FP64>;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const int t = tissue_cell ? int(tissue_cell[c]) : tissue;
    double C[M::NC] = {};
    double y[M::NS] = {};   // states initConsts leaves unset are zero
    double sc[6];
    const double* scp = nullptr;
    if (scales) {
        for (int j = 0; j < 6; ++j) sc[j] = scales[j * scale_stride + c];
        scp = sc;
    }
    M::init(C, y, t, scp);
#pragma unroll
    for (int i = 0; i < M::NS; ++i) {
        if (FP64) {
            yw[(long long)L::slot(i) * n + c] = y[i];
        } else if (is_wide<M::WIDE_MASK>(i)) {
            // mixed form: the slot holds the FP32 pair (hi, lo) of the state
            const float hi = float(y[i]);
            reinterpret_cast<float2*>(yw)[(long long)L::slot(i) * n + c] =
                make_float2(hi, float(y[i] - double(hi)));
        } else {
            yn[(long long)L::slot(i) * n + c] = float(y[i]);
        }
    }
    step[c] = init_step;
}

}  // namespace cfg
