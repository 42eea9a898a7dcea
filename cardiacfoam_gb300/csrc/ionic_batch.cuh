// Batched single cells: SingleCellSolver::evolve (singleCellSolver.C:179-230)
// for many independently parameterised cells (conductance scales, S1/S2
// protocol, run length) in one persistent launch, with the restitution
// post-processing (APD90 and peak Ca per beat, postProcessing_restCurves.py)
// done on the fly.
//
// Work stealing: every thread takes the next cell from a queue counter,
// advances it by up to `chunk` solver steps, stores it and takes another;
// finished cells are skipped.  The host relaunches until no cell is left,
// so uneven run lengths do not idle the GPU and no launch runs for long.
//
// Per-cell scales change only a handful of constants (the scaled
// conductances and what initConsts derives from them); those come from a
// per-cell vector, every other constant is the tissue's compile-time value.
#pragma once

#include "apd.cuh"
#include "ionic_kernels.cuh"
#include "ionic_mixed.cuh"

namespace cfg {

// Constants of a uniform tissue with the scale-dependent ones per cell.
template <class R, class M, int T>
struct ScaledFold {
    const R* dep;   // [NSD] this cell's scale-dependent constants
    CFG_D __forceinline__ R operator()(int i) const
    {
        return M::sd_slot(i) >= 0 ? dep[M::sd_slot(i)] : R(M::template constant<T>(i));
    }
};

struct BatchLaunch {
    long long n;
    double dt;                      // SingleCellSolver deltaT [s]
    long long chunk;                // solver steps per claim
    OdeSettings ode;
    const CfgStimulus* stim;        // [n]
    const long long* n_steps;       // [n] solver steps of each cell
    long long* done;                // [n] steps taken
    double* t;                      // [n] time [s]
    double* yw;                     // wide states [NW][n] (FP64, or (hi, lo) pairs)
    float* yn;                      // narrow states [NN][n] (mixed form)
    double* step;                   // [n] persistent ODE step [model time]
    double* dep;                    // [NSD][n] scale-dependent constants
    ApdTracker* apd;                // [n]
    double* ring_t;                 // [ring][n]
    double* ring_v;
    ApdParams apdp;
    double* trace;                  // [trace_cells][2][trace_cap]: Vm [mV], Ca
    long long trace_cells, trace_cap;
    unsigned long long* queue;      // next cell to claim (zeroed before a launch)
    long long* active;              // cells not finished
    int* status;
    unsigned long long* rhs_evals;
    double* fail_record;
};

template <class M>
CFG_D __forceinline__ double state0_to_mv(double u)
{
    if constexpr (M::VM_MAP == CFG_VM_ALIEV) return u * 100.0 - 80.0;
    else if constexpr (M::VM_MAP == CFG_VM_BUENO) return u * 85.7 - 84.0;
    else if constexpr (M::VM_MAP == CFG_VM_IDENTITY) return u;
    else return u;
}

// sample of the cell after a step, its trace entry and the beat detector
template <class M>
CFG_D __forceinline__ void batch_sample(const BatchLaunch& p, long long c, long long k,
                                        ApdTracker& a, double t, double v0, double ca)
{
    const double v = state0_to_mv<M>(v0);
    apd_sample(a, p.apdp, t, v, ca, p.ring_t + c, p.ring_v + c, p.n);
    if (c < p.trace_cells && k < p.trace_cap) {
        p.trace[(c * 2 + 0) * p.trace_cap + k] = v;
        p.trace[(c * 2 + 1) * p.trace_cap + k] = ca;
    }
}

CFG_D __forceinline__ void batch_fail(const BatchLaunch& p, long long c, const IonicFailure& why)
{
    const int prev = atomicOr(p.status, CFG_ERR_ODE_STEPS);
    if (p.fail_record && !(prev & CFG_ERR_ODE_STEPS)) {
        double* r = p.fail_record;
        r[0] = double(c); r[1] = why.reason; r[2] = why.x; r[3] = why.dx;
        r[4] = why.worst; r[5] = why.err; r[6] = why.value; r[7] = double(why.steps);
    }
}

// Initial states (initConsts with the cell's scales), its scale-dependent
// constants, and sample 0 of the trace.
template <class M, bool FP64>
__global__ void batch_init_kernel(BatchLaunch p, const double* scales, int tissue,
                                  double init_step)
{
    using L = Layout<M, FP64>;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= p.n) return;
    double C[M::NC] = {};
    double y[M::NS] = {};   // states initConsts leaves unset are zero
    double sc[6];
    const double* scp = nullptr;
    if (scales) {
        for (int j = 0; j < 6; ++j) sc[j] = scales[j * p.n + c];
        scp = sc;
    }
    M::init(C, y, tissue, scp);
    for (int k = 0; k < M::NSD; ++k) p.dep[k * p.n + c] = C[M::sd_const(k)];
#pragma unroll
    for (int i = 0; i < M::NS; ++i) {
        if (FP64) {
            p.yw[(long long)L::slot(i) * p.n + c] = y[i];
        } else if (is_wide<M::WIDE_MASK>(i)) {
            const float hi = float(y[i]);
            reinterpret_cast<float2*>(p.yw)[(long long)L::slot(i) * p.n + c] =
                make_float2(hi, float(y[i] - double(hi)));
        } else {
            p.yn[(long long)L::slot(i) * p.n + c] = float(y[i]);
        }
    }
    p.step[c] = init_step;
    p.t[c] = 0.0;
    p.done[c] = 0;
    ApdTracker a{};
    a.last_apd = cfg_nan();
    a.last_ca = cfg_nan();
    a.last_t_up = cfg_nan();
    batch_sample<M>(p, c, 0, a, 0.0, y[0], M::CA_STATE >= 0 ? y[M::CA_STATE] : 0.0);
    if (p.n_steps[c] <= 0) apd_end(a, p.apdp);   // nothing to integrate
    p.apd[c] = a;
}

// FP64 plain form: per-thread stage arrays, as the tissue kernel.
template <class M, int T>
__global__ void __launch_bounds__(128) batch_fp64_kernel(BatchLaunch p)
{
    using L = Layout<M, true>;
    constexpr int NS = M::NS;
    unsigned evals = 0;
    double k6[6][NS];
    for (;;) {
        const long long c = (long long)atomicAdd(p.queue, 1ull);
        if (c >= p.n) break;
        long long k = p.done[c];
        const long long total = p.n_steps[c];
        if (k >= total) continue;
        // derivatives a model does not assign stay zero, as in a zeroed dydt
        for (int j = 0; j < 6; ++j)
            for (int i = 0; i < NS; ++i) k6[j][i] = 0.0;
        CellState<M, double> cs;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            cs.y[i] = p.yw[(long long)L::slot(i) * p.n + c];
            cs.yf[i] = cs.y[i];
        }
        double dep[M::NSD > 0 ? M::NSD : 1];
#pragma unroll
        for (int j = 0; j < M::NSD; ++j) dep[j] = p.dep[j * p.n + c];
        const ScaledFold<double, M, T> Kc{dep};
        const CfgStimulus stim = p.stim[c];
        ApdTracker a = p.apd[c];
        double t = p.t[c];
        double step = p.step[c];
        const long long k_end = total < k + p.chunk ? total : k + p.chunk;
        bool failed = false;
        for (; k < k_end; ++k) {
            const double t_new = t + p.dt;   // runTime++
            double ts, te, dtm;
            model_times<M>(t_new - p.dt, p.dt, ts, te, dtm);
            if (dtm < step) step = dtm;
            IonicFailure why;
            const long long nsub =
                rkf45_solve<M, true, double>(ts, te, cs, step, k6, Kc, T, stim, p.ode, evals, &why);
            if (nsub < 0) {
                batch_fail(p, c, why);
                failed = true;
                break;
            }
            t = t_new;
            batch_sample<M>(p, c, k + 1, a, t, cs.y[0],
                            M::CA_STATE >= 0 ? cs.y[M::CA_STATE] : 0.0);
        }
#pragma unroll
        for (int i = 0; i < NS; ++i) p.yw[(long long)L::slot(i) * p.n + c] = cs.y[i];
        p.step[c] = step;
        p.t[c] = t;
        if (failed) k = total;
        p.done[c] = k;
        if (k >= total) {
            apd_end(a, p.apdp);
            atomicAdd((unsigned long long*)p.active, (unsigned long long)-1ll);
        }
        p.apd[c] = a;
    }
    if (p.rhs_evals) {
        unsigned long long v = evals;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(p.rhs_evals, v);
    }
}

// Mixed form: stage data in shared memory, FP32 arithmetic, slow states as
// (hi, lo) pairs (see ionic_mixed.cuh).
template <class M, int T>
__global__ void __launch_bounds__(mixed::Slice<M>::block, mixed::Slice<M>::min_blocks)
batch_mixed_kernel(BatchLaunch p)
{
    using S = mixed::Slice<M>;
    using L = Layout<M, false>;
    constexpr int NS = M::NS, P = S::NSP;
    extern __shared__ float cfg_batch_smem[];
    float* K = cfg_batch_smem + threadIdx.x * S::len;
    float Y[NS];
    float LO[S::NWA];
    unsigned evals = 0;
    for (;;) {
        const long long c = (long long)atomicAdd(p.queue, 1ull);
        if (c >= p.n) break;
        long long k = p.done[c];
        const long long total = p.n_steps[c];
        if (k >= total) continue;
        for (int i = 0; i < 5 * P; ++i) K[i] = 0.0f;
        const float2* yw2 = reinterpret_cast<const float2*>(p.yw);
        int w = 0;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            if (is_wide<M::WIDE_MASK>(i)) {
                const float2 v = yw2[(long long)L::slot(i) * p.n + c];
                Y[i] = v.x;
                LO[w++] = v.y;
            } else {
                Y[i] = p.yn[(long long)L::slot(i) * p.n + c];
            }
        }
        float dep[M::NSD > 0 ? M::NSD : 1];
#pragma unroll
        for (int j = 0; j < M::NSD; ++j) dep[j] = float(p.dep[j * p.n + c]);
        const ScaledFold<float, M, T> Kc{dep};
        const CfgStimulus stim = p.stim[c];
        ApdTracker a = p.apd[c];
        double t = p.t[c];
        float dx_try = float(p.step[c]);
        const long long k_end = total < k + p.chunk ? total : k + p.chunk;
        bool failed = false;
        for (; k < k_end; ++k) {
            const double t_new = t + p.dt;
            double ts, te, dtm;
            model_times<M>(t_new - p.dt, p.dt, ts, te, dtm);
            dx_try = fminf(dx_try, float(dtm));
            IonicFailure why;
            float iion;
            const long long nsub = mixed::solve<M, true>(ts, te, float(dtm), Y, K, LO,
                                                         dx_try, Kc, T, stim, p.ode, evals,
                                                         why, iion);
            if (nsub < 0) {
                batch_fail(p, c, why);
                failed = true;
                break;
            }
            t = t_new;
            const double v0 = is_wide<M::WIDE_MASK>(0) ? double(Y[0]) + double(LO[0])
                                                       : double(Y[0]);
            double ca = 0.0;
            if constexpr (M::CA_STATE >= 0) {
                if (is_wide<M::WIDE_MASK>(M::CA_STATE)) {
                    constexpr int wc = Layout<M, false>::slot(M::CA_STATE);
                    ca = double(Y[M::CA_STATE]) + double(LO[wc]);
                } else {
                    ca = double(Y[M::CA_STATE]);
                }
            }
            batch_sample<M>(p, c, k + 1, a, t, v0, ca);
        }
        float2* yw2o = reinterpret_cast<float2*>(p.yw);
        w = 0;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            if (is_wide<M::WIDE_MASK>(i))
                yw2o[(long long)L::slot(i) * p.n + c] = make_float2(Y[i], LO[w++]);
            else
                p.yn[(long long)L::slot(i) * p.n + c] = Y[i];
        }
        p.step[c] = double(dx_try);
        p.t[c] = t;
        if (failed) k = total;
        p.done[c] = k;
        if (k >= total) {
            apd_end(a, p.apdp);
            atomicAdd((unsigned long long*)p.active, (unsigned long long)-1ll);
        }
        p.apd[c] = a;
    }
    if (p.rhs_evals) {
        unsigned long long v = evals;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(p.rhs_evals, v);
    }
}

}  // namespace cfg
