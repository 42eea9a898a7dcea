// Mixed-precision ionic step with the RKF45 stage data in shared memory.
//
// The six stage derivatives, the stage input and the state of one cell
// (~1.2 KB for ORd) do not fit in registers; as per-thread local arrays they
// overflow the L1 at useful occupancy and round-trip through L2/DRAM.  Here
// each thread owns a slice of dynamic shared memory instead:
//
//   Y[NSP]   states in FP32 (the high part for the slow states)
//   T[NSP]   stage input
//   K[5][NSP] stage slots: k1..k5, then (after the stage-6 input is formed)
//            P = sum b_j k_j (j<6), E = sum e_j k_j (j<6), k6, and the FP32
//            round-off bound of E
//   LO[NW]   low parts of the slow (WIDE_MASK) states
//
// The slice length is odd, so the 32 threads of a warp touching the same
// element hit 32 different banks.
//
// Arithmetic: right-hand sides, stage sums, error norm and step control in
// FP32 (with step control relative to the start of the PDE step, which keeps
// its FP32 resolution); slow states as unevaluated FP32 sums hi + lo
// (Knuth two-sum), which keeps ~48 bits for concentrations whose increments
// are below the FP32 resolution of their values; in global memory each slow
// state is that (hi, lo) pair in the 8 bytes of its slot.  FP64 is left only
// for the PDE fields (Vm in, Iion out) and the persistent step, a handful of
// operations per cell: GB300 issues FP64 at 1/64 of the FP32 rate, so FP64
// inside the RKF45 loop, or on every state, would cost as much as the model
// body itself.
#pragma once

#include "ionic_kernels.cuh"

namespace cfg {

namespace mixed {

// dynamic shared memory per SM available to blocks (228 KB) and the
// per-block reservation
constexpr int kSmemPerSm = 233472;
constexpr int kSmemReserve = 1024;

constexpr int blocks_per_sm(int block, int len)
{
    return kSmemPerSm / (block * len * 4 + kSmemReserve);
}

// Per thread: the five stage slots in shared memory (the state Y and the
// low parts of the slow states live in registers).
template <class M>
struct Slice {
    static constexpr int NSP = M::NS | 1;   // odd stride for each array
    static constexpr int NW = Layout<M, false>::n_wide();
    static constexpr int NWA = NW > 0 ? NW : 1;
    static constexpr int raw = 5 * NSP;     // five stage slots
    static constexpr int len = raw | 1;       // odd slice length: conflict-free
    // 64 threads per block unless 32 keeps more threads resident per SM
    static constexpr int block =
        32 * blocks_per_sm(32, len) > 64 * blocks_per_sm(64, len) ? 32 : 64;
    static constexpr int fit = blocks_per_sm(block, len);
#ifdef CFG_MIXED_MIN_BLOCKS
    // register budget of the model (its right-hand side plus the state in
    // registers) when that, not shared memory, limits the resident blocks
    static constexpr int want = fit < CFG_MIXED_MIN_BLOCKS ? fit : CFG_MIXED_MIN_BLOCKS;
#else
    static constexpr int want = fit;
#endif
    static constexpr int min_blocks = want < 1 ? 1 : (want > 16 ? 16 : want);
    static constexpr int smem_bytes = block * len * 4;
};

constexpr float fa21 = float(rkf::a21);
constexpr float fa31 = float(rkf::a31), fa32 = float(rkf::a32);
constexpr float fa41 = float(rkf::a41), fa42 = float(rkf::a42), fa43 = float(rkf::a43);
constexpr float fa51 = float(rkf::a51), fa52 = float(rkf::a52), fa53 = float(rkf::a53),
                fa54 = float(rkf::a54);
constexpr float fa61 = float(rkf::a61), fa62 = float(rkf::a62), fa63 = float(rkf::a63),
                fa64 = float(rkf::a64), fa65 = float(rkf::a65);
constexpr float fb1 = float(rkf::b1), fb3 = float(rkf::b3), fb4 = float(rkf::b4),
                fb5 = float(rkf::b5), fb6 = float(rkf::b6);
constexpr float fe1 = float(rkf::e1), fe3 = float(rkf::e3), fe4 = float(rkf::e4),
                fe5 = float(rkf::e5), fe6 = float(rkf::e6);
CFG_D __forceinline__ float stage_c(int s)
{
    switch (s) {
    case 1: return float(rkf::c2);
    case 2: return float(rkf::c3);
    case 3: return float(rkf::c4);
    case 4: return float(rkf::c5);
    case 5: return float(rkf::c6);
    default: return 0.0f;
    }
}

// hi + lo += d, renormalised (two-sum of hi and d, low parts added after)
CFG_D __forceinline__ void add_wide(float& hi, float& lo, float d)
{
    const float s = hi + d;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (d - bp);
    const float l = lo + err;
    const float h = s + l;
    lo = l - (h - s);
    hi = h;
}

// Stage input T = Y + h * sum_j a_sj k_j for stages 2..5 (s = 1..4); T is
// the stage's own slot K + s P, where its derivative is then evaluated in
// place.
template <class M>
CFG_D __forceinline__ void stage_input(int s, float h, const float (&Y)[M::NS], float* T,
                                       const float* K)
{
    constexpr int NS = M::NS, P = Slice<M>::NSP;
    switch (s) {
    case 1:
#pragma unroll
        for (int i = 0; i < NS; ++i) T[i] = Y[i] + h * (fa21 * K[i]);
        break;
    case 2:
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            float acc = fa31 * K[i];
            acc += fa32 * K[P + i];
            T[i] = Y[i] + h * acc;
        }
        break;
    case 3:
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            float acc = fa41 * K[i];
            acc += fa42 * K[P + i];
            acc += fa43 * K[2 * P + i];
            T[i] = Y[i] + h * acc;
        }
        break;
    default:
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            float acc = fa51 * K[i];
            acc += fa52 * K[P + i];
            acc += fa53 * K[2 * P + i];
            acc += fa54 * K[3 * P + i];
            T[i] = Y[i] + h * acc;
        }
        break;
    }
}

// Stage-6 input into slot 3 (k4's, read first), and P, E and the round-off
// bound of E into slots 1, 2, 4 (k2 and the old k3..k5 are not needed
// afterwards: b2 = e2 = 0).
template <class M>
CFG_D __forceinline__ void stage6_input(float h, const float (&Y)[M::NS], float* T, float* K)
{
    constexpr int NS = M::NS, P = Slice<M>::NSP;
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        const float k1 = K[i], k2 = K[P + i], k3 = K[2 * P + i], k4 = K[3 * P + i],
                    k5 = K[4 * P + i];
        float acc = fa61 * k1;
        acc += fa62 * k2;
        acc += fa63 * k3;
        acc += fa64 * k4;
        acc += fa65 * k5;
        T[i] = Y[i] + h * acc;
        K[P + i] = fb1 * k1 + fb3 * k3 + fb4 * k4 + fb5 * k5;
        K[2 * P + i] = fe1 * k1 + fe3 * k3 + fe4 * k4 + fe5 * k5;
        K[4 * P + i] = fabsf(fe1 * k1) + fabsf(fe3 * k3) + fabsf(fe4 * k4) + fabsf(fe5 * k5);
    }
}

// ODESolver::solve over [xs, xs + D] (RKF45 inside adaptiveSolver::solve),
// then the right-hand side at the end of the interval for the current.
// Returns accepted substeps, or -1 on maxSteps overflow / step underflow.
// Every stage's derivative is evaluated in place, in the slot that holds the
// stage input (the generated right-hand side reads every state before it
// writes a derivative); in tissue mode the slot's state-0 entry, which the
// model leaves unassigned or sets to zero, is then zeroed.
// State i of Y at a run-time index (for failure records), without indexing
// the register array at run time.
template <int NS>
CFG_D __forceinline__ double state_at(const float (&Y)[NS], int i)
{
    float v = 0.0f;
#pragma unroll
    for (int k = 0; k < NS; ++k)
        if (k == i) v = Y[k];
    return double(v);
}

template <class M, bool SV, class KS>
CFG_D __forceinline__ long long solve(double xs, double xe, float D, float (&Y)[M::NS], float* K,
                                      float (&LO)[Slice<M>::NWA],
                                      float& dx_try, const KS& Kc, int tissue,
                                      const CfgStimulus& st, const OdeSettings& s,
                                      unsigned& evals, IonicFailure& why, float& iion,
                                      const float* H = nullptr)
{
    constexpr int NS = M::NS, P = Slice<M>::NSP;
    const float abs_tol = float(s.abs_tol), rel_tol = float(s.rel_tol);
    const float safe = float(s.safe_scale), min_scale = float(s.min_scale),
                max_scale = float(s.max_scale), a_inc = float(s.alpha_inc),
                a_dec = float(s.alpha_dec), inc_thr = float(s.inc_threshold);
    constexpr float noise_ulps = float(kFp32NoiseUlps * 1.1920929e-07);

    float u = 0.0f;            // x - xs
    float u_prev = 0.0f;
    float step_dx = dx_try;
    float dx = 0.0f, dx_try0 = 0.0f;
    bool last = false, to_end = false;
    long long n = 0;           // substep (ODESolver::solve loop index)
    int sg = 0;                // next evaluation: stage 0..5, 6 = current at xs + D
    bool begin = true;
    float err = 0.0f;
    int worst = -1;
    for (;;) {
        if (begin) {
            if (n >= s.max_steps) {
                // the last accepted substep, as ODESolver reports it
                why.reason = 1;
                why.x = xs + double(u_prev); why.dx = dx; why.err = err; why.worst = worst;
                why.value = worst >= 0 ? state_at(Y, worst) : 0.0;
                why.steps = n - 1;
                return -1;
            }
            begin = false;
            dx_try0 = step_dx;
            to_end = false;
            if (u + step_dx > D) {
                last = true;
                step_dx = D - u;
            }
            if (u + step_dx >= D) to_end = true;
            dx = step_dx;
            sg = 0;
        }
        const float h = dx;
        float* out;
        if (sg == 0) {
            // k1 = f(y), evaluated in slot 0 from a copy of y
            out = K;
#pragma unroll
            for (int i = 0; i < NS; ++i) out[i] = Y[i];
        } else if (sg < 5) {
            out = K + sg * P;
            stage_input<M>(sg, h, Y, out, K);
        } else if (sg == 5) {
            out = K + 3 * P;
            stage6_input<M>(h, Y, out, K);
        } else {
            // the current at the end, from y in a free slot
            out = K + P;
#pragma unroll
            for (int i = 0; i < NS; ++i) out[i] = Y[i];
        }
        const float* in = out;
        double t = 0.0;
        if constexpr (SV) t = sg == 6 ? xe : xs + double(u) + double(stage_c(sg) * h);
        float r;
        if constexpr (!SV && M::NH > 0)
            r = M::template rates_tissue<float>(t, ArrayView<float>{in}, Kc, ArrayView<float>{H},
                                                out, tissue, st);
        else
            r = M::template rates<float, SV>(t, ArrayView<float>{in}, Kc, out, tissue, st);
        if constexpr (!SV) out[0] = 0.0f;
        ++evals;
        if (sg == 6) {
            iion = r;
            return n;
        }
        if (sg < 5) {
            ++sg;
            continue;
        }
        // --- RKF45::solve error estimate and ODESolver::normalizeError
        float maxerr = 0.0f;
        bool finite = true;
        worst = -1;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            const float k6 = K[3 * P + i];
            const float y0 = Y[i];
            const float y5 = y0 + h * (K[P + i] + fb6 * k6);
            const float e_i = h * (K[2 * P + i] + fe6 * k6);
            const float noise = noise_ulps * h * (K[4 * P + i] + fabsf(fe6 * k6));
            const float a = fabsf(y0), b = fabsf(y5);
            const float tol = abs_tol + rel_tol * (a > b ? a : b) + noise;
            const float e = fabsf(e_i) / tol;
            if (e > maxerr) { maxerr = e; worst = i; }
            if (!(e == e)) { finite = false; worst = i; }
        }
        err = finite ? maxerr : __int_as_float(0x7fc00000);
        // A trial stage can overflow FP32 (exp of an overshooting voltage):
        // a non-finite error norm rejects the step with the smallest scale,
        // where the FP64 form would see a large but finite error.
        if (!(err <= 1.0f)) {
            float scale = err == err ? safe * __powf(err, -a_dec) : min_scale;
            if (!(scale >= min_scale)) scale = min_scale;
            dx *= scale;
            if (!(dx >= 1e-37f)) {
                why.reason = 2;
                why.x = xs + double(u); why.dx = dx; why.err = err; why.worst = worst;
                why.value = worst >= 0 ? state_at(Y, worst) : 0.0;
                why.steps = n;
                return -1;
            }
            sg = 1;   // k1 = f(y) is reused
            continue;
        }
        // --- accept: y = y5 (slow states as hi + lo)
        int w = 0;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            const float incr = h * (K[P + i] + fb6 * K[3 * P + i]);
            if (is_wide<M::WIDE_MASK>(i)) {
                float hi = Y[i], lo = LO[w];
                add_wide(hi, lo, incr);
                Y[i] = hi;
                LO[w] = lo;
                ++w;
            } else {
                Y[i] = Y[i] + incr;
            }
        }
        u_prev = u;
        u = (to_end && dx == step_dx) ? D : u + dx;
        if (err > inc_thr) {
            float scale = safe * __powf(err, -a_inc);
            if (scale > max_scale) scale = max_scale;
            step_dx = scale * dx;
        } else {
            step_dx = safe * max_scale * dx;
        }
        if (u >= D) {
            if (n > 0 && last) step_dx = dx_try0;
            dx_try = step_dx;
            ++n;
            sg = 6;
            continue;
        }
        ++n;
        begin = true;
    }
}

}  // namespace mixed

// Mixed-form tissue / single-cell step with shared-memory stage data.
// TISSUE > 0: uniform tissue with compile-time constants; TISSUE == 0:
// constants per cell (per-cell tissue flags or conductance scales).
template <class M, bool SV, int TISSUE>
__global__ void __launch_bounds__(mixed::Slice<M>::block, mixed::Slice<M>::min_blocks)
ionic_mixed_kernel(IonicLaunch p)
{
    using S = mixed::Slice<M>;
    using L = Layout<M, false>;
    constexpr int NS = M::NS, P = S::NSP;
    extern __shared__ float cfg_mixed_smem[];
    float* K = cfg_mixed_smem + threadIdx.x * S::len;
    float Y[NS];
    float LO[S::NWA];
    unsigned evals = 0;
    const long long end = p.first + p.count;
    for (long long c = p.first + (long long)blockIdx.x * blockDim.x + threadIdx.x; c < end;
         c += (long long)gridDim.x * blockDim.x) {
        const long long cell = p.perm ? p.perm[c] : c;
        const double t0 = p.t_dev ? p.t_dev[0] : p.t0;
        double ts, te, dtm;
        model_times<M>(t0, p.dt, ts, te, dtm);
        // derivatives the model does not assign (Vm in tissue mode) are zero
        // in every stage slot, as in a zero-filled dydt array
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
        if constexpr (!SV) {
            // Vm from the PDE field, split into hi + lo
            const double v = vm_to_state0<M::VM_MAP>(p.vm[cell]);
            const float hi = float(v);
            Y[0] = hi;
            if (is_wide<M::WIDE_MASK>(0)) LO[0] = float(v - double(hi));
        }
        // step = min(step, dt_model); rounding to FP32 keeps the order
        float dx_try = fminf(float(p.step[c]), float(dtm));

        IonicFailure why;
        long long nsub;
        float iion = 0.0f;
        // tissue mode: the membrane-potential-only values, once per cell and step
        Hoisted<M, float> H;
        if constexpr (TISSUE > 0) {
            const ConstFold<float, M, TISSUE> Kc{};
            if constexpr (!SV) M::template hoist_vm<float>(Y[0], Kc, TISSUE, H.v);
            nsub = mixed::solve<M, SV>(ts, te, float(dtm), Y, K, LO, dx_try, Kc, TISSUE, p.stim,
                                       p.ode, evals, why, iion, H.v);
        } else {
            const int tissue = p.tissue_cell ? int(p.tissue_cell[c]) : p.tissue;
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
            const ConstView<float> Kc{C};
            if constexpr (!SV) M::template hoist_vm<float>(Y[0], Kc, tissue, H.v);
            nsub = mixed::solve<M, SV>(ts, te, float(dtm), Y, K, LO, dx_try, Kc, tissue, p.stim,
                                       p.ode, evals, why, iion, H.v);
        }
        if (nsub < 0) {
            const int prev = atomicOr(p.status, CFG_ERR_ODE_STEPS);
            if (p.fail_record && !(prev & CFG_ERR_ODE_STEPS)) {
                double* r = p.fail_record;
                r[0] = double(cell); r[1] = why.reason; r[2] = why.x; r[3] = why.dx;
                r[4] = why.worst; r[5] = why.err; r[6] = why.value; r[7] = double(why.steps);
            }
        }
        const double im = double(iion) * M::IION_SCALE;
        if (!isfinite(im)) atomicOr(p.status, CFG_ERR_NONFINITE);
        if (p.im) p.im[cell] = im;
        float2* yw2o = reinterpret_cast<float2*>(p.yw);
        w = 0;
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            if (is_wide<M::WIDE_MASK>(i)) {
                yw2o[(long long)L::slot(i) * p.n + c] = make_float2(Y[i], LO[w++]);
            } else {
                p.yn[(long long)L::slot(i) * p.n + c] = Y[i];
            }
        }
        p.step[c] = double(dx_try);
    }
    if (p.rhs_evals) {
        unsigned long long v = evals;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(p.rhs_evals, v);
    }
}

}  // namespace cfg
