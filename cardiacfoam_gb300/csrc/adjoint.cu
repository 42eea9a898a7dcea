// Differentiable monodomain steps and their adjoint: FP64, or with the
// ionic right-hand side and its derivative in FP32 (mixed form; states,
// adjoint accumulations, PCG and the conductivity derivative stay FP64).
//
// Forward step n -> n+1 on an orthogonal mesh (implicit Euler ddt, one
// linear solve per step):
//   ionic:      (y_{n+1}, Im_{n+1}) = Phi(y_n, Vm_n; p)   fixed RKF45 substeps
//   diffusion:  A(sigma) Vm_{n+1} = C/dt Vm_n - C Im_{n+1} + V src_n
//               A = C/dt + L(sigma),  C = chi Cm V (per cell),
//               L = the Laplacian's matrix, linear in (sigma_l, sigma_t)
// Loss: J = sum over the sampled steps and probe cells of (Vm - target)^2.
//
// Reverse step n+1 -> n, given the adjoints Vbar_{n+1} (incl. the loss) and
// ybar_{n+1}:
//   A mu = Vbar_{n+1}                              (A symmetric: one PCG solve)
//   sigmabar_k -= sum_faces G_k,f (mu_P - mu_N)(Vm_P - Vm_N)_{n+1}
//   Vbar_n = C/dt mu + dPhi/dVm^T (.),  Imbar = -C mu
//   (ybar_n, pbar) from the reverse of the substeps: each stage through the
//   generated vector-Jacobian product of the right-hand side (rhs_vjp).
// The parameters are per-cell log-scales of two conductances (GNa and GK1:
// p = p0 exp(theta), so thetabar = pbar p) and the two conductivities.
//
// The forward keeps a checkpoint (states and Vm) every k steps; the reverse
// recomputes each k-step window from its checkpoint into a window buffer and
// runs back through it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "grid_sync.cuh"
#include "host_common.h"
#include "ionic_kernels.cuh"
#include "models/tnnp.cuh"
#include "models/tnnp_adjoint.cuh"

namespace cfg {
namespace adj {

using M = tnnp::Model;
constexpr int NS = M::NS;
constexpr int kMaxSub = 16;
constexpr int kBlock = 128;
constexpr int kPcgBlock = 256;

// dVm-state/dVm of the PDE -> state-0 map
template <int MAP>
constexpr double vm_map_slope()
{
    return MAP == CFG_VM_ALIEV ? 10.0 : MAP == CFG_VM_BUENO ? 1000.0 / 85.7
                                      : MAP == CFG_VM_IDENTITY ? 1.0 : 1000.0;
}

// constants of cell c from the [NC][n] table, read as R
template <class R>
struct ColView {
    const double* c;
    long long n, cell;
    CFG_D __forceinline__ R operator()(int i) const { return R(c[(long long)i * n + cell]); }
};

struct IonicArgs {
    long long n;
    int substeps, tissue;
    double t0, dtm;             // model time of the step start, model step
    const double* consts;       // [NC][n]
    double* y;                  // [NS][n] states (forward: in/out)
    const double* vm;           // [n]
    double* im;                 // [n] forward output
    // reverse
    const double* y_start;      // [NS][n] states at the step start (window)
    double* ybar;               // [NS][n] in: adjoint of the end states; out: of the start states
    const double* imbar;        // [n] adjoint of Im
    double* vbar;               // [n] += adjoint of Vm through the ionic update
    double* pbar;               // [6][n] += adjoint of the scalable conductances
};

// RKF45 tableau as arrays
struct Tableau {
    double a[6][5], b[6], c[6];
};
__device__ __forceinline__ Tableau tableau()
{
    using namespace rkf;
    return Tableau{{{0, 0, 0, 0, 0},
                    {a21, 0, 0, 0, 0},
                    {a31, a32, 0, 0, 0},
                    {a41, a42, a43, 0, 0},
                    {a51, a52, a53, a54, 0},
                    {a61, a62, a63, a64, a65}},
                   {b1, 0.0, b3, b4, b5, b6},
                   {0.0, c2, c3, c4, c5, c6}};
}

// The six stages of one RKF45 substep from the (double) state y: stage
// inputs Y_s = y + h sum_j a_sj k_j accumulated in double and handed to the
// right-hand side in R; k_s = f(Y_s) in R.
template <class R>
__device__ __forceinline__ void stages(double t, double h, const double* y,
                                       const ColView<R>& K, int tissue, R (*k)[NS],
                                       R (*Y)[NS])
{
    const Tableau T = tableau();
    const CfgStimulus none{};
    for (int s = 0; s < 6; ++s) {
        for (int i = 0; i < NS; ++i) {
            double acc = 0.0;
            for (int j = 0; j < s; ++j) acc += T.a[s][j] * double(k[j][i]);
            Y[s][i] = R(y[i] + h * acc);
            k[s][i] = R(0);           // RATES of V stay zero in tissue mode
        }
        M::rates<R, false>(t + T.c[s] * h, ArrayView<R>{Y[s]}, K, k[s], tissue, none);
    }
}

// y += h sum_s b_s k_s, in double
template <class R>
__device__ __forceinline__ void substep(double h, double* y, const R (*k)[NS])
{
    const Tableau T = tableau();
    for (int i = 0; i < NS; ++i) {
        double acc = 0.0;
        for (int s = 0; s < 6; ++s) acc += T.b[s] * double(k[s][i]);
        y[i] += h * acc;
    }
}

// Forward ionic update of one PDE step with fixed substeps.  R = double is
// the FP64 form; R = float evaluates the right-hand side in FP32 and keeps
// the states and their accumulation in FP64.
template <class R>
__global__ void __launch_bounds__(kBlock) k_ionic_forward(IonicArgs a)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n) return;
    const ColView<R> K{a.consts, a.n, c};
    double y[NS];
    for (int i = 0; i < NS; ++i) y[i] = a.y[(long long)i * a.n + c];
    y[0] = vm_to_state0<M::VM_MAP>(a.vm[c]);
    R k[6][NS], Y[6][NS];
    const double h = a.dtm / a.substeps;
    for (int j = 0; j < a.substeps; ++j) {
        stages<R>(a.t0 + j * h, h, y, K, a.tissue, k, Y);
        substep<R>(h, y, k);
    }
    R yr[NS], d[NS];
    for (int i = 0; i < NS; ++i) {
        yr[i] = R(y[i]);
        d[i] = R(0);
    }
    const CfgStimulus none{};
    const R iion = M::rates<R, false>(a.t0 + a.dtm, ArrayView<R>{yr}, K, d, a.tissue, none);
    a.im[c] = double(iion) * M::IION_SCALE;
    for (int i = 0; i < NS; ++i) a.y[(long long)i * a.n + c] = y[i];
}

// Reverse of one PDE step of the ionic update (the same arithmetic as the
// forward recomputed, then the stages backwards through rhs_vjp<R>); the
// adjoints accumulate in double.
template <class R>
__global__ void __launch_bounds__(kBlock) k_ionic_reverse(IonicArgs a)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n) return;
    const Tableau T = tableau();
    const ColView<R> K{a.consts, a.n, c};
    const double h = a.dtm / a.substeps;
    // forward again, keeping the start of every substep
    double ys[kMaxSub + 1][NS];
    for (int i = 0; i < NS; ++i) ys[0][i] = a.y_start[(long long)i * a.n + c];
    ys[0][0] = vm_to_state0<M::VM_MAP>(a.vm[c]);
    R k[6][NS], Y[6][NS];
    for (int j = 0; j < a.substeps; ++j) {
        for (int i = 0; i < NS; ++i) ys[j + 1][i] = ys[j][i];
        stages<R>(a.t0 + j * h, h, ys[j], K, a.tissue, k, Y);
        substep<R>(h, ys[j + 1], k);
    }
    double pb[6] = {0, 0, 0, 0, 0, 0};
    double yb[NS];
    for (int i = 0; i < NS; ++i) yb[i] = a.ybar[(long long)i * a.n + c];
    yb[0] = 0.0;                      // the next step overwrites state 0 with Vm
    R Yb[NS], dbR[NS], pbR[6], yr[NS];
    auto vjp = [&](double t, const R* y, const R* dbar, R ibar) {
        for (int i = 0; i < NS; ++i) Yb[i] = R(0);
        for (int q = 0; q < 6; ++q) pbR[q] = R(0);
        tnnp::rhs_vjp<R>(t, y, K, a.tissue, dbar, ibar, Yb, pbR);
        for (int q = 0; q < 6; ++q) pb[q] += double(pbR[q]);
    };
    // the current at the end of the step
    for (int i = 0; i < NS; ++i) {
        yr[i] = R(ys[a.substeps][i]);
        dbR[i] = R(0);
    }
    vjp(a.t0 + a.dtm, yr, dbR, R(a.imbar[c] * M::IION_SCALE));
    for (int i = 0; i < NS; ++i) yb[i] += double(Yb[i]);
    double kb[6][NS];
    for (int j = a.substeps - 1; j >= 0; --j) {
        stages<R>(a.t0 + j * h, h, ys[j], K, a.tissue, k, Y);
        for (int s = 0; s < 6; ++s)
            for (int i = 0; i < NS; ++i) kb[s][i] = h * T.b[s] * yb[i];
        // yb stays as the adjoint of the substep's start (identity part)
        for (int s = 5; s >= 0; --s) {
            for (int i = 0; i < NS; ++i) dbR[i] = R(kb[s][i]);
            dbR[0] = R(0);                // RATES of V are not part of the map
            vjp(a.t0 + j * h + T.c[s] * h, Y[s], dbR, R(0));
            for (int i = 0; i < NS; ++i) yb[i] += double(Yb[i]);
            for (int l = 0; l < s; ++l)
                for (int i = 0; i < NS; ++i) kb[l][i] += h * T.a[s][l] * double(Yb[i]);
        }
    }
    a.vbar[c] += yb[0] * vm_map_slope<M::VM_MAP>();
    yb[0] = 0.0;
    for (int i = 0; i < NS; ++i) a.ybar[(long long)i * a.n + c] = yb[i];
    for (int q = 0; q < 6; ++q) a.pbar[(long long)q * a.n + c] += pb[q];
}

// ------------------------------------------------------------------ PCG
struct PcgArgs {
    long long n;
    int width;
    const int* col;             // [width][n]
    const unsigned char* cnt;   // [n]
    const double* coef;         // [width][n] off-diagonal -coef
    const double* diag;         // [n]
    const double* b;            // [n]
    double* x;                  // [n] in: initial guess; out: solution
    double *r, *z, *p, *ap;     // work
    double* partial;            // [2 sets][2][blocks]
    unsigned* bar_count;
    int* bar_abort;
    double tol;                 // ||r||_2 <= tol ||b||_2
    int max_iter;
    int* iters;                 // out
    int* status;                // out: CFG_ERR_PCG when not converged or aborted
};

__device__ __forceinline__ double amul(const PcgArgs& a, long long c, const double* q)
{
    double acc = a.diag[c] * __ldcg(&q[c]);
    const int cnt = a.cnt[c];
    for (int e = 0; e < cnt; ++e) {
        const long long i = (long long)e * a.n + c;
        acc -= a.coef[i] * __ldcg(&q[a.col[i]]);
    }
    return acc;
}

// Jacobi-preconditioned CG, one cooperative launch, deterministic reductions.
__global__ void __launch_bounds__(kPcgBlock) k_pcg(PcgArgs a)
{
    const long long first = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned epoch = 0;
    int set = 0;
    double s[2] = {0.0, 0.0};
    // r = b - A x, z = D^-1 r, p = z; sums r.z and b.b
    for (long long c = first; c < a.n; c += stride) {
        const double r = a.b[c] - amul(a, c, a.x);
        const double z = r / a.diag[c];
        a.r[c] = r;
        a.z[c] = z;
        __stcg(&a.p[c], z);
        s[0] += r * z;
        s[1] += a.b[c] * a.b[c];
    }
    gsync::block_sums<kPcgBlock, 2>(a.partial, set, s);
    if (!gsync::grid_barrier(a.bar_count, a.bar_abort, epoch)) goto aborted;
    {
        double g[2];
        gsync::grid_sums<2>(a.partial, set, g);
        set ^= 1;
        double rz = g[0];
        const double bnorm = sqrt(g[1]);
        int it = 0;
        double rr = 0.0;
        {
            // initial residual norm
            double t[1] = {0.0};
            for (long long c = first; c < a.n; c += stride) t[0] += a.r[c] * a.r[c];
            gsync::block_sums<kPcgBlock, 1>(a.partial, set, t);
            if (!gsync::grid_barrier(a.bar_count, a.bar_abort, epoch)) goto aborted;
            double gt[1];
            gsync::grid_sums<1>(a.partial, set, gt);
            set ^= 1;
            rr = gt[0];
        }
        while (sqrt(rr) > a.tol * bnorm && it < a.max_iter) {
            // Ap and p.Ap
            double t[1] = {0.0};
            for (long long c = first; c < a.n; c += stride) {
                const double q = amul(a, c, a.p);
                a.ap[c] = q;
                t[0] += a.p[c] * q;
            }
            gsync::block_sums<kPcgBlock, 1>(a.partial, set, t);
            if (!gsync::grid_barrier(a.bar_count, a.bar_abort, epoch)) goto aborted;
            double gt[1];
            gsync::grid_sums<1>(a.partial, set, gt);
            set ^= 1;
            const double alpha = rz / gt[0];
            // x, r, z; r.z and r.r
            double u[2] = {0.0, 0.0};
            for (long long c = first; c < a.n; c += stride) {
                a.x[c] += alpha * a.p[c];
                const double r = a.r[c] - alpha * a.ap[c];
                const double z = r / a.diag[c];
                a.r[c] = r;
                a.z[c] = z;
                u[0] += r * z;
                u[1] += r * r;
            }
            gsync::block_sums<kPcgBlock, 2>(a.partial, set, u);
            if (!gsync::grid_barrier(a.bar_count, a.bar_abort, epoch)) goto aborted;
            double gu[2];
            gsync::grid_sums<2>(a.partial, set, gu);
            set ^= 1;
            const double beta = gu[0] / rz;
            rz = gu[0];
            rr = gu[1];
            ++it;
            for (long long c = first; c < a.n; c += stride) __stcg(&a.p[c], a.z[c] + beta * a.p[c]);
            if (!gsync::grid_barrier(a.bar_count, a.bar_abort, epoch)) goto aborted;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            *a.iters = it;
            if (sqrt(rr) > a.tol * bnorm) atomicOr(a.status, CFG_ERR_PCG);
        }
        return;
    }
aborted:
    if (threadIdx.x == 0) atomicOr(a.status, CFG_ERR_PCG);
}

// ------------------------------------------------------------------ elementwise
struct StepArgs {
    long long n;
    const double* vol;
    double chicm, rdt;
    const double* vm_old;
    const double* im;
    const unsigned char* box;   // [n] box membership bits, or null
    int n_boxes;
    double box_start[8], box_end[8], box_intensity[8];
    double t0;
    double* b;
};

// b = chi Cm V/dt Vm_n - chi Cm V Im + V src(t0)
__global__ void k_rhs(StepArgs a)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n) return;
    const double V = a.vol[c];
    double src = 0.0;
    if (a.box) {
        const unsigned m = a.box[c];
        for (int q = 0; q < a.n_boxes; ++q)
            if (a.t0 >= a.box_start[q] && a.t0 <= a.box_end[q] && (m & (1u << q)))
                src += a.box_intensity[q];
    }
    a.b[c] = a.chicm * V * a.rdt * a.vm_old[c] - a.chicm * V * a.im[c] + V * src;
}

// Adjoint of b: Vbar_n = chi Cm V/dt mu, Imbar = -chi Cm V mu.
__global__ void k_rhs_adjoint(long long n, const double* vol, double chicm, double rdt,
                              const double* mu, double* vbar, double* imbar)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double w = chicm * vol[c] * mu[c];
    vbar[c] = w * rdt;
    imbar[c] = -w;
}

// sigmabar_k -= sum over faces of G_k (mu_P - mu_N)(Vm_P - Vm_N): per row,
// the faces whose other cell has a larger index (each face once); each block
// adds its sum to its own slot, so the total over steps is deterministic.
__global__ void __launch_bounds__(kBlock) k_sigma_grad(long long n, int width, const int* col,
                                                       const unsigned char* cnt, const double* gl,
                                                       const double* gt, const double* mu,
                                                       const double* vm, double* partial)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double s[2] = {0.0, 0.0};
    if (c < n) {
        for (int e = 0; e < cnt[c]; ++e) {
            const long long i = (long long)e * n + c;
            const long long nb = col[i];
            if (nb <= c) continue;
            const double w = (mu[c] - mu[nb]) * (vm[c] - vm[nb]);
            s[0] -= gl[i] * w;
            s[1] -= gt[i] * w;
        }
    }
    __shared__ double sh[2][kBlock / 32];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    for (int k = 0; k < 2; ++k) {
        double v = s[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][wp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        double v = 0.0;
        for (int j = 0; j < kBlock / 32; ++j) v += sh[threadIdx.x][j];
        partial[(long long)threadIdx.x * gridDim.x + blockIdx.x] += v;   // summed over steps
    }
}

// The probes of one sample: J += sum (Vm[p] - T)^2, and optionally
// Vbar[p] += 2 (Vm[p] - T); records the probe values.
__global__ void k_probes(int np, const int* probes, const double* vm, const double* target,
                         double* trace, double* loss, double* vbar)
{
    if (blockIdx.x != 0) return;
    double s = 0.0;
    for (int q = threadIdx.x; q < np; q += blockDim.x) {
        const double v = vm[probes[q]];
        if (trace) trace[q] = v;
        if (target) {
            const double d = v - target[q];
            s += d * d;
            if (vbar) vbar[probes[q]] += 2.0 * d;
        }
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ double sh[32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0 && loss) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) t += sh[w];
        *loss += t;
    }
}

// constants per cell: initConsts with the cell's conductance scales
__global__ void k_consts(long long n, int tissue, const double* scales, double* consts,
                         double* y)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double C[M::NC] = {};
    double y0[NS] = {};
    double sc[6];
    for (int q = 0; q < 6; ++q) sc[q] = scales[(long long)q * n + c];
    M::init(C, y0, tissue, sc);
    for (int i = 0; i < M::NC; ++i) consts[(long long)i * n + c] = C[i];
    if (y)
        for (int i = 0; i < NS; ++i) y[(long long)i * n + c] = y0[i];
}

}  // namespace adj
}  // namespace cfg

// ====================================================================== host

using namespace cfg;
using namespace cfg::adj;

struct cfg_adjoint {
    long long n = 0;
    int width = 0;
    int tissue = 1;
    int substeps = 1;
    long long n_steps = 0;
    int ck_every = 1;
    int sample_every = 1;
    long long n_samples = 0;
    int n_probes = 0;
    double dt = 0, dtm = 0, chicm = 0, vm0 = -0.084;
    double pcg_tol = 1e-13;
    int pcg_max_iter = 10000;
    int n_boxes = 0;
    double box_start[8], box_end[8], box_intensity[8];
    double sigma[2] = {0, 0};
    int pcg_blocks = 0;
    bool fp32 = false;          // FP32 right-hand side and its derivative (mixed form)
    cudaStream_t stream = nullptr;
    // device
    int* d_col = nullptr;
    unsigned char* d_cnt = nullptr;
    double *d_gl = nullptr, *d_gt = nullptr, *d_coef = nullptr, *d_diag = nullptr;
    double* d_vol = nullptr;
    unsigned char* d_box = nullptr;
    int* d_probes = nullptr;
    double *d_target = nullptr, *d_trace = nullptr;
    double *d_scales = nullptr, *d_consts = nullptr;
    double *d_y = nullptr, *d_vm = nullptr, *d_vm_old = nullptr, *d_im = nullptr, *d_b = nullptr;
    double *d_r = nullptr, *d_z = nullptr, *d_p = nullptr, *d_ap = nullptr, *d_partial = nullptr;
    unsigned* d_bar = nullptr;
    int *d_abort = nullptr, *d_iters = nullptr, *d_status = nullptr;
    double* d_loss = nullptr;
    // checkpoints and the window
    double *d_ck_y = nullptr, *d_ck_vm = nullptr;     // [n_ck][NS][n], [n_ck][n]
    double *d_win_y = nullptr, *d_win_vm = nullptr;   // [k+1][NS][n], [k+1][n]
    // adjoint state
    double *d_ybar = nullptr, *d_vbar = nullptr, *d_mu = nullptr, *d_imbar = nullptr;
    double* d_pbar = nullptr;
    double* d_sig_partial = nullptr;
    std::vector<double> h_sig_partial;
    bool forward_done = false;
    double scale_value_na = 1, scale_value_k1 = 1;
};

namespace {

void adj_free(cfg_adjoint* a)
{
    if (!a) return;
    for (void* p : {(void*)a->d_col, (void*)a->d_cnt, (void*)a->d_gl, (void*)a->d_gt,
                    (void*)a->d_coef, (void*)a->d_diag, (void*)a->d_vol, (void*)a->d_box,
                    (void*)a->d_probes, (void*)a->d_target, (void*)a->d_trace,
                    (void*)a->d_scales, (void*)a->d_consts, (void*)a->d_y, (void*)a->d_vm,
                    (void*)a->d_vm_old, (void*)a->d_im, (void*)a->d_b, (void*)a->d_r,
                    (void*)a->d_z, (void*)a->d_p, (void*)a->d_ap, (void*)a->d_partial,
                    (void*)a->d_bar, (void*)a->d_abort, (void*)a->d_iters, (void*)a->d_status,
                    (void*)a->d_loss, (void*)a->d_ck_y, (void*)a->d_ck_vm, (void*)a->d_win_y,
                    (void*)a->d_win_vm, (void*)a->d_ybar, (void*)a->d_vbar, (void*)a->d_mu,
                    (void*)a->d_imbar, (void*)a->d_pbar, (void*)a->d_sig_partial})
        if (p) cudaFree(p);
    if (a->stream) cudaStreamDestroy(a->stream);
    delete a;
}

unsigned grid_of(long long n, int block) { return unsigned((n + block - 1) / block); }

int solve(cfg_adjoint* a, const double* b, double* x)
{
    PcgArgs p{};
    p.n = a->n;
    p.width = a->width;
    p.col = a->d_col;
    p.cnt = a->d_cnt;
    p.coef = a->d_coef;
    p.diag = a->d_diag;
    p.b = b;
    p.x = x;
    p.r = a->d_r; p.z = a->d_z; p.p = a->d_p; p.ap = a->d_ap;
    p.partial = a->d_partial;
    p.bar_count = a->d_bar;
    p.bar_abort = a->d_abort;
    p.tol = a->pcg_tol;
    p.max_iter = a->pcg_max_iter;
    p.iters = a->d_iters;
    p.status = a->d_status;
    CFG_CUDA_TRY(cudaMemsetAsync(a->d_bar, 0, sizeof(unsigned), a->stream));
    CFG_CUDA_TRY(cudaMemsetAsync(a->d_abort, 0, sizeof(int), a->stream));
    void* args[] = {&p};
    CFG_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(k_pcg), dim3(a->pcg_blocks),
                                             dim3(kPcgBlock), args, 0, a->stream));
    return CFG_OK;
}

IonicArgs ionic_args(cfg_adjoint* a, long long step)
{
    IonicArgs g{};
    g.n = a->n;
    g.substeps = a->substeps;
    g.tissue = a->tissue;
    g.dtm = a->dtm;
    g.t0 = double(step) * a->dtm;
    g.consts = a->d_consts;
    g.y = a->d_y;
    g.vm = a->d_vm;
    g.im = a->d_im;
    return g;
}

StepArgs step_args(cfg_adjoint* a, long long step)
{
    StepArgs s{};
    s.n = a->n;
    s.vol = a->d_vol;
    s.chicm = a->chicm;
    s.rdt = 1.0 / a->dt;
    s.vm_old = a->d_vm_old;
    s.im = a->d_im;
    s.box = a->d_box;
    s.n_boxes = a->n_boxes;
    for (int q = 0; q < a->n_boxes; ++q) {
        s.box_start[q] = a->box_start[q];
        s.box_end[q] = a->box_end[q];
        s.box_intensity[q] = a->box_intensity[q];
    }
    s.t0 = double(step) * a->dt;
    s.b = a->d_b;
    return s;
}

// One forward step n -> n+1 on the current state (d_y, d_vm).
int forward_step(cfg_adjoint* a, long long step)
{
    cudaStream_t s = a->stream;
    const size_t bytes = sizeof(double) * size_t(a->n);
    CFG_CUDA_TRY(cudaMemcpyAsync(a->d_vm_old, a->d_vm, bytes, cudaMemcpyDeviceToDevice, s));
    if (a->fp32)
        k_ionic_forward<float><<<grid_of(a->n, kBlock), kBlock, 0, s>>>(ionic_args(a, step));
    else
        k_ionic_forward<double><<<grid_of(a->n, kBlock), kBlock, 0, s>>>(ionic_args(a, step));
    k_rhs<<<grid_of(a->n, kBlock), kBlock, 0, s>>>(step_args(a, step));
    CFG_CUDA_TRY(cudaGetLastError());
    return solve(a, a->d_b, a->d_vm);     // the previous Vm is the initial guess
}

int check(cfg_adjoint* a)
{
    int st = 0;
    CFG_CUDA_TRY(cudaMemcpyAsync(&st, a->d_status, sizeof(int), cudaMemcpyDeviceToHost, a->stream));
    CFG_CUDA_TRY(cudaStreamSynchronize(a->stream));
    if (st) return fail(CFG_ERR_PCG, "adjoint: PCG did not reach the tolerance %.3g", a->pcg_tol);
    return CFG_OK;
}

// Conductance scales exp(theta) for GNa and GK1 (others 1), per-cell
// constants and initial states; face coefficients and the diagonal for
// (sigma_l, sigma_t).
int set_parameters(cfg_adjoint* a, const double* log_gna, const double* log_gk1, double sigma_l,
                   double sigma_t)
{
    const long long n = a->n;
    std::vector<double> sc(size_t(6 * n), 1.0);
    for (long long c = 0; c < n; ++c) {
        sc[size_t(tnnp::SCALE_GNa * n + c)] = log_gna ? std::exp(log_gna[c]) : 1.0;
        sc[size_t(tnnp::SCALE_GK1 * n + c)] = log_gk1 ? std::exp(log_gk1[c]) : 1.0;
    }
    cudaStream_t s = a->stream;
    CFG_CUDA_TRY(cudaMemcpyAsync(a->d_scales, sc.data(), sc.size() * sizeof(double),
                                 cudaMemcpyHostToDevice, s));
    k_consts<<<grid_of(n, kBlock), kBlock, 0, s>>>(n, a->tissue, a->d_scales, a->d_consts, a->d_y);
    CFG_CUDA_TRY(cudaGetLastError());
    // A = chi Cm V/dt + L(sigma): coef = sigma_l G_l + sigma_t G_t per ELL slot
    const size_t slots = size_t(a->width) * size_t(n);
    std::vector<double> gl(slots), gt(slots), vol(static_cast<size_t>(n));
    std::vector<unsigned char> cnt(static_cast<size_t>(n));
    CFG_CUDA_TRY(cudaMemcpy(gl.data(), a->d_gl, slots * sizeof(double), cudaMemcpyDeviceToHost));
    CFG_CUDA_TRY(cudaMemcpy(gt.data(), a->d_gt, slots * sizeof(double), cudaMemcpyDeviceToHost));
    CFG_CUDA_TRY(cudaMemcpy(vol.data(), a->d_vol, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost));
    CFG_CUDA_TRY(cudaMemcpy(cnt.data(), a->d_cnt, size_t(n), cudaMemcpyDeviceToHost));
    std::vector<double> coef(slots, 0.0), diag(static_cast<size_t>(n));
    for (long long c = 0; c < n; ++c) {
        double d = a->chicm * vol[size_t(c)] / a->dt;
        for (int e = 0; e < cnt[size_t(c)]; ++e) {
            const size_t i = size_t(e) * size_t(n) + size_t(c);
            coef[i] = sigma_l * gl[i] + sigma_t * gt[i];
            d += coef[i];
        }
        diag[size_t(c)] = d;
    }
    CFG_CUDA_TRY(cudaMemcpy(a->d_coef, coef.data(), slots * sizeof(double), cudaMemcpyHostToDevice));
    CFG_CUDA_TRY(cudaMemcpy(a->d_diag, diag.data(), size_t(n) * sizeof(double),
                            cudaMemcpyHostToDevice));
    a->sigma[0] = sigma_l;
    a->sigma[1] = sigma_t;
    return CFG_OK;
}

}  // namespace

extern "C" {

int cfg_adjoint_create(const cfg_adjoint_desc* d, const cfg_mesh_desc* m, cfg_adjoint** out)
{
    clear_error();
    if (!d || !m || !out) return fail(CFG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (!d->ionic_model || std::strcmp(d->ionic_model, "TNNP") != 0)
        return fail(CFG_ERR_UNSUPPORTED, "the adjoint step is built for TNNP only (got %s)",
                    d->ionic_model ? d->ionic_model : "null");
    const int flag = tissue_flag(d->tissue ? d->tissue : "");
    if (!tnnp::tissue_supported(flag))
        return fail(CFG_ERR_INVALID, "Unsupported tissue '%s' for TNNP", d->tissue ? d->tissue : "");
    if (m->face_centres)
        return fail(CFG_ERR_UNSUPPORTED, "the adjoint step needs an orthogonal mesh (no face_centres)");
    if (!m->owner || !m->neighbour || !m->volumes || !m->face_sf || !m->face_delta_coeffs ||
        (d->n_boxes && !m->centres))
        return fail(CFG_ERR_INVALID, "incomplete mesh description");
    if (d->substeps < 1 || d->substeps > kMaxSub)
        return fail(CFG_ERR_INVALID, "substeps must be 1..%d", kMaxSub);
    if (d->n_steps < 1 || d->checkpoint_every < 1 || d->sample_every < 1 || d->n_probes < 0 ||
        (d->n_probes && !d->probes) || !(d->delta_t > 0) || d->n_boxes < 0 || d->n_boxes > 8)
        return fail(CFG_ERR_INVALID, "invalid adjoint settings");
    const long long n = m->n_cells, nf = m->n_faces;
    for (int q = 0; q < d->n_probes; ++q)
        if (d->probes[q] < 0 || d->probes[q] >= n) return fail(CFG_ERR_INVALID, "probe %d outside the mesh", q);
    cfg_adjoint* a = new cfg_adjoint();
    auto bail = [&](int rc) {
        adj_free(a);
        return rc;
    };
    a->n = n;
    a->tissue = flag;
    a->substeps = d->substeps;
    a->n_steps = d->n_steps;
    a->ck_every = d->checkpoint_every;
    a->sample_every = d->sample_every;
    a->n_samples = d->n_steps / d->sample_every;
    a->n_probes = d->n_probes;
    a->dt = d->delta_t;
    a->dtm = d->delta_t * 1000.0;      // TNNP model time in ms
    a->chicm = d->chi * d->cm;
    a->vm0 = d->vm0;
    a->pcg_tol = d->pcg_tol > 0 ? d->pcg_tol : 1e-13;
    a->fp32 = d->precision == CFG_PRECISION_MIXED;
    a->pcg_max_iter = d->pcg_max_iter > 0 ? d->pcg_max_iter : 10000;
    a->n_boxes = d->n_boxes;
    for (int q = 0; q < d->n_boxes; ++q) {
        a->box_start[q] = d->box_start[q];
        a->box_end[q] = d->box_start[q] + d->box_duration[q];
        a->box_intensity[q] = d->box_intensity[q];
    }
    if (cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(CFG_ERR_CUDA, "stream creation failed"));
    // ELL rows (columns ascending) with the conductivity parts of each face:
    // Sf.sigma.Sf/|Sf| = sigma_t |Sf| + (sigma_l - sigma_t) (f.Sf)^2/|Sf|
    double f[3] = {d->fibre[0], d->fibre[1], d->fibre[2]};
    const double fn = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fn > 0)) return bail(fail(CFG_ERR_INVALID, "zero fibre direction"));
    for (double& v : f) v /= fn;
    struct E {
        int col;
        double gl, gt;
    };
    std::vector<std::vector<E>> rows(static_cast<size_t>(n));
    for (long long k = 0; k < nf; ++k) {
        const int l = m->owner[k], u = m->neighbour[k];
        if (l < 0 || u < 0 || l >= n || u >= n || l == u)
            return bail(fail(CFG_ERR_INVALID, "face %lld has invalid owner/neighbour", k));
        const double* S = m->face_sf + 3 * k;
        const double mag = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
        const double fs = f[0] * S[0] + f[1] * S[1] + f[2] * S[2];
        const double dc = m->face_delta_coeffs[k];
        const double gl = dc * fs * fs / mag;
        const double gt = dc * (mag * mag - fs * fs) / mag;
        rows[size_t(l)].push_back({u, gl, gt});
        rows[size_t(u)].push_back({l, gl, gt});
    }
    int width = 0;
    for (auto& r : rows) {
        std::sort(r.begin(), r.end(), [](const E& x, const E& y) { return x.col < y.col; });
        width = std::max(width, int(r.size()));
    }
    if (width > 255) return bail(fail(CFG_ERR_INVALID, "cell with more than 255 faces"));
    a->width = width;
    const size_t slots = size_t(width) * size_t(n);
    std::vector<int> col(slots, 0);
    std::vector<double> gl(slots, 0.0), gt(slots, 0.0);
    std::vector<unsigned char> cnt(static_cast<size_t>(n));
    for (long long c = 0; c < n; ++c) {
        cnt[size_t(c)] = (unsigned char)rows[size_t(c)].size();
        for (size_t q = 0; q < rows[size_t(c)].size(); ++q) {
            const size_t i = q * size_t(n) + size_t(c);
            col[i] = rows[size_t(c)][q].col;
            gl[i] = rows[size_t(c)][q].gl;
            gt[i] = rows[size_t(c)][q].gt;
        }
    }
    std::vector<unsigned char> box(size_t(n), 0);
    for (long long c = 0; c < n; ++c)
        for (int q = 0; q < d->n_boxes; ++q) {
            const double* p = m->centres + 3 * c;
            bool in = true;
            for (int k = 0; k < 3; ++k) in = in && p[k] >= d->box_min[q][k] && p[k] <= d->box_max[q][k];
            if (in) box[size_t(c)] |= (unsigned char)(1u << q);
        }
    const long long n_ck = (d->n_steps + d->checkpoint_every - 1) / d->checkpoint_every;
    const size_t nn = size_t(n);
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, kPcgBlock, 0);
    const long long want = (n + kPcgBlock - 1) / kPcgBlock;
    a->pcg_blocks = int(std::min<long long>(want, (long long)sms * std::max(per_sm, 1)));
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto** ptr, size_t count) {
        if (!e) e = dmalloc(ptr, count);
    };
    alloc(&a->d_col, slots);
    alloc(&a->d_cnt, nn);
    alloc(&a->d_gl, slots);
    alloc(&a->d_gt, slots);
    alloc(&a->d_coef, slots);
    alloc(&a->d_diag, nn);
    alloc(&a->d_vol, nn);
    alloc(&a->d_box, nn);
    alloc(&a->d_probes, size_t(std::max(d->n_probes, 1)));
    alloc(&a->d_target, size_t(std::max<long long>(a->n_samples * d->n_probes, 1)));
    alloc(&a->d_trace, size_t(std::max<long long>(a->n_samples * d->n_probes, 1)));
    alloc(&a->d_scales, 6 * nn);
    alloc(&a->d_consts, size_t(M::NC) * nn);
    alloc(&a->d_y, size_t(NS) * nn);
    for (double** v : {&a->d_vm, &a->d_vm_old, &a->d_im, &a->d_b, &a->d_r, &a->d_z, &a->d_p,
                       &a->d_ap, &a->d_vbar, &a->d_mu, &a->d_imbar})
        alloc(v, nn);
    alloc(&a->d_partial, size_t(4 * std::max(a->pcg_blocks, 1)));
    alloc(&a->d_bar, 1);
    alloc(&a->d_abort, 1);
    alloc(&a->d_iters, 1);
    alloc(&a->d_status, 1);
    alloc(&a->d_loss, 1);
    alloc(&a->d_ck_y, size_t(n_ck) * NS * nn);
    alloc(&a->d_ck_vm, size_t(n_ck) * nn);
    alloc(&a->d_win_y, size_t(d->checkpoint_every + 1) * NS * nn);
    alloc(&a->d_win_vm, size_t(d->checkpoint_every + 1) * nn);
    alloc(&a->d_ybar, size_t(NS) * nn);
    alloc(&a->d_pbar, 6 * nn);
    alloc(&a->d_sig_partial, 2 * size_t(grid_of(n, kBlock)));
    if (e) return bail(fail(CFG_ERR_CUDA, "adjoint allocation failed: %s", cudaGetErrorString(e)));
    e = cudaMemcpy(a->d_col, col.data(), slots * sizeof(int), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(a->d_cnt, cnt.data(), nn, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(a->d_gl, gl.data(), slots * sizeof(double), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(a->d_gt, gt.data(), slots * sizeof(double), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(a->d_vol, m->volumes, nn * sizeof(double), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(a->d_box, box.data(), nn, cudaMemcpyHostToDevice);
    if (!e && d->n_probes)
        e = cudaMemcpy(a->d_probes, d->probes, sizeof(int) * size_t(d->n_probes), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemset(a->d_target, 0, sizeof(double) * size_t(std::max<long long>(a->n_samples * d->n_probes, 1)));
    if (e) return bail(fail(CFG_ERR_CUDA, "adjoint set-up failed: %s", cudaGetErrorString(e)));
    *out = a;
    return CFG_OK;
}

int cfg_adjoint_set_target(cfg_adjoint* a, const double* target)
{
    if (!a || !target) return fail(CFG_ERR_INVALID, "null argument");
    CFG_CUDA_TRY(cudaMemcpy(a->d_target, target,
                            sizeof(double) * size_t(a->n_samples * a->n_probes),
                            cudaMemcpyHostToDevice));
    return CFG_OK;
}

int cfg_adjoint_forward(cfg_adjoint* a, const double* log_gna, const double* log_gk1,
                        double sigma_l, double sigma_t, double* loss, double* probe_trace)
{
    if (!a) return fail(CFG_ERR_INVALID, "null argument");
    clear_error();
    if (int rc = set_parameters(a, log_gna, log_gk1, sigma_l, sigma_t)) return rc;
    cudaStream_t s = a->stream;
    const size_t nn = size_t(a->n), bytes = nn * sizeof(double);
    std::vector<double> vm0(nn, a->vm0);
    CFG_CUDA_TRY(cudaMemcpyAsync(a->d_vm, vm0.data(), bytes, cudaMemcpyHostToDevice, s));
    CFG_CUDA_TRY(cudaMemsetAsync(a->d_loss, 0, sizeof(double), s));
    CFG_CUDA_TRY(cudaMemsetAsync(a->d_status, 0, sizeof(int), s));
    for (long long step = 0; step < a->n_steps; ++step) {
        if (step % a->ck_every == 0) {
            const long long k = step / a->ck_every;
            CFG_CUDA_TRY(cudaMemcpyAsync(a->d_ck_y + size_t(k) * NS * nn, a->d_y, NS * bytes,
                                         cudaMemcpyDeviceToDevice, s));
            CFG_CUDA_TRY(cudaMemcpyAsync(a->d_ck_vm + size_t(k) * nn, a->d_vm, bytes,
                                         cudaMemcpyDeviceToDevice, s));
        }
        if (int rc = forward_step(a, step)) return rc;
        if ((step + 1) % a->sample_every == 0 && a->n_probes) {
            const long long q = (step + 1) / a->sample_every - 1;
            k_probes<<<1, 128, 0, s>>>(a->n_probes, a->d_probes, a->d_vm,
                                       a->d_target + size_t(q) * a->n_probes,
                                       a->d_trace + size_t(q) * a->n_probes, a->d_loss, nullptr);
        }
        if ((step & 255) == 255)
            if (int rc = check(a)) return rc;
    }
    CFG_CUDA_TRY(cudaGetLastError());
    if (int rc = check(a)) return rc;
    if (loss) CFG_CUDA_TRY(cudaMemcpy(loss, a->d_loss, sizeof(double), cudaMemcpyDeviceToHost));
    if (probe_trace && a->n_probes)
        CFG_CUDA_TRY(cudaMemcpy(probe_trace, a->d_trace,
                                sizeof(double) * size_t(a->n_samples * a->n_probes),
                                cudaMemcpyDeviceToHost));
    a->forward_done = true;
    return CFG_OK;
}

int cfg_adjoint_backward(cfg_adjoint* a, double* grad_log_gna, double* grad_log_gk1,
                         double* grad_sigma)
{
    if (!a) return fail(CFG_ERR_INVALID, "null argument");
    if (!a->forward_done) return fail(CFG_ERR_INVALID, "cfg_adjoint_backward before a forward run");
    clear_error();
    cudaStream_t s = a->stream;
    const long long n = a->n;
    const size_t nn = size_t(n), bytes = nn * sizeof(double);
    const unsigned g = grid_of(n, kBlock);
    CFG_CUDA_TRY(cudaMemsetAsync(a->d_ybar, 0, NS * bytes, s));
    CFG_CUDA_TRY(cudaMemsetAsync(a->d_vbar, 0, bytes, s));
    CFG_CUDA_TRY(cudaMemsetAsync(a->d_pbar, 0, 6 * bytes, s));
    CFG_CUDA_TRY(cudaMemsetAsync(a->d_sig_partial, 0, 2 * size_t(g) * sizeof(double), s));
    CFG_CUDA_TRY(cudaMemsetAsync(a->d_status, 0, sizeof(int), s));
    const long long n_ck = (a->n_steps + a->ck_every - 1) / a->ck_every;
    for (long long w = n_ck - 1; w >= 0; --w) {
        const long long start = w * a->ck_every;
        const long long end = std::min(start + a->ck_every, a->n_steps);
        CFG_CUDA_TRY(cudaMemcpyAsync(a->d_y, a->d_ck_y + size_t(w) * NS * nn, NS * bytes,
                                     cudaMemcpyDeviceToDevice, s));
        CFG_CUDA_TRY(cudaMemcpyAsync(a->d_vm, a->d_ck_vm + size_t(w) * nn, bytes,
                                     cudaMemcpyDeviceToDevice, s));
        for (long long step = start; step < end; ++step) {
            const size_t j = size_t(step - start);
            CFG_CUDA_TRY(cudaMemcpyAsync(a->d_win_y + j * NS * nn, a->d_y, NS * bytes,
                                         cudaMemcpyDeviceToDevice, s));
            CFG_CUDA_TRY(cudaMemcpyAsync(a->d_win_vm + j * nn, a->d_vm, bytes,
                                         cudaMemcpyDeviceToDevice, s));
            if (int rc = forward_step(a, step)) return rc;
        }
        CFG_CUDA_TRY(cudaMemcpyAsync(a->d_win_vm + size_t(end - start) * nn, a->d_vm, bytes,
                                     cudaMemcpyDeviceToDevice, s));
        for (long long step = end - 1; step >= start; --step) {
            const size_t j = size_t(step - start);
            const double* vm_next = a->d_win_vm + (j + 1) * nn;
            if ((step + 1) % a->sample_every == 0 && a->n_probes) {
                const long long q = (step + 1) / a->sample_every - 1;
                k_probes<<<1, 128, 0, s>>>(a->n_probes, a->d_probes, vm_next,
                                           a->d_target + size_t(q) * a->n_probes, nullptr, nullptr,
                                           a->d_vbar);
            }
            CFG_CUDA_TRY(cudaMemsetAsync(a->d_mu, 0, bytes, s));
            if (int rc = solve(a, a->d_vbar, a->d_mu)) return rc;
            k_sigma_grad<<<g, kBlock, 0, s>>>(n, a->width, a->d_col, a->d_cnt, a->d_gl, a->d_gt,
                                              a->d_mu, vm_next, a->d_sig_partial);
            k_rhs_adjoint<<<g, kBlock, 0, s>>>(n, a->d_vol, a->chicm, 1.0 / a->dt, a->d_mu,
                                               a->d_vbar, a->d_imbar);
            IonicArgs ia = ionic_args(a, step);
            ia.y_start = a->d_win_y + j * NS * nn;
            ia.vm = a->d_win_vm + j * nn;
            ia.ybar = a->d_ybar;
            ia.imbar = a->d_imbar;
            ia.vbar = a->d_vbar;
            ia.pbar = a->d_pbar;
            if (a->fp32) k_ionic_reverse<float><<<g, kBlock, 0, s>>>(ia);
            else k_ionic_reverse<double><<<g, kBlock, 0, s>>>(ia);
            CFG_CUDA_TRY(cudaGetLastError());
        }
        if (int rc = check(a)) return rc;
    }
    // outputs: thetabar = pbar * p (p = the scaled conductance of the cell)
    std::vector<double> pbar(6 * nn), cst(size_t(M::NC) * nn), part(2 * size_t(g));
    CFG_CUDA_TRY(cudaMemcpy(pbar.data(), a->d_pbar, 6 * bytes, cudaMemcpyDeviceToHost));
    CFG_CUDA_TRY(cudaMemcpy(cst.data(), a->d_consts, size_t(M::NC) * bytes, cudaMemcpyDeviceToHost));
    CFG_CUDA_TRY(cudaMemcpy(part.data(), a->d_sig_partial, part.size() * sizeof(double),
                            cudaMemcpyDeviceToHost));
    for (long long c = 0; c < n; ++c) {
        if (grad_log_gna)
            grad_log_gna[c] = pbar[size_t(tnnp::SCALE_GNa * n + c)] * cst[size_t(tnnp::C_g_Na * n + c)];
        if (grad_log_gk1)
            grad_log_gk1[c] = pbar[size_t(tnnp::SCALE_GK1 * n + c)] * cst[size_t(tnnp::C_g_K1 * n + c)];
    }
    if (grad_sigma) {
        double sl = 0.0, st = 0.0;
        for (unsigned b = 0; b < g; ++b) {
            sl += part[b];
            st += part[size_t(g) + b];
        }
        grad_sigma[0] = sl;
        grad_sigma[1] = st;
    }
    return CFG_OK;
}

int cfg_adjoint_destroy(cfg_adjoint* a)
{
    if (a) {
        cudaStreamSynchronize(a->stream);
        adj_free(a);
    }
    return CFG_OK;
}

}  // extern "C"
