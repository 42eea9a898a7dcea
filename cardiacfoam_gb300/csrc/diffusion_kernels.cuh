// Diffusion half of the monodomain step on the GPU:
//   chi*Cm*ddt(Vm) == laplacian(sigma, Vm) - chi*Cm*Iion + src
// (MonodomainSolver::solveDiffusionImplicit/Explicit, monodomainSolver.C:103-150).
//
// Matrix: OpenFOAM's symmetric lduMatrix re-laid as ELL rows (column-major,
// neighbours sorted ascending, per-row counts) so a row sum visits the
// off-diagonals in the same order as lduMatrix::Amul's face loop; the
// diagonal is rebuilt each solve from the ddt coefficient and the static
// Laplacian row sum.
//
// PCG restates lduMatrix PCG (normFactor, L1 residual, convergence test)
// with the diagonal preconditioner.  Scalars live in device memory; every
// reduction writes per-block partials and the last block to finish sums them
// in a fixed order, so results do not depend on scheduling.  Kernels of a
// finished solve return at once, which lets a fixed launch sequence (or a
// graph with conditional nodes) run a data-dependent number of iterations.
#pragma once

#include <cuda_runtime.h>

#include "../../include/cardiac_gpu.h"
#include "float_pair.cuh"

namespace cfg {

constexpr int kDiffBlock = 256;
constexpr int kMaxSolves = 16;

struct PcgState {
    // --- control (device-owned during a step)
    int n_old;            // stored old-time levels of Vm (GeometricField::nOldTimes)
    int corr;             // PIMPLE corrector of the current step (1-based)
    int solve_active;     // current PCG solve still iterating
    int outer_active;     // PIMPLE loop continues
    int converged_outer;  // residualControl met; the running corrector is the final one
    int iter;             // iterations of the current solve
    int n_solves;
    int variant;          // ddt coefficient set of the current corrector
    int status;           // CFG_ERR_* bits
    long long step_iters; // PCG iterations of the current step (loop guard)
    // --- settings
    double tol, rel_tol, outer_tol;
    int max_iter, n_outer;
    // --- scalars
    double sum_x, avg, sum_absr, normf, init_res, res, wArA, wArAold, wApA, alpha, beta;
    double t, t0;         // runTime value and step start
    unsigned int arrive[4];
    // grid barrier of the persistent diffusion kernel (reset every step)
    unsigned int bar_count;
    int bar_abort;
    // --- statistics of the last step
    int iters[kMaxSolves];
    double init_r[kMaxSolves], final_r[kMaxSolves];
};

struct DiffusionArgs {
    long long n;
    int width;                 // ELL width
    const int* ell_col;        // [width][n]
    const double* ell_coef;    // [width][n] face coefficient (>0)
    const unsigned char* ell_cnt;  // [n]
    const double* lapdiag;     // [n] sum of -coef in row order
    const double* vol;         // [n]
    // explicit correction of the Laplacian on a general mesh (null: none):
    // per ELL slot the gradient weight of (x_nb - x_c), the correction
    // vector signed for the row (+ for the face's owner) and the row cell's
    // interpolation weight; per cell the wall factor and the gradient.
    // Arrays of double, or of float when nc_fp32 (the mixed form).
    const void* nc_gw;         // [3][width][n]
    const void* nc_k;          // [3][width][n]
    const void* nc_om;         // [width][n]
    const void* nc_bk;         // [3][n]
    void* grad;                // [3][n]
    int nc_fp32;
    // corrector-independent part of the source (ddt, -chi*Cm*Iion, stimulus),
    // kept by the persistent kernel from the first corrector of a step
    double* bsrc;              // [n]
    // stencil form (structured block, uniform coefficient per direction)
    int sx, sy, sz;            // nx, ny, nz (0 = use ELL)
    double cx, cy, cz;
    // fields
    double* vm;                // x
    double* vm_old;
    double* vm_oldold;
    const double* iion;
    double* act;
    unsigned char* act_flag;
    // boxes
    const unsigned char* box_mask;  // [n] bit b: centre inside box b
    int n_boxes;
    double box_start[8], box_end[8], box_intensity[8];
    // matrix diagonal, its reciprocal (diagonal preconditioner) and row sums
    // for the two ddt coefficient sets: [0] while fewer than two old-time
    // levels exist (backward falls back to deltaT0 = GREAT), [1] afterwards
    double* diag2;             // [2][n]
    double* rdiag2;            // [2][n]
    double* sumA2;             // [2][n]
    double cft[2], cft0[2], cft00[2];
    double rdt;
    // PCG work
    double *b, *r, *z, *ax, *pA, *pB, *ap;
    double* partial;           // [4][nblocks]
    int nblocks;
    PcgState* st;
    // graph control: conditional handles of the PIMPLE and PCG while-nodes
    // (set only when the kernels run inside the step graph)
    int use_graph;
    cudaGraphConditionalHandle h_outer, h_inner;
    long long iter_cap;        // PCG iterations per step before the step is aborted
    long long spin_limit;      // spins a block waits at a grid barrier before it aborts
    // per-cell source density of the step when a conduction network is
    // coupled (box stimulus plus the PVJ deposits, set before the step);
    // null: the box stimulus alone
    const double* src_total;
    // step constants
    double dt, chicm;
    int ddt_backward;
    // float-pair form of the persistent solve (pair != 0): the matrix and
    // the source scaled by 2^pair_shift (a power of two, so the scaled system
    // has exactly the same solution and residual ratios) and held as (hi,
    // lo) float pairs; b, r, z, A.x, p and A.p then hold pairs in their
    // 8-byte slots, px the iterate
    int pair, pair_shift;
    float2* pdiag2;            // [2][n]
    float2* prdiag2;           // [2][n] reciprocal of the scaled diagonal
    float2* psumA2;            // [2][n]
    float2* pcoef;             // [width][n]
    float2 pcx, pcy, pcz;      // stencil form
    float2* px;                // [n]
};

// ------------------------------------------------------------------ helpers

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-level sums of up to 3 values into partial[k][blockIdx.x] (fixed order).
template <int K>
__device__ __forceinline__ void block_partials(const DiffusionArgs& a, double (&v)[K])
{
    __shared__ double sh[K][kDiffBlock / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = warp_sum(v[k]);
        if (lane == 0) sh[k][w] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = 0.0;
            for (int j = 0; j < kDiffBlock / 32; ++j) s += sh[k][j];
            a.partial[k * a.nblocks + blockIdx.x] = s;
        }
    }
}

// True in exactly one block: the last to arrive.  Its threads then sum the
// partials with sum_partials().
__device__ __forceinline__ bool last_block(const DiffusionArgs& a, int slot)
{
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned prev = atomicAdd(&a.st->arrive[slot], 1u);
        is_last = (prev == unsigned(a.nblocks) - 1);
        if (is_last) a.st->arrive[slot] = 0;
    }
    __syncthreads();
    if (is_last) __threadfence();
    return is_last;
}

// Deterministic sum of partial[k][0..nblocks) by the calling block.
__device__ __forceinline__ double sum_partials(const DiffusionArgs& a, int k)
{
    __shared__ double sh[kDiffBlock];
    double s = 0.0;
    for (int i = threadIdx.x; i < a.nblocks; i += kDiffBlock)
        s += *((volatile double*)&a.partial[k * a.nblocks + i]);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int h = kDiffBlock / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
        __syncthreads();
    }
    double r = sh[0];
    __syncthreads();
    return r;
}

// A.x for row c with A = diag - offdiag: diag*x, then each (-coef)*x_nb
// added in column order (bitwise the same as lduMatrix::Amul).
template <class F>
__device__ __forceinline__ double row_amul(const DiffusionArgs& a, long long c, double d, F f)
{
    double acc = d * f(c);
    if (a.sx) {
        const long long nx = a.sx, nxy = (long long)a.sx * a.sy;
        const long long i = c % nx, j = (c / nx) % a.sy, k = c / nxy;
        if (k > 0) acc += (-a.cz) * f(c - nxy);
        if (j > 0) acc += (-a.cy) * f(c - nx);
        if (i > 0) acc += (-a.cx) * f(c - 1);
        if (i + 1 < nx) acc += (-a.cx) * f(c + 1);
        if (j + 1 < a.sy) acc += (-a.cy) * f(c + nx);
        if (k + 1 < a.sz) acc += (-a.cz) * f(c + nxy);
    } else {
        const int cnt = a.ell_cnt[c];
        for (int q = 0; q < cnt; ++q)
            acc += (-a.ell_coef[(long long)q * a.n + c]) * f(a.ell_col[(long long)q * a.n + c]);
    }
    return acc;
}

// Cell gradient of x at row c on a general mesh: sum over the row's slots
// of gw_e (x_nb - x_c) (leastSquares or Gauss linear weights), in R (the
// differences are taken in FP64).
// Streaming loads of the operator's per-slot arrays: read once per pass and
// larger than L2 on big meshes, so they are loaded evict-first and leave L2
// to the vectors whose entries the neighbours gather.
template <class T>
__device__ __forceinline__ T ld_stream(const T* p)
{
    return __ldcs(p);
}

// W > 0: every row is visited over W slots (the ELL width); padded slots
// hold zero weights and coefficients, so they add exact zeros, and the
// fixed trip count lets all of a row's loads be issued together.
// x_nb - x_c in the gradient's type: from FP64 values, or from float pairs
// (the float-pair solve's iterate) without the FP64 pipe
template <class R>
__device__ __forceinline__ R value_diff(double u, double v) { return R(u - v); }
template <class R>
__device__ __forceinline__ R value_diff(fp::P u, fp::P v)
{
    const fp::P d = fp::sub(u, v);
    return R(d.x) + R(d.y);
}

template <class R, int W = 0, class F>
__device__ __forceinline__ void nc_gradient(const DiffusionArgs& a, long long c, F x, R (&g)[3])
{
    const R* gw = static_cast<const R*>(a.nc_gw);
    const long long n = a.n, wn = (long long)a.width * n;
    const auto xc = x(c);
    g[0] = g[1] = g[2] = R(0);
    const int cnt = W > 0 ? W : a.ell_cnt[c];
#pragma unroll
    for (int e = 0; e < (W > 0 ? W : cnt); ++e) {
        const long long i = (long long)e * n + c;
        const R dv = value_diff<R>(x(ld_stream(&a.ell_col[i])), xc);
        g[0] += ld_stream(&gw[i]) * dv;
        g[1] += ld_stream(&gw[wn + i]) * dv;
        g[2] += ld_stream(&gw[2 * wn + i]) * dv;
    }
}

// fvc::div of the explicit correction fluxes times V at row c: each face's
// flux k.(w (g_P - g_N) + g_N) with the sign of the row (faces in column
// order, the order of the face loop), then the wall term bk.g_c.  g(q, k)
// reads component k of cell q's gradient.
template <class R, int W = 0, class G>
__device__ __forceinline__ double nc_correction(const DiffusionArgs& a, long long c, G g)
{
    const R* kc = static_cast<const R*>(a.nc_k);
    const R* omv = static_cast<const R*>(a.nc_om);
    const R* bk = static_cast<const R*>(a.nc_bk);
    const long long n = a.n, wn = (long long)a.width * n;
    const R g0 = g(c, 0), g1 = g(c, 1), g2 = g(c, 2);
    R s = R(0);
    const int cnt = W > 0 ? W : a.ell_cnt[c];
#pragma unroll
    for (int e = 0; e < (W > 0 ? W : cnt); ++e) {
        const long long i = (long long)e * n + c;
        const long long nb = ld_stream(&a.ell_col[i]);
        const R om = ld_stream(&omv[i]);
        const R n0 = g(nb, 0), n1 = g(nb, 1), n2 = g(nb, 2);
        const R f0 = om * (g0 - n0) + n0;
        const R f1 = om * (g1 - n1) + n1;
        const R f2 = om * (g2 - n2) + n2;
        s += ld_stream(&kc[i]) * f0 + ld_stream(&kc[wn + i]) * f1 + ld_stream(&kc[2 * wn + i]) * f2;
    }
    s += ld_stream(&bk[c]) * g0 + ld_stream(&bk[n + c]) * g1 + ld_stream(&bk[2 * n + c]) * g2;
    return double(s);
}

// The correction at row c from the gradient array (plain loads).
__device__ __forceinline__ double nc_correction_plain(const DiffusionArgs& a, long long c)
{
    const long long n = a.n;
    if (a.nc_fp32) {
        const float* gr = static_cast<const float*>(a.grad);
        return nc_correction<float>(a, c, [gr, n](long long q, int k) { return gr[k * n + q]; });
    }
    const double* gr = static_cast<const double*>(a.grad);
    return nc_correction<double>(a, c, [gr, n](long long q, int k) { return gr[k * n + q]; });
}

// The gradient of x at row c into the gradient array (plain loads/stores).
__device__ __forceinline__ void nc_gradient_plain(const DiffusionArgs& a, long long c,
                                                  const double* x)
{
    const long long n = a.n;
    if (a.nc_fp32) {
        float g[3];
        nc_gradient<float>(a, c, [x](long long q) { return x[q]; }, g);
        float* gr = static_cast<float*>(a.grad);
        gr[c] = g[0]; gr[n + c] = g[1]; gr[2 * n + c] = g[2];
    } else {
        double g[3];
        nc_gradient<double>(a, c, [x](long long q) { return x[q]; }, g);
        double* gr = static_cast<double*>(a.grad);
        gr[c] = g[0]; gr[n + c] = g[1]; gr[2 * n + c] = g[2];
    }
}

// row sum of the matrix (lduMatrix::sumA): diag then each -coef
__device__ __forceinline__ double row_sum(const DiffusionArgs& a, long long c, double d)
{
    return row_amul(a, c, d, [](long long) { return 1.0; });
}

// ddt coefficient set in use: backwardDdtScheme takes deltaT0 = GREAT while
// fewer than two old-time levels exist (Euler has one set)
__device__ __forceinline__ int ddt_variant(const DiffusionArgs& a, int n_old)
{
    return (a.ddt_backward && n_old >= 2) ? 1 : 0;
}

// MyocardiumDomain::updateExternalStimulusCurrent for one cell
__device__ __forceinline__ double box_source(const DiffusionArgs& a, long long c, double t0)
{
    if (a.src_total) return a.src_total[c];
    double s = 0.0;
    if (!a.box_mask) return s;
    const unsigned m = a.box_mask[c];
    for (int b = 0; b < a.n_boxes; ++b) {
        if (t0 < a.box_start[b] || t0 > a.box_end[b]) continue;
        if (m & (1u << b)) s += a.box_intensity[b];
    }
    return s;
}

// PIMPLE control after a solve ends (pimpleLoop::loop / criteriaSatisfied):
// the next corrector runs unless the loop already converged; it is the
// final one when this solve's initial residual met residualControl.
__device__ __forceinline__ void end_solve(PcgState* st)
{
    int k = st->n_solves;
    if (k < kMaxSolves) {
        st->iters[k] = st->iter;
        st->init_r[k] = st->init_res;
        st->final_r[k] = st->res;
    }
    st->n_solves = k + 1;
    st->solve_active = 0;
    if (st->converged_outer || st->corr + 1 > st->n_outer) {
        st->outer_active = 0;
    } else {
        if (st->init_res < st->outer_tol) st->converged_outer = 1;
        st->outer_active = 1;
    }
    st->corr += 1;
}

// Publish the loop conditions to the step graph's while-nodes.
__device__ __forceinline__ void set_inner(const DiffusionArgs& a, int v)
{
    if (a.use_graph) cudaGraphSetConditional(a.h_inner, unsigned(v));
}
__device__ __forceinline__ void set_outer(const DiffusionArgs& a, int v)
{
    if (a.use_graph) cudaGraphSetConditional(a.h_outer, unsigned(v));
}

// MyocardiumDomain::updateActivationTime (myocardiumDomain.C:345-374)
__device__ __forceinline__ void activation(const DiffusionArgs& a, long long c, double vnew,
                                           double vold, double old_time)
{
    if (a.act_flag[c] && vnew > 1e-15) {
        a.act_flag[c] = 0;
        const double w = (0.0 - vold) / (vnew - vold);
        a.act[c] = old_time + w * a.dt;
    }
}

__device__ __forceinline__ bool pcg_converged(const PcgState* st, double r)
{
    return r < st->tol || (st->rel_tol > 1e-20 && r < st->rel_tol * st->init_res);
}

}  // namespace cfg
