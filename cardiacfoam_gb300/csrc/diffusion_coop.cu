// Implicit diffusion of one monodomain step as ONE persistent kernel: every
// PIMPLE corrector and every PCG iteration of the step runs inside a single
// cooperative launch whose blocks meet at grid barriers, instead of two to
// four kernel launches per iteration.
//
// The numerics are those of the per-kernel path (diffusion.cu): the same
// right-hand side, lduMatrix::Amul order, normFactor, L1 residual,
// convergence test and PIMPLE residual control.  Two things change:
//   * each thread owns a fixed set of rows for the whole step, so its own
//     entries of x, r, p, b, A.x and A.p are only ever touched by it; z and
//     x (read at the neighbours) and the reduction partials cross blocks,
//     and those are read through L2 (ld.global.cg), which is coherent;
//   * A.p is updated as A.z + beta A.p, so one halo exchange (of z) serves
//     both the new direction and its product, and an iteration needs two
//     grid barriers; reductions are per thread over its rows, then per
//     block, then summed by every block in the same fixed order.  GB300
//     executes FP64 at 1/64 of the FP32 rate, so the FP64 instruction count
//     per row (15 per PCG iteration here) and the barriers set the speed of
//     the solve, not HBM: its vectors stay in L2.
//
// On a general mesh every corrector first forms the cell gradient of the
// iterate (one more barrier) for the explicit correction of the Laplacian
// in the source.
//
// k_implicit_pair is the same solve with the PCG in float pairs (the mixed
// form's default on meshes without explicit corrections).
//
// Grid barriers are cooperative-launch safe (all blocks co-resident) and
// bounded: a block that waits longer than the context's spin limit (~1 s by
// default) sets an abort flag, every block leaves at its next barrier, and
// the step reports CFG_ERR_PCG.
#include <cuda_runtime.h>

#include "diffusion_kernels.cuh"
#include "grid_sync.cuh"

namespace cfg {

namespace {

constexpr int kCoopBlock = 512;
__device__ __forceinline__ bool grid_barrier(PcgState* st, unsigned& epoch, long long spin_limit)
{
    return gsync::grid_barrier(&st->bar_count, &st->bar_abort, epoch, spin_limit);
}

template <int K>
__device__ __forceinline__ void block_sums(double* partial, int set, double (&v)[K])
{
    gsync::block_sums<kCoopBlock, K>(partial, set, v);
}

using gsync::grid_sums;

// x / d for 0 <= x < 2^31 by multiply-high (round-up method): avoids the
// 64-bit integer division of a cell index in every stencil row.
struct FastDiv {
    unsigned m, s;
};

__device__ __forceinline__ unsigned fdiv(unsigned x, FastDiv f)
{
    return (__umulhi(x, f.m) + x) >> f.s;
}

}  // namespace

struct CoopArgs {
    FastDiv div_nx, div_ny;   // stencil form only
};

// A.q for row c (diag*q_c, then each -coef*q_nb in column order), q read
// through L2.  Stencil neighbours come from (i, j, k) = row decomposition.
template <int W>
__device__ __forceinline__ double amul_cg(const DiffusionArgs& a, const CoopArgs& ca,
                                          unsigned c, double d, const double* q)
{
    double acc = d * __ldcg(&q[c]);
    if (a.sx) {
        const unsigned nx = unsigned(a.sx), nxy = nx * unsigned(a.sy);
        const unsigned line = fdiv(c, ca.div_nx), i = c - line * nx;
        const unsigned k = fdiv(line, ca.div_ny), j = line - k * unsigned(a.sy);
        if (k > 0) acc += (-a.cz) * __ldcg(&q[c - nxy]);
        if (j > 0) acc += (-a.cy) * __ldcg(&q[c - nx]);
        if (i > 0) acc += (-a.cx) * __ldcg(&q[c - 1]);
        if (i + 1 < nx) acc += (-a.cx) * __ldcg(&q[c + 1]);
        if (j + 1 < unsigned(a.sy)) acc += (-a.cy) * __ldcg(&q[c + nx]);
        if (k + 1 < unsigned(a.sz)) acc += (-a.cz) * __ldcg(&q[c + nxy]);
    } else if constexpr (W > 0) {
        // padded slots: coefficient 0 and column 0, an exact zero term
#pragma unroll
        for (int e = 0; e < W; ++e)
            acc += (-ld_stream(&a.ell_coef[(long long)e * a.n + c])) *
                   __ldcg(&q[ld_stream(&a.ell_col[(long long)e * a.n + c])]);
    } else {
        const int cnt = a.ell_cnt[c];
        for (int e = 0; e < cnt; ++e)
            acc += (-a.ell_coef[(long long)e * a.n + c]) *
                   __ldcg(&q[a.ell_col[(long long)e * a.n + c]]);
    }
    return acc;
}

// The whole implicit diffusion of one step (all correctors, all PCG
// iterations) and the activation-time update.  Launched cooperatively with
// every block resident; rows are strided over the grid, two per loop trip so
// that two independent FP64 chains are in flight per thread.
//
// PCG iteration with two grid barriers (lduMatrix PCG in exact arithmetic):
//   halo pass:   w = A.z (z of the neighbours through L2), p = z + beta p,
//                A.p = w + beta A.p (linearity of A), sum p.A.p  | barrier
//   update pass: x += alpha p, r -= alpha A.p, z = D^-1 r (published for
//                the next halo pass), sums |r| and z.r           | barrier
template <class CR, int W>
__global__ void __launch_bounds__(kCoopBlock, W == 4 ? 2 : 1)
    k_implicit_coop(DiffusionArgs a, CoopArgs ca)
{
    PcgState* st = a.st;
    const unsigned n = unsigned(a.n);
    const unsigned stride = gridDim.x * blockDim.x;
    const unsigned first = blockIdx.x * blockDim.x + threadIdx.x;
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    // values every block reads before block 0 may update them
    int n_old = st->n_old;
    const double t_step = st->t, t0 = st->t0;
    const double tol = st->tol, rel_tol = st->rel_tol, outer_tol = st->outer_tol;
    const int max_iter = st->max_iter, n_outer = st->n_outer;
    double* __restrict__ x = a.vm;
    double* __restrict__ b = a.b;
    double* __restrict__ ax = a.ax;
    double* __restrict__ r = a.r;
    double* __restrict__ z = a.z;     // published: read by neighbours
    double* __restrict__ p = a.pA;    // own rows only
    double* __restrict__ ap = a.ap;   // own rows only
    unsigned epoch = 0;               // arrivals expected at the next barrier
    int set = 0;                      // partial buffer of the next reduction
    int n_solves = 0, status = 0;
    bool converged_outer = false, abort_step = false;
    long long step_iters = 0;
    double last_init = 0.0, last_res = 0.0;
    int last_iter = 0, last_v = 0;
    int bsrc_variant = -1;            // ddt coefficient set of the kept source

    for (int corr = 1;; ++corr) {
        const int v = ddt_variant(a, n_old);
        const double* __restrict__ diag = a.diag2 + size_t(v) * n;
        const double* __restrict__ rdiag = a.rdiag2 + size_t(v) * n;
        const double* __restrict__ sumA = a.sumA2 + size_t(v) * n;
        const double cft0 = a.cft0[v], cft00 = a.cft00[v];
        // --- general mesh: gradient of the current iterate for the
        // Laplacian's explicit correction, published for the neighbours
        CR* __restrict__ grad = static_cast<CR*>(a.grad);
        if (a.nc_gw) {
            for (unsigned c = first; c < n; c += stride) {
                CR g[3];
                nc_gradient<CR, W>(a, c, [x](long long q) { return __ldcg(&x[q]); }, g);
                __stcg(&grad[c], g[0]);
                __stcg(&grad[size_t(n) + c], g[1]);
                __stcg(&grad[2 * size_t(n) + c], g[2]);
            }
            if (!grid_barrier(st, epoch, a.spin_limit)) { abort_step = true; break; }
        }
        // --- source, A.x, r = b - A.x; sums of x and |r|.  The ddt, ionic
        // and stimulus parts of the source change between correctors only
        // with the ddt coefficient set (the first step creates the old-time
        // levels in its first corrector): kept in bsrc for the others.
        double s1[2] = {0.0, 0.0};
        const bool fresh = corr == 1 || v != bsrc_variant;
        bsrc_variant = v;
        auto rhs_row = [&](unsigned c) {
            double rhs;
            if (fresh) {
                const double V = a.vol[c];
                double ddt_src;
                if (a.ddt_backward)
                    ddt_src = a.rdt * V * (cft0 * a.vm_old[c] - cft00 * a.vm_oldold[c]);
                else
                    ddt_src = a.rdt * a.vm_old[c] * V;
                double bb = a.chicm * ddt_src;
                double su = -(a.chicm * a.iion[c]) * V;
                su = su + box_source(a, c, t0) * V;
                rhs = bb + su;
                a.bsrc[c] = rhs;
            } else {
                rhs = a.bsrc[c];
            }
            if (a.nc_gw)
                rhs = rhs + nc_correction<CR, W>(a, c, [grad, n](long long q, int k) {
                          return __ldcg(&grad[size_t(k) * n + size_t(q)]);
                      });
            return rhs;
        };
        for (unsigned c = first; c < n; c += 2 * stride) {
            const unsigned c2 = c + stride;
            const bool two = c2 < n;
            const double b0 = rhs_row(c), b1 = two ? rhs_row(c2) : 0.0;
            const double a0 = amul_cg<W>(a, ca, c, diag[c], x);
            const double a1 = two ? amul_cg<W>(a, ca, c2, diag[c2], x) : 0.0;
            const double r0 = b0 - a0, r1 = b1 - a1;
            b[c] = b0; ax[c] = a0; r[c] = r0;
            s1[0] += x[c];
            s1[1] += fabs(r0);
            if (two) {
                b[c2] = b1; ax[c2] = a1; r[c2] = r1;
                s1[0] += x[c2];
                s1[1] += fabs(r1);
            }
        }
        block_sums<2>(a.partial, set, s1);
        if (!grid_barrier(st, epoch, a.spin_limit)) { abort_step = true; break; }
        double g1[2];
        grid_sums<2>(a.partial, set, g1);
        set ^= 1;
        const double avg = g1[0] / double(n);
        // fvm::ddt created the old time levels
        if (n_old < 1) n_old = 1;
        if (a.ddt_backward && n_old < 2) n_old = 2;
        // --- normFactor, z = D^-1 r (published), z.r
        double s2[2] = {0.0, 0.0};
        for (unsigned c = first; c < n; c += stride) {
            const double pa = sumA[c] * avg;
            s2[0] += fabs(ax[c] - pa) + fabs(b[c] - pa);
            const double zc = rdiag[c] * r[c];
            __stcg(&z[c], zc);
            s2[1] += zc * r[c];
        }
        block_sums<2>(a.partial, set, s2);
        if (!grid_barrier(st, epoch, a.spin_limit)) { abort_step = true; break; }
        double g2[2];
        grid_sums<2>(a.partial, set, g2);
        set ^= 1;
        const double normf = g2[0] + 1e-20;
        const double init_res = g1[1] / normf;
        double res = init_res;
        double wArA = g2[1], beta = 0.0;
        int iter = 0;
        bool aborted = false;
        const auto conv = [&](double rr) {
            return rr < tol || (rel_tol > 1e-20 && rr < rel_tol * init_res);
        };
        if (!conv(res)) {
            for (;;) {
                // --- halo pass: w = A.z, p = z + beta p, A.p = w + beta A.p
                double s3[1] = {0.0};
                const bool first_it = iter == 0;
                for (unsigned c = first; c < n; c += 2 * stride) {
                    const unsigned c2 = c + stride;
                    const bool two = c2 < n;
                    const double w0 = amul_cg<W>(a, ca, c, diag[c], z);
                    const double w1 = two ? amul_cg<W>(a, ca, c2, diag[c2], z) : 0.0;
                    const double z0 = __ldcg(&z[c]);
                    const double z1 = two ? __ldcg(&z[c2]) : 0.0;
                    double p0, p1, q0, q1;
                    if (first_it) {
                        p0 = z0; p1 = z1; q0 = w0; q1 = w1;
                    } else {
                        p0 = z0 + beta * p[c];
                        q0 = w0 + beta * ap[c];
                        p1 = two ? z1 + beta * p[c2] : 0.0;
                        q1 = two ? w1 + beta * ap[c2] : 0.0;
                    }
                    p[c] = p0; ap[c] = q0;
                    s3[0] += q0 * p0;
                    if (two) {
                        p[c2] = p1; ap[c2] = q1;
                        s3[0] += q1 * p1;
                    }
                }
                block_sums<1>(a.partial, set, s3);
                if (!grid_barrier(st, epoch, a.spin_limit)) { aborted = true; break; }
                double g3[1];
                grid_sums<1>(a.partial, set, g3);
                set ^= 1;
                // checkSingularity and alpha, once per block
                double q3[2];
                gsync::block_scalars<2>(q3, [&](double* v) {
                    v[0] = fabs(g3[0]) / normf < 1e-300 ? 1.0 : 0.0;
                    v[1] = wArA / g3[0];
                });
                if (q3[0] != 0.0) break;
                const double alpha = q3[1];
                // --- update pass: x, r, z; |r| and z.r
                double s4[2] = {0.0, 0.0};
                for (unsigned c = first; c < n; c += 2 * stride) {
                    const unsigned c2 = c + stride;
                    const bool two = c2 < n;
                    const double x0 = x[c] + alpha * p[c];
                    const double r0 = r[c] - alpha * ap[c];
                    const double z0 = rdiag[c] * r0;
                    x[c] = x0; r[c] = r0;
                    __stcg(&z[c], z0);
                    s4[0] += fabs(r0);
                    s4[1] += z0 * r0;
                    if (two) {
                        const double x1 = x[c2] + alpha * p[c2];
                        const double r1 = r[c2] - alpha * ap[c2];
                        const double z1 = rdiag[c2] * r1;
                        x[c2] = x1; r[c2] = r1;
                        __stcg(&z[c2], z1);
                        s4[0] += fabs(r1);
                        s4[1] += z1 * r1;
                    }
                }
                block_sums<2>(a.partial, set, s4);
                if (!grid_barrier(st, epoch, a.spin_limit)) { aborted = true; break; }
                double g4[2];
                grid_sums<2>(a.partial, set, g4);
                set ^= 1;
                // the residual and beta, once per block
                double q4[2];
                gsync::block_scalars<2>(q4, [&](double* v) {
                    v[0] = g4[0] / normf;
                    v[1] = g4[1] / wArA;
                });
                res = q4[0];
                ++iter;
                ++step_iters;
                if (conv(res) || iter >= max_iter) {
                    if (!conv(res)) status |= CFG_ERR_PCG;
                    break;
                }
                if (step_iters >= a.iter_cap) {
                    // guard of the in-kernel loops: give up the step
                    status |= CFG_ERR_PCG;
                    aborted = true;
                    break;
                }
                wArA = g4[1];
                beta = q4[1];
            }
        }
        if (lead && n_solves < kMaxSolves) {
            st->iters[n_solves] = iter;
            st->init_r[n_solves] = init_res;
            st->final_r[n_solves] = res;
        }
        ++n_solves;
        last_init = init_res; last_res = res; last_iter = iter; last_v = v;
        if (aborted) { abort_step = true; break; }
        // pimpleLoop: the corrector after a converged one is the last
        if (converged_outer || corr + 1 > n_outer) break;
        if (init_res < outer_tol) converged_outer = true;
        // the next corrector reads other blocks' rows of x only through
        // amul_cg (L2), after the last barrier of this one
    }
    // --- activation time (MyocardiumDomain::updateActivationTime)
    if (abort_step) status |= CFG_ERR_PCG;
    else
        for (unsigned c = first; c < n; c += stride)
            activation(a, c, x[c], a.vm_old[c], t_step - a.dt);
    if (lead) {
        st->n_old = n_old;
        st->n_solves = n_solves;
        st->iter = last_iter;
        st->init_res = last_init;
        st->res = last_res;
        st->variant = last_v;
        st->step_iters = step_iters;
        st->corr = n_solves + 1;
        st->solve_active = 0;
        st->outer_active = 0;
        st->converged_outer = converged_outer ? 1 : 0;
    }
    if (status && threadIdx.x == 0) atomicOr(&st->status, status);
}

// ---------------------------------------------------------------- float pairs
// The same solve with the PCG in float pairs (the mixed form): the operator,
// the source and every vector of the iteration as (hi, lo) pairs on the FP32
// pipe, the system scaled by 2^pair_shift so that its quantities sit well
// inside the float range.  The corrector's source is formed in FP64 as above
// (once per corrector) and split; the iterate x is published as a pair (px)
// for the neighbours and written back to Vm in FP64 after each solve.  The
// scalars (alpha, beta, the residuals) are formed by every thread from the
// same block-order sums, so every block takes the same decisions without a
// shared-memory broadcast.

template <int W, class F>
__device__ __forceinline__ fp::P amul_pair(const DiffusionArgs& a, const CoopArgs& ca, unsigned c,
                                           fp::P d, F q)
{
    fp::Acc acc;
    acc.add_prod(d, q(c));
    if (a.sx) {
        const unsigned nx = unsigned(a.sx), nxy = nx * unsigned(a.sy);
        const unsigned line = fdiv(c, ca.div_nx), i = c - line * nx;
        const unsigned k = fdiv(line, ca.div_ny), j = line - k * unsigned(a.sy);
        if (k > 0) acc.sub_prod(a.pcz, q(c - nxy));
        if (j > 0) acc.sub_prod(a.pcy, q(c - nx));
        if (i > 0) acc.sub_prod(a.pcx, q(c - 1));
        if (i + 1 < nx) acc.sub_prod(a.pcx, q(c + 1));
        if (j + 1 < unsigned(a.sy)) acc.sub_prod(a.pcy, q(c + nx));
        if (k + 1 < unsigned(a.sz)) acc.sub_prod(a.pcz, q(c + nxy));
    } else if constexpr (W > 0) {
#pragma unroll
        for (int e = 0; e < W; ++e)
            acc.sub_prod(ld_stream(&a.pcoef[(long long)e * a.n + c]),
                         q(unsigned(ld_stream(&a.ell_col[(long long)e * a.n + c]))));
    } else {
        const int cnt = a.ell_cnt[c];
        for (int e = 0; e < cnt; ++e)
            acc.sub_prod(a.pcoef[(long long)e * a.n + c],
                         q(unsigned(a.ell_col[(long long)e * a.n + c])));
    }
    return acc.value();
}

template <class CR, int W>
__global__ void __launch_bounds__(kCoopBlock, 2) k_implicit_pair(DiffusionArgs a, CoopArgs ca)
{
    using fp::P;
    PcgState* st = a.st;
    const unsigned n = unsigned(a.n);
    const unsigned stride = gridDim.x * blockDim.x;
    const unsigned first = blockIdx.x * blockDim.x + threadIdx.x;
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    int n_old = st->n_old;
    const double t_step = st->t, t0 = st->t0;
    const bool use_rel = st->rel_tol > 1e-20;
    const P tol = fp::split(st->tol), outer_tol = fp::split(st->outer_tol);
    const P rel = fp::split(st->rel_tol);
    const int max_iter = st->max_iter, n_outer = st->n_outer;
    const int sh = a.pair_shift;
    // the ratio sum|r| / normFactor is scale free when the small number
    // lduMatrix adds to normFactor is scaled with the system
    const P small = fp::split(1e-20, sh);
    const P count = fp::split(double(n));
    double* __restrict__ x = a.vm;
    P* __restrict__ px = a.px;                          // published
    P* __restrict__ b = reinterpret_cast<P*>(a.b);
    P* __restrict__ ax = reinterpret_cast<P*>(a.ax);
    P* __restrict__ r = reinterpret_cast<P*>(a.r);
    P* __restrict__ z = reinterpret_cast<P*>(a.z);      // published
    P* __restrict__ p = reinterpret_cast<P*>(a.pA);
    P* __restrict__ ap = reinterpret_cast<P*>(a.ap);
    float2* partial = reinterpret_cast<float2*>(a.partial);
    unsigned epoch = 0;
    int set = 0;
    int n_solves = 0, status = 0;
    bool converged_outer = false, abort_step = false;
    long long step_iters = 0;
    P last_init = fp::make(0.0f), last_res = fp::make(0.0f);
    int last_iter = 0, last_v = 0;
    int bsrc_variant = -1;

    for (int corr = 1;; ++corr) {
        const int v = ddt_variant(a, n_old);
        const P* __restrict__ diag = a.pdiag2 + size_t(v) * n;
        const P* __restrict__ rdiag = a.prdiag2 + size_t(v) * n;
        const P* __restrict__ sumA = a.psumA2 + size_t(v) * n;
        const double cft0 = a.cft0[v], cft00 = a.cft00[v];
        // the iterate of the neighbours: Vm itself in the first corrector,
        // the published pair afterwards
        const bool from_vm = corr == 1;
        const auto xq = [x, px, from_vm](unsigned q) {
            return from_vm ? fp::split(__ldcg(&x[q])) : __ldcg(&px[q]);
        };
        CR* __restrict__ grad = static_cast<CR*>(a.grad);
        if (a.nc_gw) {
            for (unsigned c = first; c < n; c += stride) {
                CR g[3];
                nc_gradient<CR, W>(a, c, [&xq](long long q) { return xq(unsigned(q)); }, g);
                __stcg(&grad[c], g[0]);
                __stcg(&grad[size_t(n) + c], g[1]);
                __stcg(&grad[2 * size_t(n) + c], g[2]);
            }
            if (!grid_barrier(st, epoch, a.spin_limit)) { abort_step = true; break; }
        }
        // --- source (FP64, split), A.x, r = b - A.x; sums of x and |r|
        P s1[2] = {fp::make(0.0f), fp::make(0.0f)};
        const bool fresh = corr == 1 || v != bsrc_variant;
        bsrc_variant = v;
        const auto row_rhs = [&](unsigned c) {
            double rhs;
            if (fresh) {
                const double V = a.vol[c];
                double ddt_src;
                if (a.ddt_backward)
                    ddt_src = a.rdt * V * (cft0 * a.vm_old[c] - cft00 * a.vm_oldold[c]);
                else
                    ddt_src = a.rdt * a.vm_old[c] * V;
                double bb = a.chicm * ddt_src;
                double su = -(a.chicm * a.iion[c]) * V;
                su = su + box_source(a, c, t0) * V;
                rhs = bb + su;
                a.bsrc[c] = rhs;
            } else {
                rhs = a.bsrc[c];
            }
            if (a.nc_gw)
                rhs = rhs + nc_correction<CR, W>(a, c, [grad, n](long long q, int k) {
                          return __ldcg(&grad[size_t(k) * n + size_t(q)]);
                      });
            return fp::split(rhs, sh);
        };
        const auto row_res = [&](unsigned c, P bc, P axc) {
            const P xc = xq(c);
            const P rc = fp::sub(bc, axc);
            b[c] = bc; ax[c] = axc; r[c] = rc;
            if (from_vm) __stcg(&px[c], xc);
            s1[0] = fp::add(s1[0], xc);
            s1[1] = fp::add(s1[1], fp::abs(rc));
        };
        for (unsigned c = first; c < n; c += 2 * stride) {
            const unsigned c2 = c + stride;
            const bool two = c2 < n;
            const P b0 = row_rhs(c);
            const P b1 = two ? row_rhs(c2) : fp::make(0.0f);
            const P a0 = amul_pair<W>(a, ca, c, diag[c], xq);
            const P a1 = two ? amul_pair<W>(a, ca, c2, diag[c2], xq) : fp::make(0.0f);
            row_res(c, b0, a0);
            if (two) row_res(c2, b1, a1);
        }
        gsync::block_sums_pair<kCoopBlock, 2>(partial, set, s1);
        if (!grid_barrier(st, epoch, a.spin_limit)) { abort_step = true; break; }
        P g1[2];
        gsync::grid_sums_pair<2>(partial, set, g1);
        set ^= 1;
        const P avg = fp::div(g1[0], count);
        if (n_old < 1) n_old = 1;
        if (a.ddt_backward && n_old < 2) n_old = 2;
        // --- normFactor, z = D^-1 r (published), z.r
        P s2[2] = {fp::make(0.0f), fp::make(0.0f)};
        const auto norm_row = [&](unsigned c, P sa, P axc, P bc, P rc, P m) {
            const P pa = fp::mul(sa, avg);
            s2[0] = fp::add(s2[0], fp::add(fp::abs(fp::sub(axc, pa)), fp::abs(fp::sub(bc, pa))));
            const P zc = fp::mul(m, rc);
            __stcg(&z[c], zc);
            s2[1] = fp::madd(zc, rc, s2[1]);
        };
        for (unsigned c = first; c < n; c += 2 * stride) {
            const unsigned c2 = c + stride;
            const bool two = c2 < n;
            const unsigned d = two ? c2 : c;
            const P sa0 = sumA[c], sa1 = sumA[d], a0 = ax[c], a1 = ax[d], b0 = b[c], b1 = b[d];
            const P r0 = r[c], r1 = r[d], m0 = rdiag[c], m1 = rdiag[d];
            norm_row(c, sa0, a0, b0, r0, m0);
            if (two) norm_row(c2, sa1, a1, b1, r1, m1);
        }
        gsync::block_sums_pair<kCoopBlock, 2>(partial, set, s2);
        if (!grid_barrier(st, epoch, a.spin_limit)) { abort_step = true; break; }
        P g2[2];
        gsync::grid_sums_pair<2>(partial, set, g2);
        set ^= 1;
        const P normf = fp::add(g2[0], small);
        const P init_res = fp::div(g1[1], normf);
        const P rel_init = fp::mul(rel, init_res);
        P res = init_res;
        P wArA = g2[1], beta = fp::make(0.0f);
        int iter = 0;
        bool aborted = false;
        const auto conv = [&](P rr) {
            return fp::less(rr, tol) || (use_rel && fp::less(rr, rel_init));
        };
        if (!conv(res)) {
            for (;;) {
                // --- halo pass: w = A.z, p = z + beta p, A.p = w + beta A.p
                P s3[1] = {fp::make(0.0f)};
                const bool first_it = iter == 0;
                const auto zq = [z](unsigned q) { return __ldcg(&z[q]); };
                const auto dir = [&](unsigned c, P w) {
                    const P zc = __ldcg(&z[c]);
                    P pc = zc, qc = w;
                    if (!first_it) {
                        pc = fp::madd(beta, p[c], zc);
                        qc = fp::madd(beta, ap[c], w);
                    }
                    p[c] = pc; ap[c] = qc;
                    s3[0] = fp::madd(qc, pc, s3[0]);
                };
                // two rows per trip: both products' loads are in flight together
                for (unsigned c = first; c < n; c += 2 * stride) {
                    const unsigned c2 = c + stride;
                    const bool two = c2 < n;
                    const P w0 = amul_pair<W>(a, ca, c, diag[c], zq);
                    const P w1 = two ? amul_pair<W>(a, ca, c2, diag[c2], zq) : fp::make(0.0f);
                    dir(c, w0);
                    if (two) dir(c2, w1);
                }
                gsync::block_sums_pair<kCoopBlock, 1>(partial, set, s3);
                if (!grid_barrier(st, epoch, a.spin_limit)) { aborted = true; break; }
                P g3[1];
                gsync::grid_sums_pair<1>(partial, set, g3);
                set ^= 1;
                if (g3[0].x == 0.0f) break;   // checkSingularity
                const P alpha = fp::div(wArA, g3[0]);
                const P nalpha = fp::neg(alpha);
                // --- update pass: x, r, z; |r| and z.r
                P s4[2] = {fp::make(0.0f), fp::make(0.0f)};
                // two rows per trip, all of their loads issued first (the
                // pass streams from HBM when the vectors exceed L2)
                for (unsigned c = first; c < n; c += 2 * stride) {
                    const unsigned c2 = c + stride;
                    const bool two = c2 < n;
                    const unsigned d = two ? c2 : c;
                    const P p0 = p[c], p1 = p[d], q0 = ap[c], q1 = ap[d];
                    const P r0 = r[c], r1 = r[d], x0 = __ldcg(&px[c]), x1 = __ldcg(&px[d]);
                    const P m0 = rdiag[c], m1 = rdiag[d];
                    __stcg(&px[c], fp::madd(alpha, p0, x0));
                    const P rc = fp::madd(nalpha, q0, r0);
                    r[c] = rc;
                    const P zc = fp::mul(m0, rc);
                    __stcg(&z[c], zc);
                    s4[0] = fp::add(s4[0], fp::abs(rc));
                    s4[1] = fp::madd(zc, rc, s4[1]);
                    if (two) {
                        __stcg(&px[c2], fp::madd(alpha, p1, x1));
                        const P rd = fp::madd(nalpha, q1, r1);
                        r[c2] = rd;
                        const P zd = fp::mul(m1, rd);
                        __stcg(&z[c2], zd);
                        s4[0] = fp::add(s4[0], fp::abs(rd));
                        s4[1] = fp::madd(zd, rd, s4[1]);
                    }
                }
                gsync::block_sums_pair<kCoopBlock, 2>(partial, set, s4);
                if (!grid_barrier(st, epoch, a.spin_limit)) { aborted = true; break; }
                P g4[2];
                gsync::grid_sums_pair<2>(partial, set, g4);
                set ^= 1;
                res = fp::div(g4[0], normf);
                ++iter;
                ++step_iters;
                if (conv(res) || iter >= max_iter) {
                    if (!conv(res)) status |= CFG_ERR_PCG;
                    break;
                }
                if (step_iters >= a.iter_cap) {
                    status |= CFG_ERR_PCG;
                    aborted = true;
                    break;
                }
                beta = fp::div(g4[1], wArA);
                wArA = g4[1];
            }
        }
        if (lead && n_solves < kMaxSolves) {
            st->iters[n_solves] = iter;
            st->init_r[n_solves] = fp::join(init_res);
            st->final_r[n_solves] = fp::join(res);
        }
        ++n_solves;
        last_init = init_res; last_res = res; last_iter = iter; last_v = v;
        if (aborted) { abort_step = true; break; }
        if (converged_outer || corr + 1 > n_outer) break;
        if (fp::less(init_res, outer_tol)) converged_outer = true;
    }
    if (abort_step) status |= CFG_ERR_PCG;
    else
        // the step's iterate back into Vm (own rows: between correctors the
        // neighbours read px, so Vm is written once), and the activation time
        for (unsigned c = first; c < n; c += stride) {
            const double xc = fp::join(__ldcg(&px[c]));
            x[c] = xc;
            activation(a, c, xc, a.vm_old[c], t_step - a.dt);
        }
    if (lead) {
        st->n_old = n_old;
        st->n_solves = n_solves;
        st->iter = last_iter;
        st->init_res = fp::join(last_init);
        st->res = fp::join(last_res);
        st->variant = last_v;
        st->step_iters = step_iters;
        st->corr = n_solves + 1;
        st->solve_active = 0;
        st->outer_active = 0;
        st->converged_outer = converged_outer ? 1 : 0;
    }
    if (status && threadIdx.x == 0) atomicOr(&st->status, status);
}

// Host helpers: fast-division constants and the cooperative launch.
static FastDiv make_fastdiv(unsigned d)
{
    unsigned s = 0;
    while ((1ull << s) < d) ++s;
    const unsigned long long m = ((1ull << 32) * ((1ull << s) - d)) / d + 1;
    return FastDiv{unsigned(m), s};
}

int coop_grid_blocks(long long n)
{
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    per_sm = 1 << 30;
    const void* fns[] = {(const void*)k_implicit_coop<double, 0>, (const void*)k_implicit_coop<float, 0>,
                         (const void*)k_implicit_coop<double, 4>, (const void*)k_implicit_coop<float, 4>,
                         (const void*)k_implicit_coop<double, 6>, (const void*)k_implicit_coop<float, 6>,
                         (const void*)k_implicit_pair<float, 0>, (const void*)k_implicit_pair<float, 4>,
                         (const void*)k_implicit_pair<float, 6>};
    for (const void* f : fns) {
        int k = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, f, kCoopBlock, 0) != cudaSuccess)
            return 0;
        per_sm = per_sm < k ? per_sm : k;
    }
    long long want = (n + kCoopBlock - 1) / kCoopBlock;
    long long cap = (long long)sms * per_sm;
    return int(want < cap ? want : cap);
}

cudaError_t launch_implicit_coop(const DiffusionArgs& a, int blocks, cudaStream_t s)
{
    CoopArgs ca{};
    if (a.sx) {
        ca.div_nx = make_fastdiv(unsigned(a.sx));
        ca.div_ny = make_fastdiv(unsigned(a.sy));
    }
    DiffusionArgs args = a;
    void* params[] = {&args, &ca};
    // rows of a general mesh visited over the full ELL width when it is 4
    // (tetrahedra) or 6 (hexahedra)
    const int w = (!a.sx && (a.width == 4 || a.width == 6)) ? a.width : 0;
    void* fn = nullptr;
    if (a.pair)
        fn = w == 4 ? (void*)k_implicit_pair<float, 4> : w == 6 ? (void*)k_implicit_pair<float, 6>
                                                               : (void*)k_implicit_pair<float, 0>;
    else if (a.nc_fp32)
        fn = w == 4 ? (void*)k_implicit_coop<float, 4> : w == 6 ? (void*)k_implicit_coop<float, 6>
                                                                : (void*)k_implicit_coop<float, 0>;
    else
        fn = w == 4 ? (void*)k_implicit_coop<double, 4> : w == 6 ? (void*)k_implicit_coop<double, 6>
                                                                 : (void*)k_implicit_coop<double, 0>;
    {
        // as many co-resident blocks as the chosen kernel fits: two per SM
        // for the float-pair solve and for tetrahedral rows, whose kernels
        // are built for 64 registers a thread (on the slab the FP64 kernel
        // measured slower that way: 0.228 against 0.190 ms per step), one
        // for the others
        int dev = 0, sms = 0, per = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kCoopBlock, 0) == cudaSuccess) {
            const long long want = (a.n + kCoopBlock - 1) / kCoopBlock;
            const long long cap = (long long)sms * per;
            blocks = int(want < cap ? want : cap);
        }
    }
    return cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kCoopBlock), params, 0, s);
}

}  // namespace cfg
