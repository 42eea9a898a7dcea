// Bidomain step (BidomainSolver, bidomainSolver.C:36-263, in
// MyocardiumDomain's staggered advance) on the GPU.
//
// Per step: box stimulus, the ionic update (cfg_ionic, either form), then per
// PIMPLE corrector
//   phiE:  laplacian(Gi + Ge, phiE) == -div(Gi & grad(Vm)), setReference
//   Vm:    chi Cm ddt(Vm) == laplacian(Gi, Vm) + div(Gi & grad(phiE))
//                            - chi Cm Iion + src
//   phiI = Vm + phiE,
// and the activation time.  The two Laplacians are solved by diagonal-
// preconditioned CG with lduMatrix's normFactor and L1 residual, the phiE one
// in its negated (positive definite) form; the explicit divergence of
// Gi & grad(x) is Gauss linear over the faces with gaussGrad's zeroGradient
// wall values.  Operators are per-row ELL slots (column, the two Laplacian
// coefficients, gradient weights, face area vector and interpolation
// weight).  On meshes whose Laplacians need explicit non-orthogonal or
// tangential corrections (tetrahedra, rotated fibres) both systems carry
// them in their sources, evaluated from the current phiE or Vm before each
// solve; solutionAlgorithm explicit runs solveDiffusionExplicit.
//
// Each PCG solve is one persistent cooperative launch (every block resident,
// rows strided over the grid) with two grid barriers per iteration: the
// direction pass forms p = z + beta p_old and applies A to it, reading the
// neighbours' z and previous p through L2 and forming their p the same way
// (lduMatrix's PCG applies A to the new direction; p is double-buffered so
// that no row is overwritten while a neighbour reads it), then the update
// pass x += alpha p, r -= alpha A p, z = D^-1 r.  Block sums are added in
// block order by every block, so the scalars are identical everywhere and
// results reproducible bit for bit.  Barrier waits are bounded (the step then
// reports CFG_ERR_PCG).  Where cooperative launch is not available the same
// iteration runs as a kernel sequence with its scalars on the device, two
// launches per iteration, replayed in chunks from a CUDA graph.  That is the
// FP64 solve; the mixed form's default is the float-pair, single-reduction
// solve (k_pcg_pair, one grid barrier per iteration).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "geometry.h"
#include "grid_sync.cuh"
#include "host_common.h"
#include "ionic_host.h"

namespace fp = cfg::fp;

namespace {

constexpr int kBlock = 256;
constexpr int kChunk = 16;          // PCG iterations enqueued per host check
constexpr int kMaxSolves = 16;

struct BdOp {
    long long n;
    int width;
    const int* col;             // [slot][cell]
    const unsigned char* cnt;   // [cell]
    const double* coef_i;       // [slot][cell] Laplacian coefficient of Gi
    const double* coef_e;       // [slot][cell] of Gi + Ge
    const double* gw;           // [3][slot][cell] gradient weight of (x_nb - x_c)
    const double* sf;           // [3][slot][cell] face area vector (owner -> neighbour)
    const double* w;            // [slot][cell] the face's owner interpolation weight
    const unsigned char* own;   // [slot][cell] 1: the row cell owns the face
    const double* bw;           // [3][cell] wall factor of the divergence
    const double* vol;
    double G[6];                // Gi: xx xy xz yy yz zz
};

struct PcgScalars {
    double avg, normf, init_res, res, wArA, wApA, alpha, beta, abs_r;
    double tol, rel;
    int iter, max_iter, done, status;
};

__device__ __forceinline__ double block_sum(double v, double* sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < kBlock / 32; ++k) s += sh[k];
    return s;   // valid in thread 0
}

// (M q)_c for M = diag - off-diagonal coefficients (lduMatrix::Amul order:
// diagonal, then the row's slots in column order)
__device__ __forceinline__ double amul(const BdOp& op, const double* coef, const double* diag,
                                      const double* q, long long c)
{
    double acc = diag[c] * q[c];
    const int k = op.cnt[c];
    for (int e = 0; e < k; ++e) {
        const long long i = (long long)e * op.n + c;
        acc += (-coef[i]) * q[op.col[i]];
    }
    return acc;
}

__device__ __forceinline__ double row_sum(const BdOp& op, const double* coef, const double* diag,
                                         long long c)
{
    double acc = diag[c];
    const int k = op.cnt[c];
    for (int e = 0; e < k; ++e) acc += -coef[(long long)e * op.n + c];
    return acc;
}

__global__ void k_gradient(BdOp op, const double* __restrict__ x, double* __restrict__ g)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c >= op.n) return;
    const long long wn = (long long)op.width * op.n;
    const double xc = x[c];
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int e = 0; e < op.cnt[c]; ++e) {
        const long long i = (long long)e * op.n + c;
        const double dv = x[op.col[i]] - xc;
        g0 += op.gw[i] * dv;
        g1 += op.gw[wn + i] * dv;
        g2 += op.gw[2 * wn + i] * dv;
    }
    g[c] = g0;
    g[op.n + c] = g1;
    g[2 * op.n + c] = g2;
}

__device__ __forceinline__ void gamma_g(const double* G, double g0, double g1, double g2,
                                        double* u)
{
    u[0] = G[0] * g0 + G[1] * g1 + G[2] * g2;
    u[1] = G[1] * g0 + G[3] * g1 + G[4] * g2;
    u[2] = G[2] * g0 + G[4] * g1 + G[5] * g2;
}

// out_c = V_c * (D_c / V_c), D_c the sum over the cell's faces of
// Sf . (G grad x)_f (outward) plus the walls: fvc::div per volume, times V as
// the equation's source takes it
__global__ void k_div_gamma_grad(BdOp op, const double* __restrict__ g, double* __restrict__ out)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c >= op.n) return;
    const long long n = op.n, wn = (long long)op.width * n;
    double uc[3];
    gamma_g(op.G, g[c], g[n + c], g[2 * n + c], uc);
    double div = 0.0;
    for (int e = 0; e < op.cnt[c]; ++e) {
        const long long i = (long long)e * n + c;
        const long long nb = op.col[i];
        double un[3];
        gamma_g(op.G, g[nb], g[n + nb], g[2 * n + nb], un);
        const double w = op.w[i];
        double uf[3];
        if (op.own[i]) {
            for (int k = 0; k < 3; ++k) uf[k] = w * (uc[k] - un[k]) + un[k];
        } else {
            for (int k = 0; k < 3; ++k) uf[k] = w * (un[k] - uc[k]) + uc[k];
        }
        const double flux = op.sf[i] * uf[0] + op.sf[wn + i] * uf[1] + op.sf[2 * wn + i] * uf[2];
        div += op.own[i] ? flux : -flux;
    }
    div += op.bw[c] * g[c] + op.bw[n + c] * g[n + c] + op.bw[2 * n + c] * g[2 * n + c];
    const double V = op.vol[c];
    out[c] = V * (div / V);
}

struct StimArgs {
    int n_boxes;
    double lo[8][3], hi[8][3], start[8], dur[8], amp[8];
};

__global__ void k_stimulus(long long n, const double* __restrict__ centres, StimArgs s, double t0,
                           double* __restrict__ src)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c >= n) return;
    const double* p = centres + 3 * c;
    double v = 0.0;
    for (int b = 0; b < s.n_boxes; ++b) {
        if (t0 < s.start[b] || t0 > s.start[b] + s.dur[b]) continue;
        if (p[0] >= s.lo[b][0] && p[0] <= s.hi[b][0] && p[1] >= s.lo[b][1] && p[1] <= s.hi[b][1] &&
            p[2] >= s.lo[b][2] && p[2] <= s.hi[b][2])
            v += s.amp[b];
    }
    src[c] = v;
}

// phiE right-hand side and diagonal of the negated system: b = V div(Gi grad Vm)
// (= -source), diag = sum of the coefficients; at the reference cell the
// diagonal doubles and b gains the diagonal times the reference value
// V fvc::div of the Laplacian's explicit correction fluxes (Gauss linear
// corrected on a non-orthogonal mesh, or a conductivity not aligned with the
// faces) at row c, from the cell gradient g of the field: each face's flux
// k.(w (g_P - g_N) + g_N) with the row's sign, in slot order, then the wall
// term bk.g_c (gaussLaplacianScheme's faceFluxCorrection, restated)
__global__ void k_correction(BdOp op, const double* __restrict__ kv,
                             const double* __restrict__ bk, const double* __restrict__ g,
                             double* __restrict__ out)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c >= op.n) return;
    const long long n = op.n, wn = (long long)op.width * n;
    const double g0 = g[c], g1 = g[n + c], g2 = g[2 * n + c];
    double s = 0.0;
    for (int e = 0; e < op.cnt[c]; ++e) {
        const long long i = (long long)e * n + c;
        const long long nb = op.col[i];
        const double om = op.own[i] ? op.w[i] : 1.0 - op.w[i];
        const double n0 = g[nb], n1 = g[n + nb], n2 = g[2 * n + nb];
        const double f0 = om * (g0 - n0) + n0;
        const double f1 = om * (g1 - n1) + n1;
        const double f2 = om * (g2 - n2) + n2;
        s += kv[i] * f0 + kv[wn + i] * f1 + kv[2 * wn + i] * f2;
    }
    s += bk[c] * g0 + bk[n + c] * g1 + bk[2 * n + c] * g2;
    out[c] = s;
}

// phiE system; cv (may be null) is the Laplacian's explicit correction of
// the current phiE, which fvm::laplacian takes off the source
__global__ void k_phie_system(BdOp op, const double* __restrict__ dv,
                              const double* __restrict__ cv, long long ref,
                              double ref_value, double* __restrict__ diag,
                              double* __restrict__ rdiag, double* __restrict__ b)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c >= op.n) return;
    double d = 0.0;
    for (int e = 0; e < op.cnt[c]; ++e) d -= op.coef_e[(long long)e * op.n + c];
    // the reference form's diagonal is d (negative); setReference: source +=
    // d * value, d += d; negated here
    double src = -dv[c];
    if (cv) src = src - cv[c];
    if (c == ref) {
        src = src + d * ref_value;
        d = d + d;
    }
    diag[c] = -d;
    rdiag[c] = 1.0 / (-d);
    b[c] = -src;
}

struct VmArgs {
    double chicm, rdt, cft, cft0, cft00;
    int backward;
};

// Vm system: diag = chi Cm ddt diagonal + sum of the Gi coefficients; b as
// the reference assembles the source (ddt, -chi Cm Iion V, + src V) plus the
// explicit V div(Gi grad phiE)
__global__ void k_vm_system(BdOp op, VmArgs a, const double* __restrict__ vm_old,
                            const double* __restrict__ vm_oldold, const double* __restrict__ iion,
                            const double* __restrict__ src, const double* __restrict__ dp,
                            const double* __restrict__ cv, double* __restrict__ diag,
                            double* __restrict__ rdiag, double* __restrict__ b)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c >= op.n) return;
    const double V = op.vol[c];
    double ddt_diag, ddt_src;
    if (a.backward) {
        ddt_diag = (a.cft * a.rdt) * V;
        ddt_src = a.rdt * V * (a.cft0 * vm_old[c] - a.cft00 * vm_oldold[c]);
    } else {
        ddt_diag = a.rdt * V;
        ddt_src = a.rdt * vm_old[c] * V;
    }
    double lapdiag = 0.0;
    for (int e = 0; e < op.cnt[c]; ++e) lapdiag -= op.coef_i[(long long)e * op.n + c];
    diag[c] = a.chicm * ddt_diag - lapdiag;
    rdiag[c] = 1.0 / diag[c];
    double bb = a.chicm * ddt_src;
    double su = -(a.chicm * iion[c]) * V;
    su = su + src[c] * V;
    bb = bb + su;
    if (cv) bb = bb + cv[c];   // the Laplacian's explicit correction of the current Vm
    b[c] = bb + dp[c];
}

// Explicit algorithm: chi Cm ddt(Vm) == V div(Gi grad(Vm + phiE)) - chi Cm
// Iion V + src V with the diagonal matrix of fvm::ddt, solved as source over
// diagonal; dv holds V div(Gi grad(Vm + phiE))
__global__ void k_vm_explicit(BdOp op, VmArgs a, const double* __restrict__ vm_old,
                              const double* __restrict__ vm_oldold,
                              const double* __restrict__ iion, const double* __restrict__ src,
                              const double* __restrict__ dv, double* __restrict__ vm)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c >= op.n) return;
    const double V = op.vol[c];
    double ddt_diag, ddt_src;
    if (a.backward) {
        ddt_diag = (a.cft * a.rdt) * V;
        ddt_src = a.rdt * V * (a.cft0 * vm_old[c] - a.cft00 * vm_oldold[c]);
    } else {
        ddt_diag = a.rdt * V;
        ddt_src = a.rdt * vm_old[c] * V;
    }
    const double diag = a.chicm * ddt_diag;
    double bb = a.chicm * ddt_src;
    double su = -(a.chicm * iion[c]) * V;
    su = su + src[c] * V;
    bb = bb + su;
    vm[c] = (bb + dv[c]) / diag;
}

// x = u + v (Vm + phiE for the explicit divergence)
__global__ void k_add(long long n, const double* u, const double* v, double* x)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c < n) x[c] = u[c] + v[c];
}

// --- PCG kernels (device scalars in PcgScalars) ---------------------------
// Each kernel ends with its reduction: the blocks' sums go to the partial
// buffer, and the last block to finish (a ticket counter) adds them in block
// order and updates the scalars of its stage (0: begin, 1: norm, 2:
// direction, 3: update), so an iteration is two launches.

template <int K>
__device__ __forceinline__ void stage_end(double (&v)[K], double* partial, unsigned* ticket,
                                          int stage, long long n, PcgScalars* st)
{
    __shared__ double sh[kBlock / 32];
    __shared__ bool last;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double s = block_sum(v[k], sh);
        if (threadIdx.x == 0) partial[(long long)k * gridDim.x + blockIdx.x] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s[2] = {0.0, 0.0};
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double a = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += kBlock)
            a += __ldcg(&partial[(long long)k * gridDim.x + b]);
        s[k] = block_sum(a, sh);
    }
    if (threadIdx.x != 0) return;
    *ticket = 0u;
    const auto conv = [&](double rr) {
        return rr < st->tol || (st->rel > 1e-20 && rr < st->rel * st->init_res);
    };
    if (stage == 0) {
        st->avg = s[0] / double(n);
        st->abs_r = s[1];
    } else if (stage == 1) {
        st->normf = s[0] + 1e-20;
        st->init_res = st->abs_r / st->normf;
        st->res = st->init_res;
        st->wArA = s[1];
        st->iter = 0;
        st->status = 0;
        st->done = conv(st->init_res) ? 1 : 0;
    } else if (stage == 2) {
        st->wApA = s[0];
        if (fabs(st->wApA) / st->normf < 1e-300) st->done = 1;   // checkSingularity
        else st->alpha = st->wArA / st->wApA;
    } else {
        st->res = s[0] / st->normf;
        st->iter = st->iter + 1;
        if (conv(st->res) || st->iter >= st->max_iter) {
            if (!conv(st->res)) st->status = 1;
            st->done = 1;
        } else {
            st->beta = s[1] / st->wArA;
            st->wArA = s[1];
        }
    }
}

struct PcgArgs {
    BdOp op;
    const double* coef;
    const double* diag;
    const double* rdiag;      // 1/diag: the diagonal preconditioner multiplies by it
    const double* b;
    double *x, *ax, *r, *z, *p, *ap, *partial;
    unsigned* ticket;
    PcgScalars* st;
};

__global__ void k_pcg_begin(PcgArgs a)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (c < a.op.n) {
        const double ax = amul(a.op, a.coef, a.diag, a.x, c);
        const double rr = a.b[c] - ax;
        a.ax[c] = ax;
        a.r[c] = rr;
        v[0] = a.x[c];
        v[1] = fabs(rr);
    }
    stage_end<2>(v, a.partial, a.ticket, 0, a.op.n, a.st);
}

__global__ void k_pcg_norm(PcgArgs a)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (c < a.op.n) {
        const double pa = row_sum(a.op, a.coef, a.diag, c) * a.st->avg;
        v[0] = fabs(a.ax[c] - pa) + fabs(a.b[c] - pa);
        const double zc = a.rdiag[c] * a.r[c];
        a.z[c] = zc;
        v[1] = zc * a.r[c];
    }
    stage_end<2>(v, a.partial, a.ticket, 1, a.op.n, a.st);
}

// w = M z, p = z + beta p, M p = w + beta M p (linearity), sum p.Mp
__global__ void k_pcg_direction(PcgArgs a)
{
    if (a.st->done) return;
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    double v[1] = {0.0};
    if (c < a.op.n) {
        const double w = amul(a.op, a.coef, a.diag, a.z, c);
        double pc, qc;
        if (a.st->iter == 0) {
            pc = a.z[c];
            qc = w;
        } else {
            pc = a.z[c] + a.st->beta * a.p[c];
            qc = w + a.st->beta * a.ap[c];
        }
        a.p[c] = pc;
        a.ap[c] = qc;
        v[0] = qc * pc;
    }
    stage_end<1>(v, a.partial, a.ticket, 2, a.op.n, a.st);
}

__global__ void k_pcg_update(PcgArgs a)
{
    if (a.st->done) return;
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (c < a.op.n) {
        const double al = a.st->alpha;
        a.x[c] = a.x[c] + al * a.p[c];
        const double rr = a.r[c] - al * a.ap[c];
        a.r[c] = rr;
        const double zc = a.rdiag[c] * rr;
        a.z[c] = zc;
        v[0] = fabs(rr);
        v[1] = zc * rr;
    }
    stage_end<2>(v, a.partial, a.ticket, 3, a.op.n, a.st);
}

// --- the persistent solve --------------------------------------------------
constexpr int kCoopBlock = 512;

struct CoopPcgArgs {
    PcgArgs a;
    double* p_alt;            // second direction buffer
    double* partial;          // [2 sets][2][gridDim.x]
    unsigned* bar_count;      // grid barrier (zeroed before the launch)
    int* bar_abort;
    long long spin_limit;
};

// The direction of row q: z + beta p_old (z at the first iteration), the
// same operations wherever a row's direction is formed.
__device__ __forceinline__ double direction(const double* z, const double* p_old, double beta,
                                            bool first, long long q)
{
    const double zq = __ldcg(&z[q]);
    return first ? zq : __fma_rn(beta, __ldcg(&p_old[q]), zq);
}

// acc plus, over the row's slots in slot (column) order, -coef * f(column):
// lduMatrix::Amul's order after the diagonal term.  W > 0: every row is
// visited over the full ELL width (padded slots have column 0 and
// coefficient 0, an exact zero term), so all of a row's loads are issued
// together; W == 0: the row's own count.
template <int W, class F>
__device__ __forceinline__ double offdiag(const BdOp& op, const double* coef, long long c, F f,
                                          double acc)
{
    if constexpr (W > 0) {
        double v[W], k[W];
#pragma unroll
        for (int e = 0; e < W; ++e) {
            const long long i = (long long)e * op.n + c;
            k[e] = coef[i];
            v[e] = f(op.col[i]);
        }
#pragma unroll
        for (int e = 0; e < W; ++e) acc += (-k[e]) * v[e];
    } else {
        const int k = op.cnt[c];
        for (int e = 0; e < k; ++e) {
            const long long i = (long long)e * op.n + c;
            acc += (-coef[i]) * f(op.col[i]);
        }
    }
    return acc;
}

template <int W>
__global__ void __launch_bounds__(kCoopBlock, 1) k_pcg_coop(CoopPcgArgs ca)
{
    using namespace cfg::gsync;
    const PcgArgs& a = ca.a;
    const BdOp& op = a.op;
    PcgScalars* st = a.st;
    const long long n = op.n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long first = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const double tol = st->tol, rel = st->rel;
    const int max_iter = st->max_iter;
    unsigned epoch = 0;
    int set = 0;
    bool aborted = false;
    double init_res = 0.0, res = 0.0;
    int iter = 0, status = 0;
    const auto conv = [&](double rr) { return rr < tol || (rel > 1e-20 && rr < rel * init_res); };
    do {
        // --- A x, r = b - A x; sums of x and |r|
        double s1[2] = {0.0, 0.0};
        for (long long c = first; c < n; c += stride) {
            const double* xx = a.x;
            const double ax = offdiag<W>(op, a.coef, c, [xx](long long q) { return xx[q]; },
                                         a.diag[c] * xx[c]);
            const double rr = a.b[c] - ax;
            a.ax[c] = ax;
            a.r[c] = rr;
            s1[0] += a.x[c];
            s1[1] += fabs(rr);
        }
        block_sums<kCoopBlock, 2>(ca.partial, set, s1);
        if (!grid_barrier(ca.bar_count, ca.bar_abort, epoch, ca.spin_limit)) { aborted = true; break; }
        double g1[2];
        grid_sums<2>(ca.partial, set, g1);
        set ^= 1;
        const double avg = g1[0] / double(n);
        // --- normFactor; z = D^-1 r (published), z.r
        double s2[2] = {0.0, 0.0};
        for (long long c = first; c < n; c += stride) {
            const double pa = row_sum(op, a.coef, a.diag, c) * avg;
            s2[0] += fabs(a.ax[c] - pa) + fabs(a.b[c] - pa);
            const double rr = a.r[c];
            const double zc = a.rdiag[c] * rr;
            __stcg(&a.z[c], zc);
            s2[1] += zc * rr;
        }
        block_sums<kCoopBlock, 2>(ca.partial, set, s2);
        if (!grid_barrier(ca.bar_count, ca.bar_abort, epoch, ca.spin_limit)) { aborted = true; break; }
        double g2[2];
        grid_sums<2>(ca.partial, set, g2);
        set ^= 1;
        const double normf = g2[0] + 1e-20;
        init_res = g1[1] / normf;
        res = init_res;
        double wArA = g2[1], beta = 0.0;
        double* p_old = a.p;
        double* p_new = ca.p_alt;
        while (!conv(res)) {
            // --- direction pass: p = z + beta p_old, A p, sum p.A p
            const bool first_it = iter == 0;
            double s3[1] = {0.0};
            for (long long c = first; c < n; c += stride) {
                const double pc = direction(a.z, p_old, beta, first_it, c);
                const double* zz = a.z;
                const double* po = p_old;
                const double acc = offdiag<W>(op, a.coef, c, [zz, po, beta, first_it](long long q) {
                    return direction(zz, po, beta, first_it, q);
                }, a.diag[c] * pc);
                __stcg(&p_new[c], pc);
                a.ap[c] = acc;
                s3[0] += acc * pc;
            }
            block_sums<kCoopBlock, 1>(ca.partial, set, s3);
            if (!grid_barrier(ca.bar_count, ca.bar_abort, epoch, ca.spin_limit)) { aborted = true; break; }
            double g3[1];
            grid_sums<1>(ca.partial, set, g3);
            set ^= 1;
            // checkSingularity and alpha, once per block
            double q3[2];
            block_scalars<2>(q3, [&](double* v) {
                v[0] = fabs(g3[0]) / normf < 1e-300 ? 1.0 : 0.0;
                v[1] = wArA / g3[0];
            });
            if (q3[0] != 0.0) break;
            const double alpha = q3[1];
            // --- update pass: x, r, z; |r| and z.r
            double s4[2] = {0.0, 0.0};
            for (long long c = first; c < n; c += stride) {
                a.x[c] = a.x[c] + alpha * __ldcg(&p_new[c]);
                const double rr = a.r[c] - alpha * a.ap[c];
                a.r[c] = rr;
                const double zc = a.rdiag[c] * rr;
                __stcg(&a.z[c], zc);
                s4[0] += fabs(rr);
                s4[1] += zc * rr;
            }
            block_sums<kCoopBlock, 2>(ca.partial, set, s4);
            if (!grid_barrier(ca.bar_count, ca.bar_abort, epoch, ca.spin_limit)) { aborted = true; break; }
            double g4[2];
            grid_sums<2>(ca.partial, set, g4);
            set ^= 1;
            // the residual and beta, once per block
            double q4[2];
            block_scalars<2>(q4, [&](double* v) {
                v[0] = g4[0] / normf;
                v[1] = g4[1] / wArA;
            });
            res = q4[0];
            ++iter;
            if (conv(res) || iter >= max_iter) {
                if (!conv(res)) status = 1;
                break;
            }
            beta = q4[1];
            wArA = g4[1];
            double* t = p_old;
            p_old = p_new;
            p_new = t;
        }
    } while (false);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->iter = iter;
        st->init_res = init_res;
        st->res = res;
        st->status = aborted ? 2 : status;
        st->done = 1;
    }
}

// ---------------------------------------------------------------- float pairs
// The mixed form's solve: the system scaled by 2^shift (a power of two, so
// the solution and the residual ratios are those of the unscaled system),
// its coefficients as (hi, lo) float pairs, the diagonal, source and iterate
// split from their FP64 values at the start, every vector and sum of the
// iteration in pairs on the FP32 pipe, and CG in its single-reduction form
// (Chronopoulos and Gear, 1989): with u = M r and w = A u, the three sums of
// an iteration, (u, r), (w, u) and |r|, are formed in one pass, so an
// iteration has one grid barrier instead of two.  In exact arithmetic the
// iterates are lduMatrix PCG's (same x, r, p and the same convergence test on
// the L1 residual after each update); rounding differs.  A row's new u needs
// the neighbours' new u, which each thread forms itself from the
// neighbours' previous r, s = A p and w (double-buffered) with the same
// operations as their owners, so no halo exchange is needed inside an
// iteration.  The scalars are formed by every thread from the same
// block-order sums.
struct PairPcgArgs {
    const float2* pcoef;   // [slot][cell] scaled coefficients of the system
    int shift;
    float2 *px, *pdiag, *prdiag, *pw;   // [cell]
};

template <int W, class F>
__device__ __forceinline__ fp::P offdiag_pair(const BdOp& op, const float2* pcoef, long long c,
                                             F f, fp::Acc& acc)
{
    if constexpr (W > 0) {
        fp::P v[W], k[W];
#pragma unroll
        for (int e = 0; e < W; ++e) {
            const long long i = (long long)e * op.n + c;
            k[e] = pcoef[i];
            v[e] = f(op.col[i]);
        }
#pragma unroll
        for (int e = 0; e < W; ++e) acc.sub_prod(k[e], v[e]);
    } else {
        const int k = op.cnt[c];
        for (int e = 0; e < k; ++e) {
            const long long i = (long long)e * op.n + c;
            acc.sub_prod(pcoef[i], f(op.col[i]));
        }
    }
    return acc.value();
}

// One row's update of an iteration, from the previous r, s, w of that row:
// s' = w + beta s (A p'), r' = r - alpha s', u' = M r'.  Owners and
// neighbours evaluate it the same way, so both see the same bits.
struct PairStep {
    fp::P alpha, nalpha, beta;
    bool first;
    __device__ __forceinline__ fp::P s_next(fp::P w, fp::P s_old) const
    {
        return first ? w : fp::madd(beta, s_old, w);
    }
    __device__ __forceinline__ fp::P r_next(fp::P r, fp::P s_new) const
    {
        return fp::madd(nalpha, s_new, r);
    }
};

template <int W, int B = kCoopBlock>
__global__ void __launch_bounds__(B, 1) k_pcg_pair(CoopPcgArgs ca, PairPcgArgs q)
{
    using namespace cfg::gsync;
    using fp::P;
    const PcgArgs& a = ca.a;
    const BdOp& op = a.op;
    PcgScalars* st = a.st;
    const long long n = op.n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long first = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const P tol = fp::split(st->tol), rel = fp::split(st->rel);
    const bool use_rel = st->rel > 1e-20;
    const int max_iter = st->max_iter;
    const int sh = q.shift;
    const P small = fp::split(1e-20, sh), count = fp::split(double(n));
    // r, s and w double-buffered: [k] holds the previous iteration's values
    // (read at the neighbours), [k ^ 1] receives this iteration's
    P* r_cur = reinterpret_cast<P*>(a.r);
    P* r_new = reinterpret_cast<P*>(a.ax);
    P* s_cur = reinterpret_cast<P*>(a.ap);
    P* s_new = reinterpret_cast<P*>(ca.p_alt);
    P* w_cur = reinterpret_cast<P*>(a.z);
    P* w_new = q.pw;
    P* p = reinterpret_cast<P*>(a.p);
    P* ax = reinterpret_cast<P*>(a.ax);
    float2* partial = reinterpret_cast<float2*>(ca.partial);
    unsigned epoch = 0;
    int set = 0;
    bool aborted = false, started = false;
    P init_res = fp::make(0.0f), res = fp::make(0.0f);
    int iter = 0, status = 0;
    do {
        // --- A x, r = b - A x; sums of x and |r|
        P s1[2] = {fp::make(0.0f), fp::make(0.0f)};
        const double* xx = a.x;
        for (long long c = first; c < n; c += stride) {
            const P d = fp::split(a.diag[c], sh);
            q.pdiag[c] = d;
            q.prdiag[c] = fp::split(a.rdiag[c], -sh);
            const P xc = fp::split(xx[c]);
            q.px[c] = xc;
            fp::Acc acc;
            acc.add_prod(d, xc);
            const P axc = offdiag_pair<W>(op, q.pcoef, c, [xx](long long k) {
                return fp::split(xx[k]);
            }, acc);
            const P rc = fp::sub(fp::split(a.b[c], sh), axc);
            ax[c] = axc;
            r_cur[c] = rc;
            s1[0] = fp::add(s1[0], xc);
            s1[1] = fp::add(s1[1], fp::abs(rc));
        }
        started = true;
        block_sums_pair<B, 2, 3>(partial, set, s1);
        if (!grid_barrier(ca.bar_count, ca.bar_abort, epoch, ca.spin_limit)) { aborted = true; break; }
        P g1[2];
        grid_sums_pair<2, 3>(partial, set, g1);
        set ^= 1;
        const P avg = fp::div(g1[0], count);
        // --- normFactor; u = M r (published in w[1] until w = A u is formed)
        P s2[2] = {fp::make(0.0f), fp::make(0.0f)};
        for (long long c = first; c < n; c += stride) {
            fp::Acc rs;
            rs.add_prod(q.pdiag[c], fp::make(1.0f));
            const P pa = fp::mul(offdiag_pair<W>(op, q.pcoef, c, [](long long) {
                return fp::make(1.0f);
            }, rs), avg);
            const P bc = fp::split(a.b[c], sh);
            s2[0] = fp::add(s2[0], fp::add(fp::abs(fp::sub(ax[c], pa)), fp::abs(fp::sub(bc, pa))));
            const P rc = r_cur[c];
            const P uc = fp::mul(q.prdiag[c], rc);
            __stcg(&w_new[c], uc);
            s2[1] = fp::madd(uc, rc, s2[1]);
        }
        block_sums_pair<B, 2, 3>(partial, set, s2);
        if (!grid_barrier(ca.bar_count, ca.bar_abort, epoch, ca.spin_limit)) { aborted = true; break; }
        P g2[2];
        grid_sums_pair<2, 3>(partial, set, g2);
        set ^= 1;
        const P normf = fp::add(g2[0], small);
        init_res = fp::div(g1[1], normf);
        const P rel_init = fp::mul(rel, init_res);
        const auto conv = [&](P rr) {
            return fp::less(rr, tol) || (use_rel && fp::less(rr, rel_init));
        };
        res = init_res;
        if (conv(res)) break;
        // --- w = A u; (w, u)
        P s3[1] = {fp::make(0.0f)};
        for (long long c = first; c < n; c += stride) {
            const P* u0 = w_new;
            fp::Acc acc;
            acc.add_prod(q.pdiag[c], __ldcg(&u0[c]));
            const P wc = offdiag_pair<W>(op, q.pcoef, c, [u0](long long k) {
                return __ldcg(&u0[k]);
            }, acc);
            w_cur[c] = wc;
            s3[0] = fp::madd(wc, __ldcg(&u0[c]), s3[0]);
        }
        block_sums_pair<B, 1, 3>(partial, set, s3);
        if (!grid_barrier(ca.bar_count, ca.bar_abort, epoch, ca.spin_limit)) { aborted = true; break; }
        P g3[1];
        grid_sums_pair<1, 3>(partial, set, g3);
        set ^= 1;
        P gamma = g2[1], delta = g3[0], gamma_old = fp::make(0.0f), alpha_old = fp::make(1.0f);
        for (;;) {
            // the scalars of this iteration; (p, A p) = delta - beta gamma / alpha_old
            PairStep ps;
            ps.first = iter == 0;
            ps.beta = ps.first ? fp::make(0.0f) : fp::div(gamma, gamma_old);
            const P pap = ps.first ? delta
                                   : fp::sub(delta, fp::div(fp::mul(ps.beta, gamma), alpha_old));
            if (pap.x == 0.0f) break;   // checkSingularity
            ps.alpha = fp::div(gamma, pap);
            ps.nalpha = fp::neg(ps.alpha);
            const P* r0 = r_cur;
            const P* s0 = s_cur;
            const P* w0 = w_cur;
            P* r1 = r_new;
            P* s1n = s_new;
            P* w1 = w_new;
            // u' of row j from its previous r, s, w
            const auto u_next = [&](long long j) {
                const P sj = ps.s_next(__ldcg(&w0[j]), __ldcg(&s0[j]));
                return fp::mul(__ldcg(&q.prdiag[j]), ps.r_next(__ldcg(&r0[j]), sj));
            };
            P s4[3] = {fp::make(0.0f), fp::make(0.0f), fp::make(0.0f)};
            for (long long c = first; c < n; c += stride) {
                const P rc = __ldcg(&r0[c]);
                const P sc = ps.s_next(__ldcg(&w0[c]), __ldcg(&s0[c]));
                const P uc_old = fp::mul(q.prdiag[c], rc);
                const P pc = ps.first ? uc_old : fp::madd(ps.beta, p[c], uc_old);
                p[c] = pc;
                q.px[c] = fp::madd(ps.alpha, pc, q.px[c]);
                const P rn = ps.r_next(rc, sc);
                const P un = fp::mul(q.prdiag[c], rn);
                fp::Acc acc;
                acc.add_prod(q.pdiag[c], un);
                const P wn = offdiag_pair<W>(op, q.pcoef, c, u_next, acc);
                __stcg(&r1[c], rn);
                __stcg(&s1n[c], sc);
                __stcg(&w1[c], wn);
                s4[0] = fp::madd(un, rn, s4[0]);
                s4[1] = fp::madd(wn, un, s4[1]);
                s4[2] = fp::add(s4[2], fp::abs(rn));
            }
            // the three sums in one set of three slots; sets alternate, so a
            // set is written again only after every block has read it
            block_sums_pair<B, 3, 3>(partial, set, s4);
            if (!grid_barrier(ca.bar_count, ca.bar_abort, epoch, ca.spin_limit)) { aborted = true; break; }
            P g4[3];
            grid_sums_pair<3, 3>(partial, set, g4);
            set ^= 1;
            res = fp::div(g4[2], normf);
            ++iter;
            P* t = r_cur; r_cur = r_new; r_new = t;
            t = s_cur; s_cur = s_new; s_new = t;
            t = w_cur; w_cur = w_new; w_new = t;
            if (conv(res) || iter >= max_iter) {
                if (!conv(res)) status = 1;
                break;
            }
            gamma_old = gamma;
            alpha_old = ps.alpha;
            gamma = g4[0];
            delta = g4[1];
        }
    } while (false);
    // the iterate back into the FP64 field (own rows)
    if (started && !aborted)
        for (long long c = first; c < n; c += stride) a.x[c] = fp::join(q.px[c]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->iter = iter;
        st->init_res = fp::join(init_res);
        st->res = fp::join(res);
        st->status = aborted ? 2 : status;
        st->done = 1;
    }
}

// scaled float-pair copy of a coefficient array
__global__ void k_pair_coef(long long m, const double* coef, int shift, float2* out)
{
    const long long i = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (i < m) out[i] = fp::split(coef[i], shift);
}

__global__ void k_phii(long long n, const double* vm, const double* phie, double* phii)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c < n) phii[c] = vm[c] + phie[c];
}

// MyocardiumDomain::updateActivationTime
__global__ void k_activation(long long n, const double* vm, const double* vm_old, double old_time,
                             double dt, unsigned char* calc, double* act)
{
    const long long c = (long long)blockIdx.x * kBlock + threadIdx.x;
    if (c >= n) return;
    if (calc[c] && vm[c] > 1e-15) {
        calc[c] = 0;
        const double w = (0.0 - vm_old[c]) / (vm[c] - vm_old[c]);
        act[c] = old_time + w * dt;
    }
}

}  // namespace

struct cfg_bidomain {
    cfg_ionic* ion = nullptr;
    cudaStream_t stream = nullptr;
    long long n = 0;
    int blocks = 0;
    BdOp op{};
    // operator storage
    int* d_col = nullptr;
    unsigned char *d_cnt = nullptr, *d_own = nullptr;
    double *d_coef_i = nullptr, *d_coef_e = nullptr, *d_gw = nullptr, *d_sf = nullptr,
           *d_w = nullptr, *d_bw = nullptr, *d_vol = nullptr, *d_centres = nullptr;
    // fields
    double *d_vm = nullptr, *d_vm_old = nullptr, *d_vm_oldold = nullptr, *d_iion = nullptr,
           *d_src = nullptr, *d_act = nullptr, *d_phie = nullptr, *d_phii = nullptr;
    unsigned char* d_calc = nullptr;
    // work
    // explicit Laplacian corrections (non-orthogonal meshes): per slot the
    // signed correction vectors of Gi and of Gi + Ge [3][slot], per cell the
    // wall factors [3][cell]; null where no correction is needed
    double *d_ki = nullptr, *d_ke = nullptr, *d_bki = nullptr, *d_bke = nullptr,
           *d_cv = nullptr;
    double *d_grad = nullptr, *d_dv = nullptr, *d_diag = nullptr, *d_rdiag = nullptr,
           *d_b = nullptr, *d_r = nullptr,
           *d_z = nullptr, *d_p = nullptr, *d_ap = nullptr, *d_ax = nullptr, *d_partial = nullptr;
    PcgScalars* d_st = nullptr;
    PcgScalars* h_st = nullptr;     // pinned
    unsigned* d_ticket = nullptr;
    // the persistent solve: grid (0: not available), second direction buffer,
    // its reduction partials and grid barrier
    int coop_blocks = 0;
    double *d_p_alt = nullptr, *d_coop_partial = nullptr;
    // float-pair PCG of the persistent solve (CFG_PCG_FLOAT_PAIRS, the mixed
    // form's default): per system [0] phiE, [1] Vm the scaled coefficients
    // and their scale, the iterate and the scaled diagonal as pairs; the
    // scale follows from bounds of the largest diagonal
    bool pair = false;
    int pair_block = 512, pair_blocks = 0;   // launch shape of the float-pair solve
    float2* d_pcoef[2] = {nullptr, nullptr};
    int pcoef_shift[2] = {0, 0};
    bool pcoef_ready[2] = {false, false};
    float2 *d_px = nullptr, *d_pdiag = nullptr, *d_prdiag = nullptr, *d_pw = nullptr;
    double max_vol = 0.0, max_row_i = 0.0, max_row_e = 0.0;
    double step_dt = 0.0;
    unsigned* d_bar = nullptr;
    int* d_abort = nullptr;
    long long spin_limit = cfg::gsync::kSpinLimit;
    // kChunk PCG iterations of each system captured as a graph: [0] phiE, [1] Vm
    cudaGraphExec_t chunk[2] = {nullptr, nullptr};
    // settings
    double chicm = 0.0;
    bool backward = true;
    double vm_tol = 1e-8, vm_rel = 0.0, e_tol = 1e-8, e_rel = 0.0;
    int vm_max = 1000, e_max = 1000, n_outer = 1;
    double outer_tol = 0.0;
    bool explicit_alg = false;
    long long ref = -1;
    double ref_value = 0.0;
    StimArgs stim{};
    // state
    double t = 0.0;
    int n_old = 0;
    cfg_step_stats vm_stats{}, e_stats{};
};

using namespace cfg;

namespace {

cudaError_t alloc_pairs(cfg_bidomain* bd)
{
    if (bd->d_px) return cudaSuccess;
    const size_t n = size_t(bd->n), m = size_t(bd->op.width > 0 ? bd->op.width : 1) * n;
    cudaError_t e = dmalloc(&bd->d_pcoef[0], m);
    if (!e) e = dmalloc(&bd->d_pcoef[1], m);
    if (!e) e = dmalloc(&bd->d_px, n);
    if (!e) e = dmalloc(&bd->d_pdiag, n);
    if (!e) e = dmalloc(&bd->d_prdiag, n);
    if (!e) e = dmalloc(&bd->d_pw, n);
    return e;
}

PcgArgs pcg_args(cfg_bidomain* bd, const double* coef, double* x)
{
    PcgArgs a{};
    a.op = bd->op;
    a.coef = coef;
    a.diag = bd->d_diag;
    a.rdiag = bd->d_rdiag;
    a.b = bd->d_b;
    a.x = x;
    a.ax = bd->d_ax;
    a.r = bd->d_r;
    a.z = bd->d_z;
    a.p = bd->d_p;
    a.ap = bd->d_ap;
    a.partial = bd->d_partial;
    a.ticket = bd->d_ticket;
    a.st = bd->d_st;
    return a;
}

// The float-pair solve's kernel for an ELL width and block size
const void* pair_kernel(int width, int block)
{
    if (block == 448)
        return width == 6 ? (const void*)k_pcg_pair<6, 448>
             : width == 4 ? (const void*)k_pcg_pair<4, 448> : (const void*)k_pcg_pair<0, 448>;
    if (block == 384)
        return width == 6 ? (const void*)k_pcg_pair<6, 384>
             : width == 4 ? (const void*)k_pcg_pair<4, 384> : (const void*)k_pcg_pair<0, 384>;
    return width == 6 ? (const void*)k_pcg_pair<6> : width == 4 ? (const void*)k_pcg_pair<4>
                                                                : (const void*)k_pcg_pair<0>;
}

// kind 0: phiE (coef_e, phiE), 1: Vm (coef_i, Vm)
int pcg_solve(cfg_bidomain* bd, int kind, double tol, double rel, int max_iter,
              cfg_step_stats& stats)
{
    cudaStream_t s = bd->stream;
    const int nb = bd->blocks;
    const PcgArgs a = kind == 0 ? pcg_args(bd, bd->op.coef_e, bd->d_phie)
                                : pcg_args(bd, bd->op.coef_i, bd->d_vm);
    if (bd->coop_blocks > 0) {
        PcgScalars init{};
        init.tol = tol;
        init.rel = rel;
        init.max_iter = max_iter;
        *bd->h_st = init;
        CFG_CUDA_TRY(cudaMemcpyAsync(bd->d_st, bd->h_st, sizeof(PcgScalars),
                                     cudaMemcpyHostToDevice, s));
        CFG_CUDA_TRY(cudaMemsetAsync(bd->d_bar, 0, sizeof(unsigned), s));
        CFG_CUDA_TRY(cudaMemsetAsync(bd->d_abort, 0, sizeof(int), s));
        CoopPcgArgs ca{a, bd->d_p_alt, bd->d_coop_partial, bd->d_bar, bd->d_abort,
                       bd->spin_limit};
        if (bd->pair) {
            // the largest diagonal is at most 2 x the largest row sum of the
            // phiE system (setReference doubles one), chi Cm 2 V / dt + the
            // largest row sum of the Vm system
            const double dmax = kind == 0 ? 2.0 * bd->max_row_e
                                          : bd->chicm * 2.0 * bd->max_vol / bd->step_dt +
                                                bd->max_row_i;
            const int shift = dmax > 0 ? -std::ilogb(dmax) : 0;
            if (!bd->pcoef_ready[kind] || bd->pcoef_shift[kind] != shift) {
                const long long m = (long long)bd->op.width * bd->n;
                k_pair_coef<<<unsigned((m + kBlock - 1) / kBlock), kBlock, 0, s>>>(
                    m, kind == 0 ? bd->op.coef_e : bd->op.coef_i, shift, bd->d_pcoef[kind]);
                CFG_CUDA_TRY(cudaGetLastError());
                bd->pcoef_shift[kind] = shift;
                bd->pcoef_ready[kind] = true;
            }
            PairPcgArgs pa{bd->d_pcoef[kind], shift, bd->d_px, bd->d_pdiag, bd->d_prdiag,
                           bd->d_pw};
            void* params[] = {&ca, &pa};
            CFG_CUDA_TRY(cudaLaunchCooperativeKernel(pair_kernel(bd->op.width, bd->pair_block),
                                                     dim3(bd->pair_blocks), dim3(bd->pair_block),
                                                     params, 0, s));
        } else {
            void* params[] = {&ca};
            const void* fn = bd->op.width == 6 ? (const void*)k_pcg_coop<6>
                           : bd->op.width == 4 ? (const void*)k_pcg_coop<4>
                                               : (const void*)k_pcg_coop<0>;
            CFG_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(bd->coop_blocks), dim3(kCoopBlock),
                                                     params, 0, s));
        }
        CFG_CUDA_TRY(cudaMemcpyAsync(bd->h_st, bd->d_st, sizeof(PcgScalars),
                                     cudaMemcpyDeviceToHost, s));
        CFG_CUDA_TRY(cudaStreamSynchronize(s));
        const PcgScalars& st = *bd->h_st;
        const int k = stats.n_solves;
        if (k < kMaxSolves) {
            stats.iterations[k] = st.iter;
            stats.initial_residual[k] = st.init_res;
            stats.final_residual[k] = st.res;
        }
        stats.n_solves = k + 1;
        if (st.status == 2)
            return fail(CFG_ERR_PCG, "bidomain PCG aborted: a grid barrier timed out");
        if (st.status)
            return fail(CFG_ERR_PCG, "bidomain PCG reached maxIter (%d) at residual %g",
                        max_iter, st.res);
        return CFG_OK;
    }
    if (!bd->chunk[kind]) {
        cudaGraph_t g = nullptr;
        CFG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < kChunk; ++k) {
            k_pcg_direction<<<nb, kBlock, 0, s>>>(a);
            k_pcg_update<<<nb, kBlock, 0, s>>>(a);
        }
        CFG_CUDA_TRY(cudaStreamEndCapture(s, &g));
        const cudaError_t e = cudaGraphInstantiate(&bd->chunk[kind], g, 0);
        cudaGraphDestroy(g);
        CFG_CUDA_TRY(e);
    }
    PcgScalars init{};
    init.tol = tol;
    init.rel = rel;
    init.max_iter = max_iter;
    *bd->h_st = init;
    CFG_CUDA_TRY(cudaMemcpyAsync(bd->d_st, bd->h_st, sizeof(PcgScalars), cudaMemcpyHostToDevice, s));
    k_pcg_begin<<<nb, kBlock, 0, s>>>(a);
    k_pcg_norm<<<nb, kBlock, 0, s>>>(a);
    CFG_CUDA_TRY(cudaGetLastError());
    for (int it = 0;; it += kChunk) {
        CFG_CUDA_TRY(cudaMemcpyAsync(bd->h_st, bd->d_st, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
        CFG_CUDA_TRY(cudaStreamSynchronize(s));
        if (bd->h_st->done) break;
        if (it > max_iter + kChunk) return fail(CFG_ERR_PCG, "bidomain PCG did not finish");
        CFG_CUDA_TRY(cudaGraphLaunch(bd->chunk[kind], s));
    }
    const PcgScalars& st = *bd->h_st;
    const int k = stats.n_solves;
    if (k < kMaxSolves) {
        stats.iterations[k] = st.iter;
        stats.initial_residual[k] = st.init_res;
        stats.final_residual[k] = st.res;
    }
    stats.n_solves = k + 1;
    if (st.status) return fail(CFG_ERR_PCG, "bidomain PCG reached maxIter (%d) at residual %g",
                               max_iter, st.res);
    return CFG_OK;
}

// V fvc::div of the explicit correction of laplacian(G, x) into bd->d_cv
// (G: kv/bk of Gi or of Gi + Ge); null where the mesh needs none
const double* correction(cfg_bidomain* bd, const double* kv, const double* bk, const double* x)
{
    if (!kv) return nullptr;
    k_gradient<<<bd->blocks, kBlock, 0, bd->stream>>>(bd->op, x, bd->d_grad);
    k_correction<<<bd->blocks, kBlock, 0, bd->stream>>>(bd->op, kv, bk, bd->d_grad, bd->d_cv);
    return bd->d_cv;
}

void div_gamma_grad(cfg_bidomain* bd, const double* x, double* out)
{
    k_gradient<<<bd->blocks, kBlock, 0, bd->stream>>>(bd->op, x, bd->d_grad);
    k_div_gamma_grad<<<bd->blocks, kBlock, 0, bd->stream>>>(bd->op, bd->d_grad, out);
}

}  // namespace

extern "C" int cfg_bidomain_destroy(cfg_bidomain* bd)
{
    if (!bd) return CFG_OK;
    if (bd->stream) cudaStreamSynchronize(bd->stream);
    for (double** p : {&bd->d_coef_i, &bd->d_coef_e, &bd->d_gw, &bd->d_sf, &bd->d_w, &bd->d_bw,
                       &bd->d_vol, &bd->d_centres, &bd->d_vm, &bd->d_vm_old, &bd->d_vm_oldold,
                       &bd->d_iion, &bd->d_src, &bd->d_act, &bd->d_phie, &bd->d_phii,
                       &bd->d_grad, &bd->d_dv, &bd->d_diag, &bd->d_rdiag, &bd->d_b, &bd->d_r,
                       &bd->d_z,
                       &bd->d_p, &bd->d_ap, &bd->d_ax, &bd->d_partial, &bd->d_p_alt,
                       &bd->d_coop_partial, &bd->d_ki, &bd->d_ke, &bd->d_bki, &bd->d_bke,
                       &bd->d_cv})
        dfree(*p);
    dfree(bd->d_bar);
    dfree(bd->d_abort);
    dfree(bd->d_pcoef[0]);
    dfree(bd->d_pcoef[1]);
    dfree(bd->d_px);
    dfree(bd->d_pdiag);
    dfree(bd->d_prdiag);
    dfree(bd->d_pw);
    dfree(bd->d_col);
    dfree(bd->d_cnt);
    dfree(bd->d_own);
    dfree(bd->d_calc);
    dfree(bd->d_st);
    dfree(bd->d_ticket);
    for (cudaGraphExec_t& g : bd->chunk)
        if (g) cudaGraphExecDestroy(g);
    if (bd->h_st) cudaFreeHost(bd->h_st);
    if (bd->ion) cfg_ionic_destroy(bd->ion);
    if (bd->stream) cudaStreamDestroy(bd->stream);
    delete bd;
    return CFG_OK;
}

extern "C" int cfg_bidomain_create(const cfg_bidomain_desc* d, const cfg_mesh_desc* m,
                                   cfg_bidomain** out)
{
    clear_error();
    if (!d || !m || !out) return fail(CFG_ERR_INVALID, "null argument");
    *out = nullptr;
    const long long n = m->n_cells, nf = m->n_faces;
    if (n <= 0) return fail(CFG_ERR_INVALID, "the mesh has no cells");
    if (d->ionic.n_cells != n)
        return fail(CFG_ERR_INVALID, "ionic n_cells %lld != mesh cells %lld", d->ionic.n_cells, n);
    if (!m->face_centres)
        return fail(CFG_ERR_INVALID, "the bidomain step needs the mesh's full geometry");
    if (d->n_outer < 1) return fail(CFG_ERR_INVALID, "nOuterCorrectors must be at least 1");
    if (d->n_boxes < 0 || d->n_boxes > 8) return fail(CFG_ERR_INVALID, "0 to 8 stimulus boxes");
    for (long long f = 0; f < nf; ++f) {
        const int l = m->owner[f], u = m->neighbour[f];
        if (l < 0 || u < 0 || l >= n || u >= n || l == u)
            return fail(CFG_ERR_INVALID, "face %lld has invalid owner/neighbour %d/%d", f, l, u);
    }
    double ge[6];
    for (int k = 0; k < 6; ++k) ge[k] = d->conductivity_i[k] + d->conductivity_e[k];
    CorrectedOperator oi, oe;
    if (int rc = assemble_corrected(m, d->conductivity_i, nullptr, d->grad_scheme, 0, oi)) return rc;
    if (int rc = assemble_corrected(m, ge, nullptr, d->grad_scheme, 0, oe)) return rc;
    double gmax = 0.0;
    for (int k = 0; k < 6; ++k) gmax = std::max(gmax, std::fabs(ge[k]));
    if (!(gmax > 0.0))
        return fail(CFG_ERR_INVALID, "the bulk conductivity Gi + Ge is zero (phiE is undefined)");
    // the explicit correction is needed where a face is non-orthogonal or a
    // conductivity is not aligned with it (k per face), or at a wall (bk)
    bool corrected = false;
    for (long long f = 0; f < nf && !corrected; ++f) {
        const double* S = m->face_sf + 3 * f;
        const double scale = gmax * std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
        for (const CorrectedOperator* o : {&oi, &oe})
            for (int k = 0; k < 3; ++k)
                if (std::fabs(o->k[size_t(3 * f + k)]) > 1e-12 * scale) corrected = true;
    }
    for (long long c = 0; c < n && !corrected; ++c)
        for (const CorrectedOperator* o : {&oi, &oe})
            for (int k = 0; k < 3; ++k)
                if (std::fabs(o->bk[size_t(3 * c + k)]) > 1e-12 * gmax * std::cbrt(m->volumes[c]) *
                                                               std::cbrt(m->volumes[c]))
                    corrected = true;
    // ELL rows: (column, face, own) sorted by column
    struct Entry {
        int col;
        long long face;
        bool own;
    };
    std::vector<std::vector<Entry>> rows(static_cast<size_t>(n));
    for (long long f = 0; f < nf; ++f) {
        rows[size_t(m->owner[f])].push_back({m->neighbour[f], f, true});
        rows[size_t(m->neighbour[f])].push_back({m->owner[f], f, false});
    }
    int width = 0;
    for (auto& r : rows) {
        std::stable_sort(r.begin(), r.end(), [](const Entry& a, const Entry& b) { return a.col < b.col; });
        width = std::max(width, int(r.size()));
    }
    if (width > 255) return fail(CFG_ERR_INVALID, "cell with more than 255 faces");
    width = std::max(width, 1);
    const size_t slots = size_t(width) * size_t(n);
    std::vector<int> col(slots, 0);
    std::vector<unsigned char> cnt(static_cast<size_t>(n)), own(slots, 0);
    std::vector<double> ci(slots, 0.0), ce(slots, 0.0), gw(3 * slots, 0.0), sf(3 * slots, 0.0),
        wv(slots, 0.0), bw(3 * size_t(n), 0.0);
    std::vector<double> kiv(corrected ? 3 * slots : 0, 0.0), kev(corrected ? 3 * slots : 0, 0.0),
        bki(corrected ? 3 * size_t(n) : 0, 0.0), bke(corrected ? 3 * size_t(n) : 0, 0.0);
    if (corrected)
        for (long long c = 0; c < n; ++c)
            for (int k = 0; k < 3; ++k) {
                bki[size_t(k) * size_t(n) + size_t(c)] = oi.bk[size_t(3 * c + k)];
                bke[size_t(k) * size_t(n) + size_t(c)] = oe.bk[size_t(3 * c + k)];
            }
    for (long long c = 0; c < n; ++c) {
        const auto& r = rows[size_t(c)];
        cnt[size_t(c)] = (unsigned char)r.size();
        for (size_t q = 0; q < r.size(); ++q) {
            const size_t i = q * size_t(n) + size_t(c);
            const long long f = r[q].face;
            col[i] = r[q].col;
            own[i] = r[q].own ? 1 : 0;
            ci[i] = oi.coeff[size_t(f)];
            ce[i] = oe.coeff[size_t(f)];
            wv[i] = oi.w[size_t(f)];
            const double* g = r[q].own ? oi.g_own.data() : oi.g_nei.data();
            const double sg = r[q].own ? 1.0 : -1.0;
            for (int k = 0; k < 3; ++k) {
                gw[size_t(k) * slots + i] = g[3 * f + k];
                sf[size_t(k) * slots + i] = m->face_sf[3 * f + k];
                if (corrected) {
                    kiv[size_t(k) * slots + i] = sg * oi.k[size_t(3 * f + k)];
                    kev[size_t(k) * slots + i] = sg * oe.k[size_t(3 * f + k)];
                }
            }
        }
    }
    // wall factor of the divergence: sum over the cell's wall faces of
    // Gi Sf - ((Gi Sf).n) n, so that Sf . Gi (g - n (n.g)) = bw . g
    const double* G = d->conductivity_i;
    for (long long b = 0; b < m->n_boundary_faces; ++b) {
        const double* S = m->boundary_sf + 3 * b;
        const double mag = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
        const double nn[3] = {S[0] / mag, S[1] / mag, S[2] / mag};
        const double gs[3] = {G[0] * S[0] + G[1] * S[1] + G[2] * S[2],
                              G[1] * S[0] + G[3] * S[1] + G[4] * S[2],
                              G[2] * S[0] + G[4] * S[1] + G[5] * S[2]};
        const double gn = gs[0] * nn[0] + gs[1] * nn[1] + gs[2] * nn[2];
        const long long c = m->boundary_cell[b];
        for (int k = 0; k < 3; ++k) bw[size_t(k) * size_t(n) + size_t(c)] += gs[k] - gn * nn[k];
    }
    // the reference cell: nearest centre, the first in cell order on ties
    long long ref = 0;
    double best = -1.0;
    for (long long c = 0; c < n; ++c) {
        const double* C = m->centres + 3 * c;
        const double dd = (C[0] - d->ref_point[0]) * (C[0] - d->ref_point[0]) +
                          (C[1] - d->ref_point[1]) * (C[1] - d->ref_point[1]) +
                          (C[2] - d->ref_point[2]) * (C[2] - d->ref_point[2]);
        if (best < 0.0 || dd < best) { best = dd; ref = c; }
    }

    auto* bd = new cfg_bidomain();
    auto bail = [&](int rc) {
        cfg_bidomain_destroy(bd);
        return rc;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&bd->stream, cudaStreamNonBlocking);
    if (e) return bail(fail(CFG_ERR_CUDA, "stream: %s", cudaGetErrorString(e)));
    if (int rc = ionic_create(&d->ionic, bd->stream, &bd->ion)) return bail(rc);
    bd->n = n;
    bd->blocks = int((n + kBlock - 1) / kBlock);
    bd->chicm = d->chi * d->cm;
    bd->backward = d->ddt_backward != 0;
    bd->vm_tol = d->pcg_tol; bd->vm_rel = d->pcg_rel_tol; bd->vm_max = d->pcg_max_iter;
    bd->e_tol = d->phie_tol; bd->e_rel = d->phie_rel_tol; bd->e_max = d->phie_max_iter;
    bd->n_outer = d->n_outer;
    bd->outer_tol = d->outer_tol;
    bd->explicit_alg = d->explicit_algorithm != 0;
    bd->ref = ref;
    bd->ref_value = d->ref_value;
    bd->stim.n_boxes = d->n_boxes;
    for (int b = 0; b < d->n_boxes; ++b) {
        for (int k = 0; k < 3; ++k) {
            bd->stim.lo[b][k] = d->box_min[b][k];
            bd->stim.hi[b][k] = d->box_max[b][k];
        }
        bd->stim.start[b] = d->box_start[b];
        bd->stim.dur[b] = d->box_duration[b];
        bd->stim.amp[b] = d->box_intensity[b];
    }
    auto up = [&](auto** dst, const auto& v) -> cudaError_t {
        cudaError_t err = dmalloc(dst, v.size());
        if (!err) err = cudaMemcpy(*dst, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice);
        return err;
    };
    std::vector<double> vol(m->volumes, m->volumes + n), cen(m->centres, m->centres + 3 * n);
    for (long long c = 0; c < n; ++c) {
        double si = 0.0, se = 0.0;
        for (int q = 0; q < width; ++q) {
            si += std::fabs(ci[size_t(q) * size_t(n) + size_t(c)]);
            se += std::fabs(ce[size_t(q) * size_t(n) + size_t(c)]);
        }
        bd->max_row_i = std::max(bd->max_row_i, si);
        bd->max_row_e = std::max(bd->max_row_e, se);
        bd->max_vol = std::max(bd->max_vol, vol[size_t(c)]);
    }
    if (!e) e = up(&bd->d_col, col);
    if (!e) e = up(&bd->d_cnt, cnt);
    if (!e) e = up(&bd->d_own, own);
    if (!e) e = up(&bd->d_coef_i, ci);
    if (!e) e = up(&bd->d_coef_e, ce);
    if (!e) e = up(&bd->d_gw, gw);
    if (!e) e = up(&bd->d_sf, sf);
    if (!e) e = up(&bd->d_w, wv);
    if (!e) e = up(&bd->d_bw, bw);
    if (!e) e = up(&bd->d_vol, vol);
    if (!e) e = up(&bd->d_centres, cen);
    if (!e && corrected) e = up(&bd->d_ki, kiv);
    if (!e && corrected) e = up(&bd->d_ke, kev);
    if (!e && corrected) e = up(&bd->d_bki, bki);
    if (!e && corrected) e = up(&bd->d_bke, bke);
    if (!e && corrected) e = dmalloc(&bd->d_cv, size_t(n));
    for (double** p : {&bd->d_vm, &bd->d_vm_old, &bd->d_vm_oldold, &bd->d_iion, &bd->d_src,
                       &bd->d_act, &bd->d_phie, &bd->d_phii, &bd->d_dv, &bd->d_diag,
                       &bd->d_rdiag, &bd->d_b,
                       &bd->d_r, &bd->d_z, &bd->d_p, &bd->d_ap, &bd->d_ax})
        if (!e) e = dmalloc(p, size_t(n));
    if (!e) e = dmalloc(&bd->d_grad, 3 * size_t(n));
    if (!e) e = dmalloc(&bd->d_partial, 2 * size_t(bd->blocks));
    if (!e) e = dmalloc(&bd->d_calc, size_t(n));
    if (!e) e = dmalloc(&bd->d_st, 1);
    if (!e) e = dmalloc(&bd->d_ticket, 1);
    if (!e) e = cudaMemset(bd->d_ticket, 0, sizeof(unsigned));
    if (!e) e = cudaMallocHost(reinterpret_cast<void**>(&bd->h_st), sizeof(PcgScalars));
    // the persistent solve: one block of kCoopBlock per resident slot, at most
    // one row per thread
    {
        int dev = 0, coop = 0, sms = 0, per_sm = 0;
        if (!e && cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess &&
            coop &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_coop<0>, kCoopBlock, 0) ==
                cudaSuccess &&
            per_sm > 0) {
            for (const void* f : {(const void*)k_pcg_coop<4>, (const void*)k_pcg_coop<6>,
                                  (const void*)k_pcg_pair<0>, (const void*)k_pcg_pair<4>,
                                  (const void*)k_pcg_pair<6>}) {
                int k = 0;
                if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, f, kCoopBlock, 0) ==
                    cudaSuccess)
                    per_sm = std::min(per_sm, k);
            }
            const long long want = (n + kCoopBlock - 1) / kCoopBlock;
            const long long cap = (long long)sms * per_sm;
            bd->coop_blocks = int(want < cap ? want : cap);
            // the float-pair solve: the smallest block of 384, 448 or 512
            // threads whose grid, one row per thread, fits one block per SM,
            // so that every SM takes part in a small system
            bd->pair_block = 512;
            bd->pair_blocks = bd->coop_blocks;
            for (int b : {384, 448}) {
                const long long nb = (n + b - 1) / b;
                int k = 0;
                if (nb <= sms &&
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                        &k, pair_kernel(width, b), b, 0) == cudaSuccess && k >= 1) {
                    bd->pair_block = b;
                    bd->pair_blocks = int(nb);
                    break;
                }
            }
        }
        cudaGetLastError();
    }
    if (!e && bd->coop_blocks > 0) {
        e = dmalloc(&bd->d_p_alt, size_t(n));
        if (!e) e = cudaMemset(bd->d_p_alt, 0, size_t(n) * sizeof(double));
        // two sets of up to three sums per block
        if (!e) e = dmalloc(&bd->d_coop_partial,
                            6 * size_t(std::max(bd->coop_blocks, bd->pair_blocks)));
        if (!e) e = dmalloc(&bd->d_bar, 1);
        if (!e) e = dmalloc(&bd->d_abort, 1);
    }
    if (e) return bail(fail(CFG_ERR_CUDA, "bidomain allocation: %s", cudaGetErrorString(e)));
    std::vector<double> v0(size_t(n), d->vm0), zero(size_t(n), 0.0);
    e = cudaMemcpy(bd->d_vm, v0.data(), size_t(n) * sizeof(double), cudaMemcpyHostToDevice);
    for (double* p : {bd->d_iion, bd->d_src, bd->d_act, bd->d_phie, bd->d_phii, bd->d_p, bd->d_ap})
        if (!e) e = cudaMemcpy(p, zero.data(), size_t(n) * sizeof(double), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemset(bd->d_calc, 1, size_t(n));
    if (e) return bail(fail(CFG_ERR_CUDA, "bidomain initialisation: %s", cudaGetErrorString(e)));
    BdOp& op = bd->op;
    op.n = n;
    op.width = width;
    op.col = bd->d_col;
    op.cnt = bd->d_cnt;
    op.coef_i = bd->d_coef_i;
    op.coef_e = bd->d_coef_e;
    op.gw = bd->d_gw;
    op.sf = bd->d_sf;
    op.w = bd->d_w;
    op.own = bd->d_own;
    op.bw = bd->d_bw;
    op.vol = bd->d_vol;
    for (int k = 0; k < 6; ++k) op.G[k] = d->conductivity_i[k];
    if (bd->coop_blocks > 0 && d->ionic.precision == CFG_PRECISION_MIXED) {
        if ((e = alloc_pairs(bd)))
            return bail(fail(CFG_ERR_CUDA, "bidomain allocation: %s", cudaGetErrorString(e)));
        bd->pair = true;
    }
    *out = bd;
    return CFG_OK;
}

extern "C" int cfg_bidomain_set_pcg_arithmetic(cfg_bidomain* bd, int arithmetic)
{
    if (!bd) return fail(CFG_ERR_INVALID, "null context");
    if (arithmetic != CFG_PCG_FP64 && arithmetic != CFG_PCG_FLOAT_PAIRS)
        return fail(CFG_ERR_INVALID, "unknown PCG arithmetic %d", arithmetic);
    if (arithmetic == CFG_PCG_FP64) {
        bd->pair = false;
        return CFG_OK;
    }
    if (bd->coop_blocks <= 0)
        return fail(CFG_ERR_UNSUPPORTED, "float pairs need the cooperative solve");
    const cudaError_t e = alloc_pairs(bd);
    if (e) return fail(CFG_ERR_CUDA, "device allocation failed: %s", cudaGetErrorString(e));
    bd->pair = true;
    return CFG_OK;
}

extern "C" int cfg_bidomain_step(cfg_bidomain* bd, double dt)
{
    if (!bd) return fail(CFG_ERR_INVALID, "null context");
    if (!(dt > 0)) return fail(CFG_ERR_INVALID, "deltaT must be positive");
    cudaStream_t s = bd->stream;
    const long long n = bd->n;
    const size_t bytes = size_t(n) * sizeof(double);
    const int nb = bd->blocks;
    bd->step_dt = dt;
    // Time::operator++ and the old-time levels of Vm
    bd->t = bd->t + dt;
    if (bd->n_old >= 1) {
        if (bd->n_old >= 2)
            CFG_CUDA_TRY(cudaMemcpyAsync(bd->d_vm_oldold, bd->d_vm_old, bytes, cudaMemcpyDeviceToDevice, s));
        CFG_CUDA_TRY(cudaMemcpyAsync(bd->d_vm_old, bd->d_vm, bytes, cudaMemcpyDeviceToDevice, s));
    }
    const double t0 = bd->t - dt;
    k_stimulus<<<nb, kBlock, 0, s>>>(n, bd->d_centres, bd->stim, t0, bd->d_src);
    if (int rc = cfg_ionic_solve_device(bd->ion, t0, dt, bd->d_vm, bd->d_iion)) return rc;
    bd->vm_stats = cfg_step_stats{};
    bd->e_stats = cfg_step_stats{};
    if (bd->explicit_alg) {
        // BidomainSolver::solveDiffusionExplicit (bidomainSolver.C:183-213)
        const double* cve = correction(bd, bd->d_ke, bd->d_bke, bd->d_phie);
        div_gamma_grad(bd, bd->d_vm, bd->d_dv);
        k_phie_system<<<nb, kBlock, 0, s>>>(bd->op, bd->d_dv, cve, bd->ref, bd->ref_value,
                                            bd->d_diag, bd->d_rdiag, bd->d_b);
        if (int rc = pcg_solve(bd, 0, bd->e_tol, bd->e_rel, bd->e_max, bd->e_stats))
            return rc;
        double cft = 1.0, cft0 = 1.0, cft00 = 0.0;
        if (bd->backward) {
            const double dt0 = bd->n_old < 2 ? 1e15 : dt;
            cft = 1 + dt / (dt + dt0);
            cft00 = dt * dt / (dt0 * (dt + dt0));
            cft0 = cft + cft00;
        }
        if (bd->n_old < 1) {
            CFG_CUDA_TRY(cudaMemcpyAsync(bd->d_vm_old, bd->d_vm, bytes, cudaMemcpyDeviceToDevice, s));
            bd->n_old = 1;
        }
        if (bd->backward && bd->n_old < 2) {
            CFG_CUDA_TRY(cudaMemcpyAsync(bd->d_vm_oldold, bd->d_vm_old, bytes, cudaMemcpyDeviceToDevice, s));
            bd->n_old = 2;
        }
        // fvc::div(Gi & fvc::grad(Vm + phiE)) of the fields before the update
        k_add<<<nb, kBlock, 0, s>>>(n, bd->d_vm, bd->d_phie, bd->d_phii);
        div_gamma_grad(bd, bd->d_phii, bd->d_dv);
        VmArgs va{bd->chicm, 1.0 / dt, cft, cft0, cft00, bd->backward ? 1 : 0};
        k_vm_explicit<<<nb, kBlock, 0, s>>>(bd->op, va, bd->d_vm_old, bd->d_vm_oldold, bd->d_iion,
                                            bd->d_src, bd->d_dv, bd->d_vm);
        k_phii<<<nb, kBlock, 0, s>>>(n, bd->d_vm, bd->d_phie, bd->d_phii);
        k_activation<<<nb, kBlock, 0, s>>>(n, bd->d_vm, bd->d_vm_old, bd->t - dt, dt, bd->d_calc,
                                           bd->d_act);
        CFG_CUDA_TRY(cudaGetLastError());
        if (int rc = ionic_check_status(bd->ion)) return rc;
        return CFG_OK;
    }
    bool converged = false;
    for (int corr = 1; corr <= bd->n_outer && !converged; ++corr) {
        if (corr > 1 && bd->vm_stats.n_solves > 0 &&
            bd->vm_stats.initial_residual[std::min(bd->vm_stats.n_solves, kMaxSolves) - 1] <
                bd->outer_tol)
            converged = true;
        // phiE
        const double* cve = correction(bd, bd->d_ke, bd->d_bke, bd->d_phie);
        div_gamma_grad(bd, bd->d_vm, bd->d_dv);
        k_phie_system<<<nb, kBlock, 0, s>>>(bd->op, bd->d_dv, cve, bd->ref, bd->ref_value,
                                            bd->d_diag, bd->d_rdiag, bd->d_b);
        if (int rc = pcg_solve(bd, 0, bd->e_tol, bd->e_rel, bd->e_max, bd->e_stats))
            return rc;
        // Vm: fvm::ddt creates the old-time levels on first access
        double cft = 1.0, cft0 = 1.0, cft00 = 0.0;
        if (bd->backward) {
            const double dt0 = bd->n_old < 2 ? 1e15 : dt;
            cft = 1 + dt / (dt + dt0);
            cft00 = dt * dt / (dt0 * (dt + dt0));
            cft0 = cft + cft00;
        }
        if (bd->n_old < 1) {
            CFG_CUDA_TRY(cudaMemcpyAsync(bd->d_vm_old, bd->d_vm, bytes, cudaMemcpyDeviceToDevice, s));
            bd->n_old = 1;
        }
        if (bd->backward && bd->n_old < 2) {
            CFG_CUDA_TRY(cudaMemcpyAsync(bd->d_vm_oldold, bd->d_vm_old, bytes, cudaMemcpyDeviceToDevice, s));
            bd->n_old = 2;
        }
        div_gamma_grad(bd, bd->d_phie, bd->d_dv);
        VmArgs va{bd->chicm, 1.0 / dt, cft, cft0, cft00, bd->backward ? 1 : 0};
        // the correction of laplacian(Gi, Vm) at the current Vm; its gradient
        // work array is free again once the divergence above is formed
        const double* cvi = correction(bd, bd->d_ki, bd->d_bki, bd->d_vm);
        k_vm_system<<<nb, kBlock, 0, s>>>(bd->op, va, bd->d_vm_old, bd->d_vm_oldold, bd->d_iion,
                                          bd->d_src, bd->d_dv, cvi, bd->d_diag, bd->d_rdiag,
                                          bd->d_b);
        if (int rc = pcg_solve(bd, 1, bd->vm_tol, bd->vm_rel, bd->vm_max, bd->vm_stats))
            return rc;
        k_phii<<<nb, kBlock, 0, s>>>(n, bd->d_vm, bd->d_phie, bd->d_phii);
    }
    if (bd->n_old < 1) {
        CFG_CUDA_TRY(cudaMemcpyAsync(bd->d_vm_old, bd->d_vm, bytes, cudaMemcpyDeviceToDevice, s));
        bd->n_old = 1;
    }
    k_activation<<<nb, kBlock, 0, s>>>(n, bd->d_vm, bd->d_vm_old, bd->t - dt, dt, bd->d_calc,
                                       bd->d_act);
    CFG_CUDA_TRY(cudaGetLastError());
    if (int rc = ionic_check_status(bd->ion)) return rc;
    return CFG_OK;
}

extern "C" int cfg_bidomain_run(cfg_bidomain* bd, double dt, long long n_steps)
{
    for (long long i = 0; i < n_steps; ++i)
        if (int rc = cfg_bidomain_step(bd, dt)) return rc;
    return CFG_OK;
}

static double* bidomain_field(cfg_bidomain* bd, int field)
{
    switch (field) {
    case CFG_FIELD_VM: return bd->d_vm;
    case CFG_FIELD_IION: return bd->d_iion;
    case CFG_FIELD_ACTIVATION: return bd->d_act;
    case CFG_FIELD_SOURCE: return bd->d_src;
    case CFG_FIELD_VM_OLD: return bd->d_vm_old;
    case CFG_FIELD_PHIE: return bd->d_phie;
    case CFG_FIELD_PHII: return bd->d_phii;
    default: return nullptr;
    }
}

extern "C" int cfg_bidomain_get_field(cfg_bidomain* bd, int field, double* host)
{
    if (!bd || !host) return fail(CFG_ERR_INVALID, "null argument");
    double* p = bidomain_field(bd, field);
    if (!p) return fail(CFG_ERR_INVALID, "unknown field %d", field);
    CFG_CUDA_TRY(cudaMemcpyAsync(host, p, size_t(bd->n) * sizeof(double), cudaMemcpyDeviceToHost,
                                 bd->stream));
    CFG_CUDA_TRY(cudaStreamSynchronize(bd->stream));
    return CFG_OK;
}

extern "C" int cfg_bidomain_set_field(cfg_bidomain* bd, int field, const double* host)
{
    if (!bd || !host) return fail(CFG_ERR_INVALID, "null argument");
    double* p = bidomain_field(bd, field);
    if (!p) return fail(CFG_ERR_INVALID, "unknown field %d", field);
    CFG_CUDA_TRY(cudaMemcpyAsync(p, host, size_t(bd->n) * sizeof(double), cudaMemcpyHostToDevice,
                                 bd->stream));
    CFG_CUDA_TRY(cudaStreamSynchronize(bd->stream));
    return CFG_OK;
}

extern "C" const double* cfg_bidomain_device_field(cfg_bidomain* bd, int field)
{
    return bd ? bidomain_field(bd, field) : nullptr;
}

extern "C" int cfg_bidomain_last_stats(const cfg_bidomain* bd, cfg_step_stats* vm,
                                       cfg_step_stats* phie)
{
    if (!bd) return fail(CFG_ERR_INVALID, "null context");
    if (vm) *vm = bd->vm_stats;
    if (phie) *phie = bd->e_stats;
    return CFG_OK;
}

extern "C" double cfg_bidomain_time(const cfg_bidomain* bd) { return bd ? bd->t : 0.0; }
extern "C" long long cfg_bidomain_reference_cell(const cfg_bidomain* bd) { return bd ? bd->ref : -1; }
extern "C" cfg_ionic* cfg_bidomain_ionic(cfg_bidomain* bd) { return bd ? bd->ion : nullptr; }
extern "C" void* cfg_bidomain_stream(cfg_bidomain* bd) { return bd ? bd->stream : nullptr; }
