// Kernels of the diffusion half of the monodomain step (see
// diffusion_kernels.cuh for the formulation and the reduction scheme).
// Each thread owns one row; the ddt coefficients, the diagonal and its
// reciprocal are precomputed per dt, so the per-step kernels carry no FP64
// division (GB300's FP64 pipe, not HBM, would otherwise bound them).
#include "diffusion_kernels.cuh"

namespace cfg {

// runTime++ and the first access of Vm in the new time step: shift the stored
// old-time levels (GeometricField::storeOldTimes) and reset the PIMPLE state.
__global__ void k_step_begin(DiffusionArgs a)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int n_old = a.st->n_old;
    if (c < a.n) {
        if (n_old >= 2) a.vm_oldold[c] = a.vm_old[c];
        if (n_old >= 1) a.vm_old[c] = a.vm[c];
    }
    if (c == 0) {
        PcgState* st = a.st;
        st->t = st->t + a.dt;
        st->t0 = st->t - a.dt;
        st->corr = 1;
        st->outer_active = 1;
        st->converged_outer = 0;
        st->solve_active = 0;
        st->n_solves = 0;
        st->iter = 0;
        st->step_iters = 0;
        st->bar_count = 0;
        st->bar_abort = 0;
    }
}

// Diagonal (chi*Cm*coefft*V/dt + sum of face coefficients), its reciprocal
// and the row sums of both ddt coefficient sets; recomputed when dt changes.
__global__ void k_prepare(DiffusionArgs a)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n) return;
    const double V = a.vol[c];
    for (int v = 0; v < 2; ++v) {
        const double ddt_diag = a.ddt_backward ? (a.cft[v] * a.rdt) * V : a.rdt * V;
        const double d = a.chicm * ddt_diag - a.lapdiag[c];
        a.diag2[v * a.n + c] = d;
        a.rdiag2[v * a.n + c] = 1.0 / d;
        a.sumA2[v * a.n + c] = row_sum(a, c, d);
        if (a.pair) {
            a.pdiag2[v * a.n + c] = fp::split(d, a.pair_shift);
            a.prdiag2[v * a.n + c] = fp::split(1.0 / d, -a.pair_shift);
            a.psumA2[v * a.n + c] = fp::split(a.sumA2[v * a.n + c], a.pair_shift);
        }
    }
    if (a.pair && !a.sx)
        for (int e = 0; e < a.width; ++e) {
            const long long i = (long long)e * a.n + c;
            a.pcoef[i] = fp::split(a.ell_coef[i], a.pair_shift);
        }
}

// Start of one PIMPLE corrector: the source of
//   chi*Cm*ddt(Vm) - laplacian(sigma,Vm) = -chi*Cm*Iion + src
// (backward/Euler fvmDdt, fvMatrix sources, box stimulus), the residual
// r = b - A.x and the sums for lduMatrix::solver::normFactor.
__global__ void __launch_bounds__(kDiffBlock) k_solve_begin(DiffusionArgs a)
{
    PcgState* st = a.st;
    if (!st->outer_active) return;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int v = ddt_variant(a, st->n_old);
    double vals[2] = {0.0, 0.0};
    if (c < a.n) {
        const double V = a.vol[c];
        double ddt_src;
        if (a.ddt_backward)
            ddt_src = a.rdt * V * (a.cft0[v] * a.vm_old[c] - a.cft00[v] * a.vm_oldold[c]);
        else
            ddt_src = a.rdt * a.vm_old[c] * V;
        const double d = a.diag2[v * a.n + c];
        double bb = a.chicm * ddt_src;
        double su = -(a.chicm * a.iion[c]) * V;
        su = su + box_source(a, c, st->t0) * V;
        bb = bb + su;
        if (a.nc_gw) bb = bb + nc_correction_plain(a, c);
        const double* x = a.vm;
        const double ax = row_amul(a, c, d, [x](long long q) { return x[q]; });
        const double r = bb - ax;
        a.b[c] = bb;
        a.ax[c] = ax;
        a.r[c] = r;
        vals[0] = x[c];
        vals[1] = fabs(r);
    }
    block_partials<2>(a, vals);
    if (last_block(a, 0)) {
        const double sx = sum_partials(a, 0);
        const double sr = sum_partials(a, 1);
        if (threadIdx.x == 0) {
            st->sum_x = sx;
            st->avg = sx / double(a.n);
            st->sum_absr = sr;
            st->variant = v;
            // fvm::ddt created Vm.oldTime() (and its old time for backward)
            if (st->n_old < 1) st->n_old = 1;
            if (a.ddt_backward && st->n_old < 2) st->n_old = 2;
        }
    }
}

// Cell gradient of Vm on a general mesh, for the explicit correction of the
// Laplacian: of the current iterate at the start of each PIMPLE corrector
// (k_grad_iterate), or of the start-of-step Vm, which vm_old holds, before
// the explicit form (k_grad_start).
__device__ __forceinline__ void grad_row(const DiffusionArgs& a, const double* x)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n) return;
    nc_gradient_plain(a, c, x);
}

__global__ void __launch_bounds__(kDiffBlock) k_grad_iterate(DiffusionArgs a)
{
    if (!a.st->outer_active) return;
    grad_row(a, a.vm);
}

__global__ void __launch_bounds__(kDiffBlock) k_grad_start(DiffusionArgs a) { grad_row(a, a.vm_old); }

// normFactor, the initial residual, and the preconditioned residual of
// iteration 0 (z = D^-1 r, z.r).
__global__ void __launch_bounds__(kDiffBlock) k_solve_norm(DiffusionArgs a)
{
    PcgState* st = a.st;
    if (!st->outer_active) return;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int v = st->variant;
    double vals[2] = {0.0, 0.0};
    if (c < a.n) {
        const double pa = a.sumA2[v * a.n + c] * st->avg;
        vals[0] = fabs(a.ax[c] - pa) + fabs(a.b[c] - pa);
        const double z = a.rdiag2[v * a.n + c] * a.r[c];
        a.z[c] = z;
        vals[1] = z * a.r[c];
    }
    block_partials<2>(a, vals);
    if (last_block(a, 1)) {
        const double nf = sum_partials(a, 0);
        const double zr = sum_partials(a, 1);
        if (threadIdx.x == 0) {
            st->normf = nf + 1e-20;
            st->init_res = st->sum_absr / st->normf;
            st->res = st->init_res;
            st->iter = 0;
            st->wArA = zr;
            if (pcg_converged(st, st->res)) {
                end_solve(st);
            } else {
                st->solve_active = 1;
            }
            set_inner(a, st->solve_active);
        }
    }
}

// p = z + beta*p_old (p = z on iteration 0), Ap = A.p and p.Ap.  The
// neighbours' p values are formed on the fly from z and p_old, so the new
// direction needs no separate pass; p_new goes to the other buffer.
__global__ void __launch_bounds__(kDiffBlock) k_pcg_p(DiffusionArgs a)
{
    PcgState* st = a.st;
    if (!st->solve_active) return;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int it = st->iter;
    const double beta = st->beta;
    const double* pold = (it & 1) ? a.pA : a.pB;
    double* pnew = (it & 1) ? a.pB : a.pA;
    const double* z = a.z;
    double vals[1] = {0.0};
    if (c < a.n) {
        auto p = [=](long long q) { return it == 0 ? z[q] : z[q] + beta * pold[q]; };
        const double pc = p(c);
        const double ap = row_amul(a, c, a.diag2[st->variant * a.n + c], p);
        pnew[c] = pc;
        a.ap[c] = ap;
        vals[0] = ap * pc;
    }
    block_partials<1>(a, vals);
    if (last_block(a, 2)) {
        const double wApA = sum_partials(a, 0);
        if (threadIdx.x == 0) {
            st->wApA = wApA;
            if (fabs(wApA) / st->normf < 1e-300) {   // checkSingularity
                end_solve(st);
            } else {
                st->alpha = st->wArA / wApA;
            }
        }
    }
}

// x += alpha p, r -= alpha Ap, |r|, and the next z = D^-1 r with z.r.
__global__ void __launch_bounds__(kDiffBlock) k_pcg_update(DiffusionArgs a)
{
    PcgState* st = a.st;
    if (!st->solve_active) {   // ended in k_pcg_p (singular)
        if (blockIdx.x == 0 && threadIdx.x == 0) set_inner(a, 0);
        return;
    }
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int it = st->iter;
    const double alpha = st->alpha;
    const double* p = (it & 1) ? a.pB : a.pA;
    double vals[2] = {0.0, 0.0};
    if (c < a.n) {
        a.vm[c] += alpha * p[c];
        const double r = a.r[c] - alpha * a.ap[c];
        a.r[c] = r;
        const double z = a.rdiag2[st->variant * a.n + c] * r;
        a.z[c] = z;
        vals[0] = fabs(r);
        vals[1] = z * r;
    }
    block_partials<2>(a, vals);
    if (last_block(a, 3)) {
        const double sr = sum_partials(a, 0);
        const double zr = sum_partials(a, 1);
        if (threadIdx.x == 0) {
            st->res = sr / st->normf;
            st->iter = it + 1;
            st->step_iters += 1;
            if (pcg_converged(st, st->res) || st->iter >= st->max_iter) {
                if (!pcg_converged(st, st->res)) st->status |= CFG_ERR_PCG;
                end_solve(st);
            } else if (st->step_iters >= a.iter_cap) {
                // guard of the device-driven loops: give up the step
                st->status |= CFG_ERR_PCG;
                end_solve(st);
                st->outer_active = 0;
            } else {
                st->wArAold = st->wArA;
                st->wArA = zr;
                st->beta = st->wArA / st->wArAold;
            }
            set_inner(a, st->solve_active);
        }
    }
}

// End of a PIMPLE corrector in the step graph: whether another one runs.
__global__ void k_outer_cond(DiffusionArgs a) { set_outer(a, a.st->outer_active); }

__global__ void k_activation(DiffusionArgs a)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n) return;
    const double old_time = a.st->t - a.dt;
    activation(a, c, a.vm[c], a.vm_old[c], old_time);
}

// Explicit form: chi*Cm*ddt(Vm) == fvc::laplacian(sigma,Vm) - chi*Cm*Iion + src
// with a diagonal matrix; the Laplacian reads the start-of-step Vm, which
// vm_old holds.  Fused with the activation-time update.
__global__ void k_explicit(DiffusionArgs a)
{
    PcgState* st = a.st;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int n_old = st->n_old;   // read before any block updates it below
    if (c < a.n) {
        const int v = ddt_variant(a, n_old);
        const double cft = a.cft[v], cft0 = a.cft0[v], cft00 = a.cft00[v];
        const double rdt = a.rdt;
        const double V = a.vol[c];
        const double* x = a.vm_old;
        const double xc = x[c];
        // fvc::div of the face fluxes in face order: += for faces the cell
        // owns, -= for faces it neighbours
        double div = 0.0;
        if (a.sx) {
            const long long nx = a.sx, nxy = (long long)a.sx * a.sy;
            const long long i = c % nx, j = (c / nx) % a.sy, k = c / nxy;
            if (k > 0) div -= a.cz * (xc - x[c - nxy]);
            if (j > 0) div -= a.cy * (xc - x[c - nx]);
            if (i > 0) div -= a.cx * (xc - x[c - 1]);
            if (i + 1 < nx) div += a.cx * (x[c + 1] - xc);
            if (j + 1 < a.sy) div += a.cy * (x[c + nx] - xc);
            if (k + 1 < a.sz) div += a.cz * (x[c + nxy] - xc);
        } else {
            const int cnt = a.ell_cnt[c];
            for (int q = 0; q < cnt; ++q) {
                const long long nb = a.ell_col[(long long)q * a.n + c];
                const double coef = a.ell_coef[(long long)q * a.n + c];
                if (nb < c) div -= coef * (xc - x[nb]);
                else div += coef * (x[nb] - xc);
            }
            if (a.nc_gw) div += nc_correction_plain(a, c);
        }
        double diag, src;
        if (a.ddt_backward) {
            diag = a.chicm * ((cft * rdt) * V);
            src = a.chicm * (rdt * V * (cft0 * a.vm_old[c] - cft00 * a.vm_oldold[c]));
        } else {
            diag = a.chicm * (rdt * V);
            src = a.chicm * (rdt * a.vm_old[c] * V);
        }
        const double lapc = div / V;
        const double rhs = lapc - a.chicm * a.iion[c] + box_source(a, c, st->t0);
        src = src + rhs * V;
        const double vnew = src / diag;
        a.vm[c] = vnew;
        activation(a, c, vnew, a.vm_old[c], st->t - a.dt);
    }
}

__global__ void k_explicit_finish(PcgState* st, int ddt_backward)
{
    if (st->n_old < 1) st->n_old = 1;
    if (ddt_backward && st->n_old < 2) st->n_old = 2;
    st->n_solves = 0;
}

}  // namespace cfg
