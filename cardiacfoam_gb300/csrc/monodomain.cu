// cfg_monodomain_*: MyocardiumDomain + MonodomainSolver on one GPU
// (src/electroModels/electroDomains/myocardiumDomain/myocardiumDomain.C:180-529,
//  src/electroModels/myocardiumModels/monodomainSolver/monodomainSolver.C:39-150).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "diffusion_kernels.cuh"
#include "geometry.h"
#include "host_common.h"
#include "ionic_host.h"
#include "monodomain_host.h"

namespace cfg {

__global__ void k_prepare(DiffusionArgs a);
__global__ void k_step_begin(DiffusionArgs a);
__global__ void k_solve_begin(DiffusionArgs a);
__global__ void k_solve_norm(DiffusionArgs a);
__global__ void k_pcg_p(DiffusionArgs a);
__global__ void k_pcg_update(DiffusionArgs a);
__global__ void k_activation(DiffusionArgs a);
__global__ void k_explicit(DiffusionArgs a);
__global__ void k_explicit_finish(PcgState* st, int ddt_backward);
__global__ void k_grad_iterate(DiffusionArgs a);
__global__ void k_grad_start(DiffusionArgs a);

static void md_free(cfg_monodomain* md)
{
    if (!md) return;
    dfree(md->d_apd);
    dfree(md->d_apd_ring_t);
    dfree(md->d_apd_ring_v);
    dfree(md->d_pdiag2); dfree(md->d_prdiag2); dfree(md->d_psumA2); dfree(md->d_pcoef);
    dfree(md->d_px);
    if (md->graph_exec) cudaGraphExecDestroy(md->graph_exec);
    for (cudaEvent_t& e : md->ev)
        if (e) cudaEventDestroy(e);
    if (md->ion) ionic_free(md->ion);
    dfree(md->d_col); dfree(md->d_coef); dfree(md->d_cnt); dfree(md->d_lapdiag);
    dfree(md->d_vol); dfree(md->d_vm); dfree(md->d_vm_old); dfree(md->d_vm_oldold);
    dfree(md->d_iion); dfree(md->d_act); dfree(md->d_act_flag); dfree(md->d_box);
    dfree(md->d_diag2); dfree(md->d_rdiag2); dfree(md->d_sumA2); dfree(md->d_b); dfree(md->d_r);
    dfree(md->d_z); dfree(md->d_ax); dfree(md->d_pA); dfree(md->d_pB); dfree(md->d_ap);
    dfree(md->d_partial); dfree(md->d_st);
    for (void** p : {&md->d_nc_gw, &md->d_nc_k, &md->d_nc_om, &md->d_nc_bk, &md->d_grad}) {
        if (*p) cudaFree(*p);
        *p = nullptr;
    }
    dfree(md->d_bsrc);
    if (md->h_st) cudaFreeHost(md->h_st);
    if (md->stream) cudaStreamDestroy(md->stream);
    delete md;
}

// lduAddressing -> ELL rows with neighbours in ascending order (the order in
// which lduMatrix::Amul's face loop reaches a row for upper-triangular face
// ordering); lapdiag = sum of -coef in that order (fvMatrix::negSumDiag).
// On a general mesh (face centres given) the coefficients and the factors of
// the explicit correction come from the corrected assembly, laid out per ELL
// slot: gradient weight, signed correction vector and the row cell's
// interpolation weight of the slot's face.
static int build_operator(cfg_monodomain* md, const cfg_mesh_desc* m, const cfg_monodomain_desc* d)
{
    const long long n = m->n_cells, nf = m->n_faces;
    const double* sigma = d->conductivity;
    const bool general = m->face_centres != nullptr;
    if (d->conductivity_per_cell && !general)
        return fail(CFG_ERR_INVALID, "a per-cell conductivity needs the mesh's face_centres");
    if (general && m->face_coeff)
        return fail(CFG_ERR_INVALID, "give face_coeff or the full geometry, not both");
    for (long long f = 0; f < nf; ++f) {
        const int l = m->owner[f], u = m->neighbour[f];
        if (l < 0 || u < 0 || l >= n || u >= n || l == u)
            return fail(CFG_ERR_INVALID, "face %lld has invalid owner/neighbour %d/%d", f, l, u);
    }
    CorrectedOperator op;
    std::vector<double> fc;
    const double* coeff = m->face_coeff;
    if (general) {
        if (int rc = assemble_corrected(m, sigma, d->conductivity_per_cell, d->grad_scheme,
                                        d->laplacian_uncorrected, op))
            return rc;
        coeff = op.coeff.data();
    } else if (!coeff) {
        // face coefficients: deltaCoeffs * (Sf.sigma.Sf)/|Sf| for the uniform
        // conductivity (gaussLaplacianScheme, fvmLaplacianUncorrected)
        if (!m->face_sf || !m->face_delta_coeffs)
            return fail(CFG_ERR_INVALID, "mesh needs face_coeff or face_sf + face_delta_coeffs");
        fc.resize(size_t(nf));
        const double* s = sigma;
        for (long long f = 0; f < nf; ++f) {
            const double* S = m->face_sf + 3 * f;
            const double magSf = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
            const double g0 = S[0] * s[0] + S[1] * s[1] + S[2] * s[2];
            const double g1 = S[0] * s[1] + S[1] * s[3] + S[2] * s[4];
            const double g2 = S[0] * s[2] + S[1] * s[4] + S[2] * s[5];
            const double sfgsn = (g0 * S[0] + g1 * S[1] + g2 * S[2]) / magSf;
            fc[size_t(f)] = m->face_delta_coeffs[f] * sfgsn;
        }
        coeff = fc.data();
    }
    // MyocardiumDomain::suggestExplicitDeltaT at maxCo = 1
    // (myocardiumDomain.C:532-550): min over internal faces of dx^2/Df with
    // dx = 1/deltaCoeffs = |C_N - C_P| and Df = n.(n.sigma_f)/(chi Cm), sigma_f
    // the linear interpolate of the cells' conductivity.  From pre-assembled
    // face coefficients (orthogonal faces: coeff = |Sf| n.sigma_f.n/|d|) the
    // normal conductivity is coeff |d|/|Sf|.
    md->explicit_dt_unit = -1.0;
    if (m->face_sf && m->centres && nf > 0) {
        const double chicm = d->chi * d->cm;
        double best = 0.0;
        bool any = false;
        for (long long f = 0; f < nf; ++f) {
            const double* S = m->face_sf + 3 * f;
            const double magSf = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
            const double* cp = m->centres + 3 * size_t(m->owner[f]);
            const double* cn = m->centres + 3 * size_t(m->neighbour[f]);
            const double dd[3] = {cn[0] - cp[0], cn[1] - cp[1], cn[2] - cp[2]};
            const double dx = std::sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
            double nsn;
            if (m->face_coeff && !general) {
                nsn = m->face_coeff[f] * dx / magSf;
            } else {
                double sf[6];
                if (d->conductivity_per_cell) {
                    const double w = op.w[size_t(f)];
                    const double* a = d->conductivity_per_cell + 6 * size_t(m->owner[f]);
                    const double* b = d->conductivity_per_cell + 6 * size_t(m->neighbour[f]);
                    for (int k = 0; k < 6; ++k) sf[k] = w * a[k] + (1.0 - w) * b[k];
                } else {
                    for (int k = 0; k < 6; ++k) sf[k] = sigma[k];
                }
                const double nx = S[0] / magSf, ny = S[1] / magSf, nz = S[2] / magSf;
                const double g0 = nx * sf[0] + ny * sf[1] + nz * sf[2];
                const double g1 = nx * sf[1] + ny * sf[3] + nz * sf[4];
                const double g2 = nx * sf[2] + ny * sf[4] + nz * sf[5];
                nsn = nx * g0 + ny * g1 + nz * g2;
            }
            const double Df = nsn / chicm;
            if (!(Df > 0)) continue;
            const double v = dx * dx / Df;
            if (!any || v < best) best = v;
            any = true;
        }
        if (any) md->explicit_dt_unit = best;
    }
    // row entries: (column, face, the row cell owns the face)
    struct Entry {
        int col;
        long long face;
        bool own;
    };
    std::vector<std::vector<Entry>> rows(static_cast<size_t>(n));
    for (long long f = 0; f < nf; ++f) {
        const int l = m->owner[f], u = m->neighbour[f];
        rows[size_t(l)].push_back({u, f, true});
        rows[size_t(u)].push_back({l, f, false});
    }
    int width = 0;
    for (auto& r : rows) {
        std::stable_sort(r.begin(), r.end(),
                         [](const Entry& a, const Entry& b) { return a.col < b.col; });
        width = std::max(width, int(r.size()));
    }
    if (width > 255) return fail(CFG_ERR_INVALID, "cell with more than 255 faces");
    md->width = width;
    const size_t slots = size_t(width) * size_t(n);
    std::vector<int> col(slots, 0);
    std::vector<double> coef(slots, 0.0);
    std::vector<unsigned char> cnt(static_cast<size_t>(n));
    std::vector<double> lapdiag(static_cast<size_t>(n));
    std::vector<double> gw, kc, om;
    if (general) {
        gw.assign(3 * slots, 0.0);
        kc.assign(3 * slots, 0.0);
        om.assign(slots, 0.0);
    }
    for (long long c = 0; c < n; ++c) {
        const auto& r = rows[size_t(c)];
        cnt[size_t(c)] = (unsigned char)r.size();
        double s = 0.0;
        for (size_t q = 0; q < r.size(); ++q) {
            const size_t i = q * size_t(n) + size_t(c);
            const long long f = r[q].face;
            col[i] = r[q].col;
            coef[i] = coeff[f];
            s -= coeff[f];
            if (general) {
                const double* g = r[q].own ? op.g_own.data() : op.g_nei.data();
                const double sg = r[q].own ? 1.0 : -1.0;
                for (int k = 0; k < 3; ++k) {
                    gw[size_t(k) * slots + i] = g[3 * f + k];
                    kc[size_t(k) * slots + i] = sg * op.k[size_t(3 * f + k)];
                }
                om[i] = r[q].own ? op.w[size_t(f)] : 1.0 - op.w[size_t(f)];
            }
        }
        lapdiag[size_t(c)] = s;
    }
    // structured block with one coefficient per direction: stencil form
    md->sx = md->sy = md->sz = 0;
    if (!general && m->structured[0] > 0 &&
        (long long)m->structured[0] * m->structured[1] * m->structured[2] == n) {
        const long long nx = m->structured[0], ny = m->structured[1];
        double cdir[3] = {0, 0, 0};
        bool ok = true, seen[3] = {false, false, false};
        for (long long f = 0; f < nf && ok; ++f) {
            const long long l = m->owner[f], u = m->neighbour[f], d = u - l;
            const int dir = d == 1 ? 0 : d == nx ? 1 : d == nx * ny ? 2 : -1;
            if (dir < 0) { ok = false; break; }
            if (!seen[dir]) { cdir[dir] = coeff[f]; seen[dir] = true; }
            else if (std::fabs(coeff[f] - cdir[dir]) > 1e-12 * std::fabs(cdir[dir])) ok = false;
        }
        if (ok) {
            md->sx = m->structured[0]; md->sy = m->structured[1]; md->sz = m->structured[2];
            md->cx = cdir[0]; md->cy = cdir[1]; md->cz = cdir[2];
        }
    }
    CFG_CUDA_TRY(dmalloc(&md->d_col, col.size()));
    CFG_CUDA_TRY(dmalloc(&md->d_coef, coef.size()));
    CFG_CUDA_TRY(dmalloc(&md->d_cnt, cnt.size()));
    for (double v : lapdiag) md->max_neglap = std::max(md->max_neglap, -v);
    CFG_CUDA_TRY(dmalloc(&md->d_lapdiag, lapdiag.size()));
    CFG_CUDA_TRY(cudaMemcpy(md->d_col, col.data(), col.size() * sizeof(int), cudaMemcpyHostToDevice));
    CFG_CUDA_TRY(cudaMemcpy(md->d_coef, coef.data(), coef.size() * sizeof(double),
                            cudaMemcpyHostToDevice));
    CFG_CUDA_TRY(cudaMemcpy(md->d_cnt, cnt.data(), cnt.size(), cudaMemcpyHostToDevice));
    CFG_CUDA_TRY(cudaMemcpy(md->d_lapdiag, lapdiag.data(), lapdiag.size() * sizeof(double),
                            cudaMemcpyHostToDevice));
    md->ell_bytes = col.size() * sizeof(int) + coef.size() * sizeof(double) + cnt.size();
    md->nnz_offdiag = 2 * nf;
    md->corrected = general;
    if (general) {
        std::vector<double> bk(size_t(3) * size_t(n));
        for (long long c = 0; c < n; ++c)
            for (int k = 0; k < 3; ++k) bk[size_t(k) * size_t(n) + size_t(c)] = op.bk[size_t(3 * c + k)];
        // the mixed form evaluates the correction (a small explicit source)
        // in FP32 from FP64 differences of Vm
        md->nc_fp32 = d->ionic.precision == CFG_PRECISION_MIXED;
        auto upload = [&](void** dst, const std::vector<double>& v) -> cudaError_t {
            if (md->nc_fp32) {
                std::vector<float> f(v.begin(), v.end());
                cudaError_t e = cudaMalloc(dst, f.size() * sizeof(float));
                if (!e) e = cudaMemcpy(*dst, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice);
                return e;
            }
            cudaError_t e = cudaMalloc(dst, v.size() * sizeof(double));
            if (!e) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice);
            return e;
        };
        const size_t esz = md->nc_fp32 ? sizeof(float) : sizeof(double);
        CFG_CUDA_TRY(upload(&md->d_nc_gw, gw));
        CFG_CUDA_TRY(upload(&md->d_nc_k, kc));
        CFG_CUDA_TRY(upload(&md->d_nc_om, om));
        CFG_CUDA_TRY(upload(&md->d_nc_bk, bk));
        CFG_CUDA_TRY(cudaMalloc(&md->d_grad, esz * 3 * size_t(n)));
        CFG_CUDA_TRY(cudaMemset(md->d_grad, 0, esz * 3 * size_t(n)));
        md->ell_bytes += (gw.size() + kc.size() + om.size()) * esz;
    }
    return CFG_OK;
}

static cudaError_t alloc_pairs(cfg_monodomain* md)
{
    if (md->d_px) return cudaSuccess;
    const size_t n = size_t(md->n);
    cudaError_t e = dmalloc(&md->d_pdiag2, 2 * n);
    if (!e) e = dmalloc(&md->d_prdiag2, 2 * n);
    if (!e) e = dmalloc(&md->d_psumA2, 2 * n);
    // the stencil form keeps its three coefficients in the launch arguments
    if (!e && !md->use_stencil) e = dmalloc(&md->d_pcoef, size_t(md->width > 0 ? md->width : 1) * n);
    if (!e) e = dmalloc(&md->d_px, n);
    return e;
}

static void fill_args(cfg_monodomain* md, double dt)
{
    DiffusionArgs& a = md->args;
    a = DiffusionArgs{};
    a.n = md->n;
    a.width = md->width;
    a.ell_col = md->d_col;
    a.ell_coef = md->d_coef;
    a.ell_cnt = md->d_cnt;
    a.lapdiag = md->d_lapdiag;
    a.vol = md->d_vol;
    a.nc_gw = md->d_nc_gw;
    a.nc_k = md->d_nc_k;
    a.nc_om = md->d_nc_om;
    a.nc_bk = md->d_nc_bk;
    a.grad = md->d_grad;
    a.nc_fp32 = md->nc_fp32 ? 1 : 0;
    a.bsrc = md->d_bsrc;
    a.sx = md->use_stencil ? md->sx : 0;
    a.sy = md->sy;
    a.sz = md->sz;
    a.cx = md->cx; a.cy = md->cy; a.cz = md->cz;
    a.vm = md->d_vm;
    a.vm_old = md->d_vm_old;
    a.vm_oldold = md->d_vm_oldold;
    a.iion = md->d_iion;
    a.act = md->d_act;
    a.act_flag = md->d_act_flag;
    a.box_mask = md->d_box;
    a.n_boxes = md->n_boxes;
    for (int b = 0; b < md->n_boxes; ++b) {
        a.box_start[b] = md->box_start[b];
        a.box_end[b] = md->box_start[b] + md->box_duration[b];   // tStart + duration
        a.box_intensity[b] = md->box_intensity[b];
    }
    a.diag2 = md->d_diag2; a.rdiag2 = md->d_rdiag2; a.sumA2 = md->d_sumA2;
    a.b = md->d_b; a.r = md->d_r; a.z = md->d_z; a.ax = md->d_ax; a.pA = md->d_pA;
    a.pB = md->d_pB; a.ap = md->d_ap;
    a.partial = md->d_partial;
    a.nblocks = int((md->n + kDiffBlock - 1) / kDiffBlock);
    a.st = md->d_st;
    a.dt = dt;
    a.chicm = md->chicm;
    a.ddt_backward = md->ddt_backward;
    a.use_graph = 0;
    a.iter_cap = md->iter_cap;
    a.spin_limit = md->spin_limit;
    a.src_total = md->d_src_total;
    // float pairs: the system scaled by the power of two that brings its
    // largest diagonal near one
    a.pair = (md->pair && md->persistent && md->implicit) ? 1 : 0;
    if (a.pair) {
        const double dmax = md->chicm * 2.0 * md->max_vol / dt + md->max_neglap;
        a.pair_shift = dmax > 0 ? -std::ilogb(dmax) : 0;
        a.pdiag2 = md->d_pdiag2; a.prdiag2 = md->d_prdiag2; a.psumA2 = md->d_psumA2;
        a.pcoef = md->d_pcoef; a.px = md->d_px;
        const auto hsplit = [&](double v) {
            const double w = std::ldexp(v, a.pair_shift);
            const float h = float(w);
            return make_float2(h, float(w - double(h)));
        };
        a.pcx = hsplit(md->cx); a.pcy = hsplit(md->cy); a.pcz = hsplit(md->cz);
    }
    // ddt coefficients (EulerDdtScheme; backwardDdtScheme with deltaT0 =
    // GREAT while fewer than two old-time levels exist, then deltaT0 = dt)
    a.rdt = 1.0 / dt;
    for (int v = 0; v < 2; ++v) {
        if (!md->ddt_backward) {
            a.cft[v] = 1.0; a.cft0[v] = 1.0; a.cft00[v] = 0.0;
            continue;
        }
        const double dt0 = v == 0 ? 1e15 : dt;
        a.cft[v] = 1 + dt / (dt + dt0);
        a.cft00[v] = dt * dt / (dt0 * (dt + dt0));
        a.cft0[v] = a.cft[v] + a.cft00[v];
    }
}

void fill_args_public(cfg_monodomain* md, double dt) { fill_args(md, dt); }

int monodomain_create(const cfg_monodomain_desc* d, const cfg_mesh_desc* m, cfg_monodomain** out)
{
    if (!d || !m || !out) return fail(CFG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (m->n_cells <= 0) return fail(CFG_ERR_INVALID, "mesh has no cells");
    if (d->ionic.n_cells != m->n_cells)
        return fail(CFG_ERR_INVALID, "ionic model has %lld integration points, mesh %lld cells",
                    d->ionic.n_cells, m->n_cells);
    if (d->ionic.solve_vm_within_ode)
        return fail(CFG_ERR_INVALID, "the tissue step needs solveVmWithinODESolver false");
    if (!m->owner || !m->neighbour || !m->volumes || (d->n_boxes && !m->centres))
        return fail(CFG_ERR_INVALID, "incomplete mesh description");
    if (d->n_boxes < 0 || d->n_boxes > 8) return fail(CFG_ERR_INVALID, "at most 8 stimulus boxes");
    if (!(d->chi > 0) || !(d->cm > 0)) return fail(CFG_ERR_INVALID, "chi and cm must be positive");
    {
        const IonicModelOps* im = nullptr;
        int flag = 0;
        if (int rc = ionic_validate(&d->ionic, &im, &flag)) return rc;
    }

    cfg_monodomain* md = new cfg_monodomain();
    auto bail = [&](int rc) {
        md_free(md);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&md->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(CFG_ERR_CUDA, "stream creation failed"));
    int rc = ionic_create(&d->ionic, md->stream, &md->ion);
    if (rc) return bail(rc);
    md->n = m->n_cells;
    md->implicit = d->implicit != 0;
    md->ddt_backward = d->ddt_backward != 0;
    md->chicm = d->chi * d->cm;   // chi*Cm evaluated first (monodomainSolver.C:129)
    md->delta_t = d->ionic.initial_delta_t;
    md->n_boxes = d->n_boxes;
    for (int b = 0; b < d->n_boxes; ++b) {
        md->box_start[b] = d->box_start[b];
        md->box_duration[b] = d->box_duration[b];
        md->box_intensity[b] = d->box_intensity[b];
        for (int k = 0; k < 3; ++k) {
            md->box_min[b][k] = d->box_min[b][k];
            md->box_max[b][k] = d->box_max[b][k];
        }
    }
    if ((rc = build_operator(md, m, d))) return bail(rc);
    md->use_stencil = md->sx > 0;
    const size_t n = size_t(md->n);
    cudaError_t e = cudaSuccess;
    double** vecs[] = {&md->d_vol, &md->d_vm, &md->d_vm_old, &md->d_vm_oldold, &md->d_iion,
                       &md->d_act, &md->d_b, &md->d_r, &md->d_z, &md->d_ax, &md->d_pA,
                       &md->d_pB, &md->d_ap, &md->d_bsrc};
    for (double** v : vecs)
        if (!e) e = dmalloc(v, n);
    if (!e) e = dmalloc(&md->d_diag2, 2 * n);
    if (!e) e = dmalloc(&md->d_rdiag2, 2 * n);
    if (!e) e = dmalloc(&md->d_sumA2, 2 * n);
    const int nblocks = int((n + kDiffBlock - 1) / kDiffBlock);
    if (!e) e = dmalloc(&md->d_partial, size_t(4) * nblocks);
    if (!e) e = dmalloc(&md->d_act_flag, n);
    if (!e) e = dmalloc(&md->d_st, 1);
    for (size_t c = 0; c < n; ++c) md->max_vol = std::max(md->max_vol, m->volumes[c]);
    // float pairs by default in the mixed form on meshes without explicit
    // corrections; on corrected (tetrahedral) meshes the solve streams from
    // HBM and the FP64 PCG measured faster
    if (!e && d->ionic.precision == CFG_PRECISION_MIXED && !md->corrected) {
        e = alloc_pairs(md);
        md->pair = !e;
    }
    if (!e) e = cudaMallocHost(reinterpret_cast<void**>(&md->h_st), sizeof(PcgState));
    if (e) return bail(fail(CFG_ERR_CUDA, "device allocation failed: %s", cudaGetErrorString(e)));
    // box membership (boundBox::contains is inclusive)
    md->h_box.assign(n, 0);
    for (size_t c = 0; c < n; ++c)
        for (int b = 0; b < d->n_boxes; ++b) {
            const double* p = m->centres + 3 * c;
            bool in = true;
            for (int k = 0; k < 3; ++k)
                in = in && p[k] >= d->box_min[b][k] && p[k] <= d->box_max[b][k];
            if (in) md->h_box[c] |= (unsigned char)(1u << b);
        }
    if (d->n_boxes) {
        if (dmalloc(&md->d_box, n) != cudaSuccess)
            return bail(fail(CFG_ERR_CUDA, "device allocation failed"));
        cudaMemcpy(md->d_box, md->h_box.data(), n, cudaMemcpyHostToDevice);
    }
    std::vector<double> vm0(n, d->vm0);
    e = cudaMemcpy(md->d_vol, m->volumes, n * sizeof(double), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(md->d_vm, vm0.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(md->d_vm_old, vm0.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(md->d_vm_oldold, vm0.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemset(md->d_iion, 0, n * sizeof(double));
    if (!e) e = cudaMemset(md->d_act, 0, n * sizeof(double));
    if (!e) e = cudaMemset(md->d_act_flag, 1, n);
    if (!e) e = cudaMemset(md->d_partial, 0, sizeof(double) * 4 * nblocks);
    PcgState st{};
    st.n_old = 0;
    st.tol = d->pcg_tol;
    st.rel_tol = d->pcg_rel_tol;
    st.max_iter = d->pcg_max_iter > 0 ? d->pcg_max_iter : 1000;
    st.n_outer = d->n_outer > 0 ? d->n_outer : 1;
    st.outer_tol = d->outer_tol;
    if (!e) e = cudaMemcpy(md->d_st, &st, sizeof st, cudaMemcpyHostToDevice);
    if (e) return bail(fail(CFG_ERR_CUDA, "device initialisation failed: %s", cudaGetErrorString(e)));
    // persistent diffusion kernel: grid of co-resident blocks, if the device
    // supports cooperative launches
    {
        int dev = 0, coop = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess && coop)
            md->coop_blocks = coop_grid_blocks(n);
        md->persistent = md->coop_blocks > 0;
        cudaGetLastError();
    }
    *out = md;
    return CFG_OK;
}

static int read_state(cfg_monodomain* md)
{
    CFG_CUDA_TRY(cudaMemcpyAsync(md->h_st, md->d_st, sizeof(PcgState), cudaMemcpyDeviceToHost,
                                 md->stream));
    CFG_CUDA_TRY(cudaStreamSynchronize(md->stream));
    return CFG_OK;
}

// Enqueue the work of one time step.  With `host_control` the PIMPLE and PCG
// loops are driven from the host by reading the device state; otherwise a
// fixed sequence is enqueued whose surplus kernels return at once.
int enqueue_step(cfg_monodomain* md, double dt, bool host_control)
{
    long long launches = 0;
    struct Count {
        cfg_monodomain* m;
        long long& n;
        ~Count() { if (m->timing) m->timed_launches += n; }
    } counter{md, launches};
    fill_args(md, dt);
    const DiffusionArgs& a = md->args;
    const unsigned grid = unsigned(a.nblocks);
    cudaStream_t s = md->stream;
    if (dt != md->prepared_dt) {
        k_prepare<<<grid, kDiffBlock, 0, s>>>(a);
        CFG_CUDA_TRY(cudaGetLastError());
        md->prepared_dt = dt;
        launches += 1;
    }
    k_step_begin<<<grid, kDiffBlock, 0, s>>>(a);
    CFG_CUDA_TRY(cudaGetLastError());
    if (md->timing) CFG_CUDA_TRY(cudaEventRecord(md->ev[0], s));
    IonicLaunch L = ionic_launch_args(md->ion, 0.0, dt, &md->d_st->t0, md->d_vm, md->d_iion);
    CFG_CUDA_TRY(ionic_enqueue(md->ion, L));
    launches += 2;
    if (md->timing) CFG_CUDA_TRY(cudaEventRecord(md->ev[1], s));
    if (!md->implicit) {
        if (md->corrected) {
            k_grad_start<<<grid, kDiffBlock, 0, s>>>(a);
            launches += 1;
        }
        k_explicit<<<grid, kDiffBlock, 0, s>>>(a);
        k_explicit_finish<<<1, 1, 0, s>>>(md->d_st, md->ddt_backward);
        launches += 2;
        CFG_CUDA_TRY(cudaGetLastError());
        if (md->timing) CFG_CUDA_TRY(cudaEventRecord(md->ev[2], s));
        return CFG_OK;
    }
    if (md->persistent) {
        CFG_CUDA_TRY(launch_implicit_coop(a, md->coop_blocks, s));
        launches += 1;
        if (md->timing) CFG_CUDA_TRY(cudaEventRecord(md->ev[2], s));
        return CFG_OK;
    }
    if (host_control) {
        for (int corr = 0; corr < 1000000; ++corr) {
            if (md->corrected) {
                k_grad_iterate<<<grid, kDiffBlock, 0, s>>>(a);
                launches += 1;
            }
            k_solve_begin<<<grid, kDiffBlock, 0, s>>>(a);
            k_solve_norm<<<grid, kDiffBlock, 0, s>>>(a);
            launches += 2;
            CFG_CUDA_TRY(cudaGetLastError());
            int rc = read_state(md);
            if (rc) return rc;
            while (md->h_st->solve_active) {
                for (int k = 0; k < md->iter_chunk; ++k) {
                    k_pcg_p<<<grid, kDiffBlock, 0, s>>>(a);
                    k_pcg_update<<<grid, kDiffBlock, 0, s>>>(a);
                }
                launches += 2 * md->iter_chunk;
                CFG_CUDA_TRY(cudaGetLastError());
                if ((rc = read_state(md))) return rc;
            }
            if (!md->h_st->outer_active) break;
        }
    } else {
        for (int corr = 0; corr < md->graph_max_corr; ++corr) {
            if (md->corrected) k_grad_iterate<<<grid, kDiffBlock, 0, s>>>(a);
            k_solve_begin<<<grid, kDiffBlock, 0, s>>>(a);
            k_solve_norm<<<grid, kDiffBlock, 0, s>>>(a);
            for (int k = 0; k < md->graph_max_iter; ++k) {
                k_pcg_p<<<grid, kDiffBlock, 0, s>>>(a);
                k_pcg_update<<<grid, kDiffBlock, 0, s>>>(a);
            }
        }
        CFG_CUDA_TRY(cudaGetLastError());
    }
    k_activation<<<grid, kDiffBlock, 0, s>>>(a);
    launches += 1;
    CFG_CUDA_TRY(cudaGetLastError());
    if (md->timing) CFG_CUDA_TRY(cudaEventRecord(md->ev[2], s));
    return CFG_OK;
}

int check_step(cfg_monodomain* md)
{
    int rc = read_state(md);
    if (rc) return rc;
    if (md->timing) {
        float a = 0, b = 0;
        CFG_CUDA_TRY(cudaEventElapsedTime(&a, md->ev[0], md->ev[1]));
        CFG_CUDA_TRY(cudaEventElapsedTime(&b, md->ev[1], md->ev[2]));
        md->ionic_ms += a;
        md->diffusion_ms += b;
        md->timed_steps++;
    }
    if ((rc = ionic_check_status(md->ion))) return rc;
    if (md->h_st->bar_abort)
        return fail(CFG_ERR_PCG, "diffusion kernel aborted: a grid barrier timed out");
    if (md->implicit && (md->h_st->outer_active || md->h_st->solve_active))
        return fail(CFG_ERR_PCG, "PIMPLE/PCG loop did not finish within the launched sequence");
    return CFG_OK;
}

}  // namespace cfg

using namespace cfg;

// --- per-cell APD tracking on the tissue's Vm ---------------------------------
__global__ void k_apd_init(long long n, ApdTracker* apd)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    ApdTracker a{};
    a.last_apd = cfg_nan();
    a.last_ca = cfg_nan();
    a.last_t_up = cfg_nan();
    apd[c] = a;
}

// one sample (t, Vm in mV) of every cell; no calcium trace in the tissue
__global__ void k_apd_sample(long long n, double t, const double* __restrict__ vm,
                             ApdTracker* apd, ApdParams P, double* ring_t, double* ring_v)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    ApdTracker a = apd[c];
    apd_sample(a, P, t, 1000.0 * vm[c], cfg_nan(), ring_t + c, ring_v + c, n);
    apd[c] = a;
}

// the trace ending at the last sample: beats and the last beat's APD90, on a
// copy of each tracker (the live one keeps running)
__global__ void k_apd_results(long long n, const ApdTracker* apd, ApdParams P, int* beats,
                              double* apd90, double* t_up)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    ApdTracker a = apd[c];
    apd_end(a, P);
    beats[c] = a.n_beats;
    apd90[c] = a.last_apd * 1000.0;
    t_up[c] = a.last_t_up;
}

namespace cfg {

// The tissue's source density of a coupled step: the box stimulus
// (MyocardiumDomain::updateExternalStimulusCurrent) then each deposit of the
// PVJ coupling in terminal order (PVJMapper::depositCoupling).
struct BoxSrc {
    const unsigned char* mask;
    int n_boxes;
    double start[8], end[8], intensity[8];
};

__global__ void k_src_total(long long n, BoxSrc b, double t0, const int* dep_off,
                            const int* dep_term, const double* dep_value, double* src)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double s = 0.0;
    if (b.mask) {
        const unsigned m = b.mask[c];
        for (int k = 0; k < b.n_boxes; ++k) {
            if (t0 < b.start[k] || t0 > b.end[k]) continue;
            if (m & (1u << k)) s += b.intensity[k];
        }
    }
    for (int k = dep_off[c]; k < dep_off[c + 1]; ++k) s += dep_value[dep_term[k]];
    src[c] = s;
}

int monodomain_source_total(cfg_monodomain* md, double t0, const int* dep_off,
                            const int* dep_term, const double* dep_value, double* src_total)
{
    BoxSrc b{};
    b.mask = md->d_box;
    b.n_boxes = md->n_boxes;
    for (int k = 0; k < md->n_boxes; ++k) {
        b.start[k] = md->box_start[k];
        b.end[k] = md->box_start[k] + md->box_duration[k];
        b.intensity[k] = md->box_intensity[k];
    }
    k_src_total<<<unsigned((md->n + 255) / 256), 256, 0, md->stream>>>(md->n, b, t0, dep_off,
                                                                      dep_term, dep_value,
                                                                      src_total);
    CFG_CUDA_TRY(cudaGetLastError());
    return CFG_OK;
}

int monodomain_attach_network(cfg_monodomain* md, cfg_purkinje* pk, double* src_total)
{
    if (md->graph_exec) {   // the source pointer is an argument of the captured kernels
        cudaGraphExecDestroy(md->graph_exec);
        md->graph_exec = nullptr;
    }
    md->pk = pk;
    md->d_src_total = src_total;
    md->prepared_dt = 0.0;  // refill the launch arguments at the next step
    return CFG_OK;
}

}  // namespace cfg

static int apd_after_step(cfg_monodomain* md)
{
    if (md->apd_every <= 0) return CFG_OK;
    if (++md->apd_steps % md->apd_every) return CFG_OK;
    const unsigned grid = unsigned((md->n + 255) / 256);
    k_apd_sample<<<grid, 256, 0, md->stream>>>(md->n, md->t_host, md->d_vm, md->d_apd, md->apdp,
                                               md->d_apd_ring_t, md->d_apd_ring_v);
    CFG_CUDA_TRY(cudaGetLastError());
    return CFG_OK;
}

extern "C" {

int cfg_monodomain_track_apd(cfg_monodomain* md, int every_steps)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    dfree(md->d_apd);
    dfree(md->d_apd_ring_t);
    dfree(md->d_apd_ring_v);
    md->d_apd = nullptr;
    md->d_apd_ring_t = md->d_apd_ring_v = nullptr;
    md->apd_every = 0;
    if (every_steps <= 0) return CFG_OK;
    if (!(md->delta_t > 0)) return fail(CFG_ERR_INVALID, "the context has no time step");
    const ApdParams P = apd_defaults(md->delta_t * every_steps);
    if (P.ring > 4096)
        return fail(CFG_ERR_INVALID, "sampling every %d steps of %g s keeps %d samples for the "
                                     "2 ms baseline window (at most 4096)", every_steps,
                    md->delta_t, P.ring);
    const size_t n = size_t(md->n);
    cudaError_t e = dmalloc(&md->d_apd, n);
    if (!e) e = dmalloc(&md->d_apd_ring_t, size_t(P.ring) * n);
    if (!e) e = dmalloc(&md->d_apd_ring_v, size_t(P.ring) * n);
    if (e) {
        dfree(md->d_apd); dfree(md->d_apd_ring_t); dfree(md->d_apd_ring_v);
        md->d_apd = nullptr;
        md->d_apd_ring_t = md->d_apd_ring_v = nullptr;
        return fail(CFG_ERR_CUDA, "device allocation failed: %s", cudaGetErrorString(e));
    }
    md->apdp = P;
    md->apd_every = every_steps;
    md->apd_steps = 0;
    const unsigned grid = unsigned((md->n + 255) / 256);
    k_apd_init<<<grid, 256, 0, md->stream>>>(md->n, md->d_apd);
    // sample 0: the field as it is now
    k_apd_sample<<<grid, 256, 0, md->stream>>>(md->n, md->t_host, md->d_vm, md->d_apd, md->apdp,
                                               md->d_apd_ring_t, md->d_apd_ring_v);
    CFG_CUDA_TRY(cudaGetLastError());
    return CFG_OK;
}

int cfg_monodomain_apd_results(cfg_monodomain* md, int* n_beats, double* apd90_ms, double* t_up)
{
    if (!md || !n_beats || !apd90_ms || !t_up) return fail(CFG_ERR_INVALID, "null argument");
    if (md->apd_every <= 0) return fail(CFG_ERR_INVALID, "APD tracking is not enabled");
    const size_t n = size_t(md->n);
    int* d_b = nullptr;
    double *d_a = nullptr, *d_t = nullptr;
    cudaError_t e = dmalloc(&d_b, n);
    if (!e) e = dmalloc(&d_a, n);
    if (!e) e = dmalloc(&d_t, n);
    if (!e) {
        const unsigned grid = unsigned((md->n + 255) / 256);
        k_apd_results<<<grid, 256, 0, md->stream>>>(md->n, md->d_apd, md->apdp, d_b, d_a, d_t);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpyAsync(n_beats, d_b, n * sizeof(int), cudaMemcpyDeviceToHost, md->stream);
    if (!e) e = cudaMemcpyAsync(apd90_ms, d_a, n * sizeof(double), cudaMemcpyDeviceToHost, md->stream);
    if (!e) e = cudaMemcpyAsync(t_up, d_t, n * sizeof(double), cudaMemcpyDeviceToHost, md->stream);
    if (!e) e = cudaStreamSynchronize(md->stream);
    dfree(d_b);
    dfree(d_a);
    dfree(d_t);
    if (e) return fail(CFG_ERR_CUDA, "APD results: %s", cudaGetErrorString(e));
    return CFG_OK;
}

int cfg_monodomain_create(const cfg_monodomain_desc* desc, const cfg_mesh_desc* mesh,
                          cfg_monodomain** out)
{
    clear_error();
    return monodomain_create(desc, mesh, out);
}

// Enqueue one step from the step graph (built on first use and whenever dt
// or the timing switch changes).
static int enqueue_graph_step(cfg_monodomain* md, double dt)
{
    if (dt != md->prepared_dt) {
        fill_args(md, dt);
        const unsigned grid = unsigned(md->args.nblocks);
        k_prepare<<<grid, kDiffBlock, 0, md->stream>>>(md->args);
        CFG_CUDA_TRY(cudaGetLastError());
        md->prepared_dt = dt;
    }
    if (!md->graph_exec || md->graph_dt != dt || md->graph_timing != md->timing ||
        md->graph_persistent != md->persistent) {
        int rc = build_step_graph(md, dt);
        if (rc) return rc;
    }
    CFG_CUDA_TRY(cudaGraphLaunch(md->graph_exec, md->stream));
    return CFG_OK;
}

// kernels a graph step launched, from the step's solver statistics
static long long graph_step_launches(const cfg_monodomain* md)
{
    if (!md->implicit) return 4;
    if (md->persistent) return 3;   // step_begin, ionic, persistent diffusion
    long long n = 3;   // step_begin, ionic, activation
    for (int k = 0; k < md->h_st->n_solves && k < kMaxSolves; ++k)
        n += 3 + 2LL * md->h_st->iters[k];
    return n;
}

int cfg_monodomain_step(cfg_monodomain* md, double dt)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    if (dt == 0.0) dt = md->delta_t;   // the context's own time step
    if (!(dt > 0)) return fail(CFG_ERR_INVALID, "deltaT must be positive");
    if (md->pk)
        if (int rc = purkinje_prepare_coupled_step(md->pk, md, md->t_host, dt)) return rc;
    int rc = md->use_graph ? enqueue_graph_step(md, dt) : enqueue_step(md, dt, true);
    if (rc) return rc;
    md->t_host = md->t_host + dt;
    md->steps++;
    if ((rc = apd_after_step(md))) return rc;
    rc = check_step(md);
    if (!rc && md->pk) rc = purkinje_check(md->pk);
    if (!rc && md->use_graph && md->timing) md->timed_launches += graph_step_launches(md);
    return rc;
}

int cfg_monodomain_run(cfg_monodomain* md, double dt, long long n_steps)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    if (dt == 0.0) dt = md->delta_t;
    if (!(dt > 0)) return fail(CFG_ERR_INVALID, "deltaT must be positive");
    if (!md->use_graph || md->timing) {
        for (long long i = 0; i < n_steps; ++i) {
            int rc = cfg_monodomain_step(md, dt);
            if (rc) return rc;
        }
        return CFG_OK;
    }
    for (long long i = 0; i < n_steps; ++i) {
        if (md->pk)
            if (int rc = purkinje_prepare_coupled_step(md->pk, md, md->t_host, dt)) return rc;
        int rc = enqueue_graph_step(md, dt);
        if (rc) return rc;
        md->t_host = md->t_host + dt;
        md->steps++;
        if ((rc = apd_after_step(md))) return rc;
    }
    if (n_steps <= 0) return CFG_OK;
    int rc = check_step(md);
    if (!rc && md->pk) rc = purkinje_check(md->pk);
    return rc;
}

int cfg_monodomain_set_graph(cfg_monodomain* md, int enable)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    md->use_graph = enable != 0;
    return CFG_OK;
}

int cfg_monodomain_autotune(cfg_monodomain* md, int* block, int* cells_per_thread,
                            float* ionic_ms)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    clear_error();
    CFG_CUDA_TRY(cudaStreamSynchronize(md->stream));
    const double dt = md->graph_dt > 0 ? md->graph_dt : (md->prepared_dt > 0 ? md->prepared_dt : 1e-5);
    int rc = ionic_autotune(md->ion, md->t_host, dt, nullptr, md->d_vm, 3, block,
                            cells_per_thread, ionic_ms);
    if (rc) return rc;
    // the launch shape is part of the captured step graph
    if (md->graph_exec) {
        cudaGraphExecDestroy(md->graph_exec);
        md->graph_exec = nullptr;
    }
    return CFG_OK;
}

int cfg_monodomain_set_wait_limit(cfg_monodomain* md, long long spins)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    md->spin_limit = spins < 0 ? gsync::kSpinLimit : spins;
    // the limit is an argument of the kernels captured in the step graph
    if (md->graph_exec) {
        cudaGraphExecDestroy(md->graph_exec);
        md->graph_exec = nullptr;
    }
    return CFG_OK;
}

int cfg_monodomain_set_persistent(cfg_monodomain* md, int enable)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    if (enable && md->coop_blocks <= 0)
        return fail(CFG_ERR_UNSUPPORTED, "cooperative launch is not available on this device");
    if (md->persistent != (enable != 0))
        md->prepared_dt = 0.0;   // the pair operator follows the persistent kernel
    md->persistent = enable != 0;
    return CFG_OK;
}

int cfg_monodomain_set_pcg_arithmetic(cfg_monodomain* md, int arithmetic)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    if (arithmetic != CFG_PCG_FP64 && arithmetic != CFG_PCG_FLOAT_PAIRS)
        return fail(CFG_ERR_INVALID, "unknown PCG arithmetic %d", arithmetic);
    const bool pair = arithmetic == CFG_PCG_FLOAT_PAIRS;
    if (pair) {
        const cudaError_t e = alloc_pairs(md);
        if (e) return fail(CFG_ERR_CUDA, "device allocation failed: %s", cudaGetErrorString(e));
    }
    if (pair != md->pair) {
        md->pair = pair;
        md->prepared_dt = 0.0;   // the pair operator is prepared with the next step
        if (md->graph_exec) {
            cudaGraphExecDestroy(md->graph_exec);
            md->graph_exec = nullptr;
        }
    }
    return CFG_OK;
}

int cfg_monodomain_get_field(cfg_monodomain* md, int field, double* host)
{
    if (!md || !host) return fail(CFG_ERR_INVALID, "null argument");
    const size_t bytes = sizeof(double) * size_t(md->n);
    const double* src = nullptr;
    switch (field) {
    case CFG_FIELD_VM: src = md->d_vm; break;
    case CFG_FIELD_IION: src = md->d_iion; break;
    case CFG_FIELD_ACTIVATION: src = md->d_act; break;
    case CFG_FIELD_VM_OLD: src = md->d_vm_old; break;
    case CFG_FIELD_SOURCE: {
        // externalStimulusCurrent of the last step start
        const double t0 = md->t_host - md->args.dt;
        for (long long c = 0; c < md->n; ++c) {
            double s = 0.0;
            for (int b = 0; b < md->n_boxes; ++b) {
                const double ts = md->box_start[b], te = ts + md->box_duration[b];
                if (md->steps == 0 || t0 < ts || t0 > te) continue;
                if (md->h_box[size_t(c)] & (1u << b)) s += md->box_intensity[b];
            }
            host[c] = s;
        }
        return CFG_OK;
    }
    default: return fail(CFG_ERR_INVALID, "unknown field %d", field);
    }
    CFG_CUDA_TRY(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, md->stream));
    CFG_CUDA_TRY(cudaStreamSynchronize(md->stream));
    return CFG_OK;
}

int cfg_monodomain_set_field(cfg_monodomain* md, int field, const double* host)
{
    if (!md || !host) return fail(CFG_ERR_INVALID, "null argument");
    const size_t bytes = sizeof(double) * size_t(md->n);
    if (field == CFG_FIELD_VM) {
        CFG_CUDA_TRY(cudaMemcpyAsync(md->d_vm, host, bytes, cudaMemcpyHostToDevice, md->stream));
        if (md->steps == 0) {
            // no old-time level exists yet: the first access copies Vm
            CFG_CUDA_TRY(cudaMemcpyAsync(md->d_vm_old, host, bytes, cudaMemcpyHostToDevice, md->stream));
            CFG_CUDA_TRY(cudaMemcpyAsync(md->d_vm_oldold, host, bytes, cudaMemcpyHostToDevice, md->stream));
        }
    } else if (field == CFG_FIELD_ACTIVATION) {
        CFG_CUDA_TRY(cudaMemcpyAsync(md->d_act, host, bytes, cudaMemcpyHostToDevice, md->stream));
    } else {
        return fail(CFG_ERR_INVALID, "field %d cannot be set", field);
    }
    CFG_CUDA_TRY(cudaStreamSynchronize(md->stream));
    return CFG_OK;
}

double cfg_monodomain_time(const cfg_monodomain* md) { return md ? md->t_host : 0.0; }

int cfg_monodomain_suggest_explicit_delta_t(const cfg_monodomain* md, double max_co, double* dt)
{
    if (!md || !dt) return fail(CFG_ERR_INVALID, "null argument");
    if (!(max_co > 0)) return fail(CFG_ERR_INVALID, "maxCo must be positive");
    if (!(md->explicit_dt_unit > 0))
        return fail(CFG_ERR_INVALID, "the explicit time-step rule needs the mesh's face_sf and "
                                     "centres and a positive normal conductivity");
    *dt = max_co * md->explicit_dt_unit;
    return CFG_OK;
}

int cfg_monodomain_delta_t(const cfg_monodomain* md, double* dt)
{
    if (!md || !dt) return fail(CFG_ERR_INVALID, "null argument");
    *dt = md->delta_t;
    return CFG_OK;
}

int cfg_monodomain_set_delta_t(cfg_monodomain* md, double dt)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    if (!(dt > 0)) return fail(CFG_ERR_INVALID, "deltaT must be positive");
    md->delta_t = dt;
    return CFG_OK;
}

cfg_ionic* cfg_monodomain_ionic(cfg_monodomain* md) { return md ? md->ion : nullptr; }

int cfg_monodomain_last_stats(const cfg_monodomain* md, cfg_step_stats* s)
{
    if (!md || !s) return fail(CFG_ERR_INVALID, "null argument");
    cfg_monodomain* m = const_cast<cfg_monodomain*>(md);
    int rc = read_state(m);
    if (rc) return rc;
    std::memset(s, 0, sizeof *s);
    s->n_solves = m->h_st->n_solves;
    for (int k = 0; k < std::min(s->n_solves, 16); ++k) {
        s->iterations[k] = m->h_st->iters[k];
        s->initial_residual[k] = m->h_st->init_r[k];
        s->final_residual[k] = m->h_st->final_r[k];
    }
    return CFG_OK;
}

int cfg_monodomain_set_timing(cfg_monodomain* md, int enable)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    for (cudaEvent_t& e : md->ev)
        if (!e) CFG_CUDA_TRY(cudaEventCreate(&e));
    md->timing = enable != 0;
    md->ionic_ms = md->diffusion_ms = 0.0;
    md->timed_steps = 0;
    md->timed_launches = 0;
    return CFG_OK;
}

int cfg_monodomain_timings(const cfg_monodomain* md, double* ionic_ms, double* diffusion_ms,
                           long long* steps, long long* kernel_launches)
{
    if (!md) return fail(CFG_ERR_INVALID, "null context");
    if (ionic_ms) *ionic_ms = md->ionic_ms;
    if (diffusion_ms) *diffusion_ms = md->diffusion_ms;
    if (steps) *steps = md->timed_steps;
    if (kernel_launches) *kernel_launches = md->timed_launches;
    return CFG_OK;
}

void* cfg_monodomain_stream(cfg_monodomain* md) { return md ? (void*)md->stream : nullptr; }

int cfg_monodomain_destroy(cfg_monodomain* md)
{
    if (md) {
        cudaStreamSynchronize(md->stream);
        if (md->pk) purkinje_detach(md->pk);   // the network may outlive the context
        md_free(md);
    }
    return CFG_OK;
}

}  // extern "C"
