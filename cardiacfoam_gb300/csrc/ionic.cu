// cfg_ionic_*: the GPU ionic model behind the ionicModel plugin interface
// (src/ionicModels/ionicModel/ionicModel.H:184-256).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "host_common.h"
#include "ionic_host.h"

namespace cfg {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

void clear_error() { g_last_error.clear(); }

int tissue_flag(const char* t)
{
    if (!t) return -1;
    if (!std::strcmp(t, "epicardialCells")) return 1;
    if (!std::strcmp(t, "mCells")) return 2;
    if (!std::strcmp(t, "endocardialCells")) return 3;
    if (!std::strcmp(t, "myocyte")) return 4;
    // the manufactured-solution model's `dimension` key
    if (!std::strcmp(t, "1D")) return 11;
    if (!std::strcmp(t, "2D")) return 12;
    if (!std::strcmp(t, "3D")) return 13;
    return -1;
}

static const char* tissue_name(int f)
{
    switch (f) {
    case 1: return "epicardialCells";
    case 2: return "mCells";
    case 3: return "endocardialCells";
    case 4: return "myocyte";
    case 11: return "1D";
    case 12: return "2D";
    case 13: return "3D";
    default: return "unknown";
    }
}

static bool supported(const IonicModelOps* m, int flag)
{
    for (const int* t = m->tissues; *t; ++t)
        if (*t == flag) return true;
    return false;
}

static std::string supported_list(const IonicModelOps* m)
{
    std::string s = "(";
    for (const int* t = m->tissues; *t; ++t) {
        if (t != m->tissues) s += ' ';
        s += tissue_name(*t);
    }
    return s + ")";
}

OdeSettings make_ode(const cfg_ode_desc& d)
{
    OdeSettings s;
    s.abs_tol = d.abs_tol >= 0 ? d.abs_tol : 1e-15;
    s.rel_tol = d.rel_tol >= 0 ? d.rel_tol : 1e-4;
    s.max_steps = d.max_steps > 0 ? d.max_steps : 10000;
    s.safe_scale = d.safe_scale > 0 ? d.safe_scale : 0.9;
    s.min_scale = d.min_scale > 0 ? d.min_scale : 0.2;
    s.max_scale = d.max_scale > 0 ? d.max_scale : 10.0;
    s.alpha_inc = d.alpha_increase > 0 ? d.alpha_increase : 0.2;
    s.alpha_dec = d.alpha_decrease > 0 ? d.alpha_decrease : 0.25;
    s.inc_threshold = std::pow(s.max_scale / s.safe_scale, -1.0 / s.alpha_inc);
    return s;
}

int ionic_validate(const cfg_ionic_desc* d, const IonicModelOps** model, int* tissue)
{
    if (!d) return fail(CFG_ERR_INVALID, "null argument");
    const IonicModelOps* m = find_ionic_model(d->ionic_model);
    if (!m)
        return fail(CFG_ERR_INVALID, "Unknown ionicModel type %s. Valid ionicModel types are: %s",
                    d->ionic_model ? d->ionic_model : "(null)", ionic_model_names());
    if (d->ode.solver && std::strcmp(d->ode.solver, "RKF45") != 0)
        return fail(CFG_ERR_UNSUPPORTED, "ODE solver %s is not available on the GPU (RKF45 is)",
                    d->ode.solver);
    if (d->n_cells < 0) return fail(CFG_ERR_INVALID, "negative cell count");
    if (d->precision != CFG_PRECISION_FP64 && d->precision != CFG_PRECISION_MIXED)
        return fail(CFG_ERR_INVALID, "unknown precision %d", d->precision);
    // ionicSelector::selectTissue (ionicSelector.C:32-53)
    if (!d->tissue) return fail(CFG_ERR_INVALID, "Normal model requires 'tissue' entry");
    const int flag = tissue_flag(d->tissue);
    if (flag < 0 || !supported(m, flag))
        return fail(CFG_ERR_INVALID, "Unsupported tissue '%s' allowed: %s", d->tissue,
                    supported_list(m).c_str());
    if (d->tissue_per_cell) {
        for (long long c = 0; c < d->n_cells; ++c)
            if (!supported(m, d->tissue_per_cell[c]))
                return fail(CFG_ERR_INVALID, "cell %lld: unsupported tissue flag %d", c,
                            int(d->tissue_per_cell[c]));
    }
    if (!(d->initial_delta_t > 0)) return fail(CFG_ERR_INVALID, "initialDeltaT must be positive");
    // MyocardiumDomain::validateNoIonicStimulusInMonodomain (myocardiumDomain.C:377-394)
    // with stimulusIO::hasActiveStimulus (stimulusIO.C:288-303)
    {
        const cfg_stimulus_desc& s = d->stimulus;
        const double small = 1e-15;
        const bool s1 = s.stim_period_s1 > small && s.nstim1 > 0 && s.stim_duration > small &&
                        std::fabs(s.stim_amplitude) > small;
        const bool s2 = s.stim_period_s2 > small && s.nstim2 > 0 && s.stim_duration > small &&
                        std::fabs(s.stim_amplitude) > small;
        if (!d->solve_vm_within_ode && (s1 || s2))
            return fail(CFG_ERR_INVALID,
                        "Detected active ionic-model stimulus protocol while using a "
                        "reaction-diffusion myocardium domain; use externalStimulus instead");
    }
    *model = m;
    *tissue = flag;
    return CFG_OK;
}

int ionic_create(const cfg_ionic_desc* d, cudaStream_t stream, cfg_ionic** out)
{
    if (!out) return fail(CFG_ERR_INVALID, "null argument");
    *out = nullptr;
    const IonicModelOps* m = nullptr;
    int flag = 0;
    if (int rc = ionic_validate(d, &m, &flag)) return rc;
    cfg_ionic* ion = new cfg_ionic();
    ion->ops = m;
    ion->n = d->n_cells;
    ion->precision = d->precision;
    ion->solve_vm = d->solve_vm_within_ode != 0;
    ion->tissue = flag;
    ion->ode = make_ode(d->ode);
    const cfg_stimulus_desc& s = d->stimulus;
    ion->stim = CfgStimulus{s.stim_start, s.stim_period_s1, s.stim_duration, s.stim_amplitude,
                            s.nstim1, s.stim_period_s2, s.nstim2};
    ion->stream = stream;
    const long long n = ion->n;
    const int p = ion->precision;
    const int nw = m->n_wide[p], nn = m->ns - m->n_wide[p];
    auto cleanup_fail = [&](int code) {
        ionic_free(ion);
        return code;
    };
    cudaError_t e = cudaSuccess;
    if (!e) e = dmalloc(&ion->d_yw, size_t(nw) * n);
    if (!e) e = dmalloc(&ion->d_yn, size_t(nn) * n);
    if (!e) e = dmalloc(&ion->d_step, size_t(n));
    if (!e) e = dmalloc(&ion->d_vm, size_t(n));
    if (!e) e = dmalloc(&ion->d_im, size_t(n));
    if (!e) e = dmalloc(&ion->d_status, 1);
    if (!e) e = dmalloc(&ion->d_evals, 1);
    if (!e) e = dmalloc(&ion->d_fail, 8);
    if (!e) e = cudaMemsetAsync(ion->d_fail, 0, 8 * sizeof(double), stream);
    std::vector<unsigned char> slot_tissue;
    if (d->tissue_per_cell && !d->scales && !ion->solve_vm) {
        // group the cells by tissue flag (stable), one specialised launch per group
        long long count[256] = {0};
        for (long long c = 0; c < n; ++c) count[d->tissue_per_cell[c]]++;
        int distinct = 0, only = 0;
        for (int t = 0; t < 256; ++t)
            if (count[t]) { ++distinct; only = t; }
        if (distinct == 1) {
            ion->tissue = only;   // one tissue after all: the uniform launch
        } else if (distinct > 1) {
            long long start[256], at = 0;
            for (int t = 0; t < 256; ++t) {
                start[t] = at;
                if (count[t]) ion->groups.push_back({at, count[t], t});
                at += count[t];
            }
            ion->h_perm.resize(size_t(n));
            slot_tissue.resize(size_t(n));
            for (long long c = 0; c < n; ++c) {
                const int t = d->tissue_per_cell[c];
                ion->h_perm[size_t(start[t])] = int(c);
                slot_tissue[size_t(start[t])] = (unsigned char)t;
                start[t]++;
            }
        }
    } else if (d->tissue_per_cell) {
        slot_tissue.assign(d->tissue_per_cell, d->tissue_per_cell + n);
    }
    if (!e && !slot_tissue.empty()) {
        e = dmalloc(&ion->d_tissue, size_t(n));
        if (!e) e = cudaMemcpyAsync(ion->d_tissue, slot_tissue.data(), size_t(n),
                                    cudaMemcpyHostToDevice, stream);
    }
    if (!e && !ion->h_perm.empty()) {
        e = dmalloc(&ion->d_perm, size_t(n));
        if (!e) e = cudaMemcpyAsync(ion->d_perm, ion->h_perm.data(), sizeof(int) * size_t(n),
                                    cudaMemcpyHostToDevice, stream);
    }
    if (!e && d->scales) {
        e = dmalloc(&ion->d_scales, size_t(6) * n);
        if (!e) e = cudaMemcpyAsync(ion->d_scales, d->scales, sizeof(double) * 6 * size_t(n),
                                    cudaMemcpyHostToDevice, stream);
    }
    if (!e) e = cudaMemsetAsync(ion->d_status, 0, sizeof(int), stream);
    if (!e) e = cudaMemsetAsync(ion->d_evals, 0, sizeof(unsigned long long), stream);
    if (!e)
        e = m->init[p](n, flag, ion->d_tissue, ion->d_scales, n, d->initial_delta_t, ion->d_yw,
                       ion->d_yn, ion->d_step, stream);
    if (!e) e = cudaStreamSynchronize(stream);
    if (e) {
        fail(CFG_ERR_CUDA, "ionic model set-up failed: %s", cudaGetErrorString(e));
        return cleanup_fail(CFG_ERR_CUDA);
    }
    *out = ion;
    return CFG_OK;
}

void ionic_free(cfg_ionic* ion)
{
    if (!ion) return;
    dfree(ion->d_yw);
    dfree(ion->d_yn);
    dfree(ion->d_step);
    dfree(ion->d_vm);
    dfree(ion->d_im);
    dfree(ion->d_status);
    dfree(ion->d_evals);
    dfree(ion->d_fail);
    dfree(ion->d_tissue);
    dfree(ion->d_scales);
    dfree(ion->d_perm);
    if (ion->own_stream && ion->stream) cudaStreamDestroy(ion->stream);
    delete ion;
}

IonicLaunch ionic_launch_args(const cfg_ionic* ion, double t0, double dt, const double* t_dev,
                              const double* vm_dev, double* im_dev)
{
    IonicLaunch L{};
    L.n = ion->n;
    L.first = 0;
    L.count = ion->n;
    L.perm = ion->d_perm;
    L.cells_per_thread = ion->cells_per_thread;
    L.t0 = t0;
    L.dt = dt;
    L.t_dev = t_dev;
    L.tissue = ion->tissue;
    L.tissue_cell = ion->d_tissue;
    L.scales = ion->d_scales;
    L.scale_stride = ion->n;
    L.stim = ion->stim;
    L.ode = ion->ode;
    L.vm = vm_dev;
    L.im = im_dev;
    L.yw = ion->d_yw;
    L.yn = ion->d_yn;
    L.step = ion->d_step;
    L.status = ion->d_status;
    L.rhs_evals = ion->d_evals;
    L.fail_record = ion->d_fail;
    return L;
}

cudaError_t ionic_enqueue(const cfg_ionic* ion, const IonicLaunch& L)
{
    const auto step = ion->ops->step[ion->precision][ion->solve_vm ? 1 : 0];
    if (ion->groups.empty()) return step(L, ion->stream, ion->block);
    for (const cfg_ionic::Group& g : ion->groups) {
        IonicLaunch G = L;
        G.first = g.first;
        G.count = g.count;
        G.tissue = g.tissue;
        G.tissue_cell = nullptr;
        if (cudaError_t e = step(G, ion->stream, ion->block)) return e;
    }
    return cudaSuccess;
}

// Time every (block, cells per thread) candidate of the step kernel on
// scratch copies of the states (the context's states are not touched) and
// keep the fastest.  Each slot's arithmetic does not depend on the launch
// shape, so the choice changes the speed only.
int ionic_autotune(cfg_ionic* ion, double t0, double dt, const double* t_dev, const double* vm_dev,
                   int repeats, int* block_out, int* cpt_out, float* ms_out)
{
    const int p = ion->precision;
    const long long n = ion->n;
    const int nw = ion->ops->n_wide[p], nn = ion->ops->ns - nw;
    const int max_b = ion->ops->max_block[p]();
    std::vector<int> blocks;
    for (int b = 32; b <= max_b; b *= 2) blocks.push_back(b);
    const int cpts[] = {1, 2, 4};
    double *yw = nullptr, *step = nullptr, *im = nullptr;
    float* yn = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t s = ion->stream;
    auto cleanup = [&]() {
        if (yw) cudaFree(yw);
        if (yn) cudaFree(yn);
        if (step) cudaFree(step);
        if (im) cudaFree(im);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t e = dmalloc(&yw, size_t(nw) * n);
    if (!e) e = dmalloc(&yn, size_t(nn) * n);
    if (!e) e = dmalloc(&step, size_t(n));
    if (!e) e = dmalloc(&im, size_t(n));
    if (!e) e = cudaEventCreate(&e0);
    if (!e) e = cudaEventCreate(&e1);
    if (e) {
        cleanup();
        return fail(CFG_ERR_CUDA, "autotune set-up failed: %s", cudaGetErrorString(e));
    }
    const int saved_b = ion->block, saved_c = ion->cells_per_thread;
    float best = 1e30f;
    int best_b = saved_b, best_c = saved_c;
    for (int b : blocks)
        for (int c : cpts) {
            ion->block = b;
            ion->cells_per_thread = c;
            float total = 0.0f;
            for (int r = 0; r <= repeats && !e; ++r) {
                // the same starting states for every launch
                e = cudaMemcpyAsync(yw, ion->d_yw, sizeof(double) * size_t(nw) * n,
                                    cudaMemcpyDeviceToDevice, s);
                if (!e && nn)
                    e = cudaMemcpyAsync(yn, ion->d_yn, sizeof(float) * size_t(nn) * n,
                                        cudaMemcpyDeviceToDevice, s);
                if (!e) e = cudaMemcpyAsync(step, ion->d_step, sizeof(double) * n,
                                            cudaMemcpyDeviceToDevice, s);
                IonicLaunch L = ionic_launch_args(ion, t0, dt, t_dev, vm_dev, im);
                L.yw = yw;
                L.yn = yn;
                L.step = step;
                L.rhs_evals = nullptr;
                L.fail_record = nullptr;
                if (!e) e = cudaEventRecord(e0, s);
                if (!e) e = ionic_enqueue(ion, L);
                if (!e) e = cudaEventRecord(e1, s);
                if (!e) e = cudaEventSynchronize(e1);
                float ms = 0.0f;
                if (!e) e = cudaEventElapsedTime(&ms, e0, e1);
                if (r > 0) total += ms;        // the first launch warms up
            }
            if (e) break;
            if (total < best) {
                best = total;
                best_b = b;
                best_c = c;
            }
        }
    ion->block = e ? saved_b : best_b;
    ion->cells_per_thread = e ? saved_c : best_c;
    // a failing candidate must not leave an error status behind
    cudaMemsetAsync(ion->d_status, 0, sizeof(int), s);
    cudaStreamSynchronize(s);
    cleanup();
    if (e) return fail(CFG_ERR_CUDA, "autotune failed: %s", cudaGetErrorString(e));
    if (block_out) *block_out = best_b;
    if (cpt_out) *cpt_out = best_c;
    if (ms_out) *ms_out = best / float(repeats > 0 ? repeats : 1);
    return CFG_OK;
}

// Reorder n values per row between the state slots and the cells.
template <class T>
static void slots_to_cells(const cfg_ionic* ion, T* a)
{
    if (ion->h_perm.empty()) return;
    std::vector<T> tmp(a, a + ion->n);
    for (long long k = 0; k < ion->n; ++k) a[ion->h_perm[size_t(k)]] = tmp[size_t(k)];
}

template <class T>
static void cells_to_slots(const cfg_ionic* ion, const T* a, T* out)
{
    if (ion->h_perm.empty()) {
        std::copy(a, a + ion->n, out);
        return;
    }
    for (long long k = 0; k < ion->n; ++k) out[k] = a[ion->h_perm[size_t(k)]];
}

// state slot of integration point 0
static long long slot_of_cell0(const cfg_ionic* ion)
{
    for (size_t k = 0; k < ion->h_perm.size(); ++k)
        if (ion->h_perm[k] == 0) return (long long)k;
    return 0;
}

int ionic_check_status(cfg_ionic* ion)
{
    int st = 0;
    CFG_CUDA_TRY(cudaMemcpyAsync(&st, ion->d_status, sizeof(int), cudaMemcpyDeviceToHost,
                                 ion->stream));
    CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
    if (st & CFG_ERR_ODE_STEPS) {
        double r[8] = {0};
        cudaMemcpy(r, ion->d_fail, sizeof r, cudaMemcpyDeviceToHost);
        const int worst = int(r[4]);
        return fail(CFG_ERR_ODE_STEPS,
                    "%s: cell %lld: %s (maximum %lld) at x = %.17g, dx = %.6g after %lld "
                    "substeps; worst state %s = %.9g with normalised error %.6g",
                    ion->ops->name, (long long)r[0],
                    r[1] == 2 ? "stepsize underflow" : "Integration steps greater than maximum",
                    (long long)ion->ode.max_steps, r[2], r[3], (long long)r[7],
                    worst >= 0 && worst < ion->ops->ns ? ion->ops->state_names[worst] : "?",
                    r[6], r[5]);
    }
    if (st & CFG_ERR_NONFINITE)
        return fail(CFG_ERR_NONFINITE, "non-finite ionic current in %s", ion->ops->name);
    return CFG_OK;
}

}  // namespace cfg

using namespace cfg;

extern "C" {

const char* cfg_last_error(void) { return g_last_error.c_str(); }

int cfg_ionic_create(const cfg_ionic_desc* desc, cfg_ionic** out)
{
    clear_error();
    const IonicModelOps* m = nullptr;
    int flag = 0;
    if (!out) return fail(CFG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (int rc = ionic_validate(desc, &m, &flag)) return rc;
    cudaStream_t s = nullptr;
    CFG_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    int rc = ionic_create(desc, s, out);
    if (rc) {
        cudaStreamDestroy(s);
        return rc;
    }
    (*out)->own_stream = true;
    return CFG_OK;
}

int cfg_ionic_solve(cfg_ionic* ion, double t0, double dt, const double* vm, double* im)
{
    if (!ion) return fail(CFG_ERR_INVALID, "null ionic model");
    const size_t bytes = sizeof(double) * size_t(ion->n);
    if (!ion->solve_vm) {
        if (!vm) return fail(CFG_ERR_INVALID, "null Vm");
        CFG_CUDA_TRY(cudaMemcpyAsync(ion->d_vm, vm, bytes, cudaMemcpyHostToDevice, ion->stream));
    }
    IonicLaunch L = ionic_launch_args(ion, t0, dt, nullptr, ion->d_vm, ion->d_im);
    CFG_CUDA_TRY(ionic_enqueue(ion, L));
    if (im)
        CFG_CUDA_TRY(cudaMemcpyAsync(im, ion->d_im, bytes, cudaMemcpyDeviceToHost, ion->stream));
    return ionic_check_status(ion);
}

int cfg_ionic_solve_device(cfg_ionic* ion, double t0, double dt, const double* vm_dev,
                           double* im_dev)
{
    if (!ion) return fail(CFG_ERR_INVALID, "null ionic model");
    IonicLaunch L = ionic_launch_args(ion, t0, dt, nullptr, vm_dev, im_dev);
    CFG_CUDA_TRY(ionic_enqueue(ion, L));
    return CFG_OK;
}

int cfg_ionic_num_states(const cfg_ionic* ion, int* n)
{
    if (!ion || !n) return fail(CFG_ERR_INVALID, "null argument");
    *n = ion->ops->ns;
    return CFG_OK;
}

int cfg_ionic_state_name(const cfg_ionic* ion, int i, char* buf, size_t len)
{
    if (!ion || !buf || i < 0 || i >= ion->ops->ns) return fail(CFG_ERR_INVALID, "bad index");
    std::snprintf(buf, len, "%s", ion->ops->state_names[i]);
    return CFG_OK;
}

int cfg_ionic_get_states(cfg_ionic* ion, double* host)
{
    if (!ion || !host) return fail(CFG_ERR_INVALID, "null argument");
    const long long n = ion->n;
    const int p = ion->precision, ns = ion->ops->ns;
    std::vector<float> tmp;
    for (int i = 0; i < ns; ++i) {
        const int w = ion->ops->wide_of[p * ns + i], s = ion->ops->slot_of[p * ns + i];
        if (w) {
            double* dst = host + size_t(i) * n;
            CFG_CUDA_TRY(cudaMemcpyAsync(dst, ion->d_yw + size_t(s) * n, sizeof(double) * n,
                                         cudaMemcpyDeviceToHost, ion->stream));
            CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
            if (p == CFG_PRECISION_MIXED) {
                // each slot holds the FP32 pair (hi, lo) of the state
                for (long long c = 0; c < n; ++c) {
                    float hl[2];
                    std::memcpy(hl, dst + c, sizeof hl);
                    dst[c] = double(hl[0]) + double(hl[1]);
                }
            }
            slots_to_cells(ion, dst);
        } else {
            tmp.resize(n);
            CFG_CUDA_TRY(cudaMemcpyAsync(tmp.data(), ion->d_yn + size_t(s) * n, sizeof(float) * n,
                                         cudaMemcpyDeviceToHost, ion->stream));
            CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
            for (long long c = 0; c < n; ++c) host[size_t(i) * n + c] = tmp[c];
            slots_to_cells(ion, host + size_t(i) * n);
        }
    }
    CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
    return CFG_OK;
}

int cfg_ionic_set_states(cfg_ionic* ion, const double* host)
{
    if (!ion || !host) return fail(CFG_ERR_INVALID, "null argument");
    const long long n = ion->n;
    const int p = ion->precision, ns = ion->ops->ns;
    std::vector<float> tmp;
    std::vector<double> row(static_cast<size_t>(n));
    for (int i = 0; i < ns; ++i) {
        const int w = ion->ops->wide_of[p * ns + i], s = ion->ops->slot_of[p * ns + i];
        cells_to_slots(ion, host + size_t(i) * n, row.data());
        if (w && p == CFG_PRECISION_MIXED) {
            std::vector<double> pairs(static_cast<size_t>(n));
            for (long long c = 0; c < n; ++c) {
                const double v = row[size_t(c)];
                const float hl[2] = {float(v), float(v - double(float(v)))};
                std::memcpy(&pairs[size_t(c)], hl, sizeof hl);
            }
            CFG_CUDA_TRY(cudaMemcpyAsync(ion->d_yw + size_t(s) * n, pairs.data(),
                                         sizeof(double) * n, cudaMemcpyHostToDevice, ion->stream));
            CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
        } else if (w) {
            CFG_CUDA_TRY(cudaMemcpyAsync(ion->d_yw + size_t(s) * n, row.data(),
                                         sizeof(double) * n, cudaMemcpyHostToDevice, ion->stream));
            CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
        } else {
            tmp.resize(n);
            for (long long c = 0; c < n; ++c) tmp[c] = float(row[size_t(c)]);
            CFG_CUDA_TRY(cudaMemcpyAsync(ion->d_yn + size_t(s) * n, tmp.data(), sizeof(float) * n,
                                         cudaMemcpyHostToDevice, ion->stream));
            CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
        }
    }
    CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
    return CFG_OK;
}

int cfg_ionic_get_steps(cfg_ionic* ion, double* host)
{
    if (!ion || !host) return fail(CFG_ERR_INVALID, "null argument");
    CFG_CUDA_TRY(cudaMemcpyAsync(host, ion->d_step, sizeof(double) * size_t(ion->n),
                                 cudaMemcpyDeviceToHost, ion->stream));
    CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
    slots_to_cells(ion, host);
    return CFG_OK;
}

int cfg_ionic_rhs_evaluations(const cfg_ionic* ion, unsigned long long* count)
{
    if (!ion || !count) return fail(CFG_ERR_INVALID, "null argument");
    CFG_CUDA_TRY(cudaMemcpyAsync(count, ion->d_evals, sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, ion->stream));
    CFG_CUDA_TRY(cudaStreamSynchronize(ion->stream));
    return CFG_OK;
}

int cfg_ionic_set_launch(cfg_ionic* ion, int block, int cells_per_thread)
{
    if (!ion) return fail(CFG_ERR_INVALID, "null ionic model");
    const int max_b = ion->ops->max_block[ion->precision]();
    if (block < 0 || block > max_b || block % 32 != 0 || cells_per_thread < 1)
        return fail(CFG_ERR_INVALID, "launch shape %d x %d: block must be a multiple of 32 up to %d",
                    block, cells_per_thread, max_b);
    ion->block = block;
    ion->cells_per_thread = cells_per_thread;
    return CFG_OK;
}

int cfg_ionic_autotune(cfg_ionic* ion, double t0, double dt, const double* vm_dev,
                       int* block, int* cells_per_thread, float* ms_per_step)
{
    if (!ion) return fail(CFG_ERR_INVALID, "null ionic model");
    clear_error();
    const double* vm = vm_dev;
    if (!ion->solve_vm && !vm) {
        // the context's Vm staging buffer at the resting value
        std::vector<double> v(size_t(ion->n), -0.084);
        CFG_CUDA_TRY(cudaMemcpy(ion->d_vm, v.data(), sizeof(double) * v.size(),
                                cudaMemcpyHostToDevice));
        vm = ion->d_vm;
    }
    return ionic_autotune(ion, t0, dt, nullptr, vm, 3, block, cells_per_thread, ms_per_step);
}

int cfg_ionic_destroy(cfg_ionic* ion)
{
    if (ion) {
        cudaStreamSynchronize(ion->stream);
        ionic_free(ion);
    }
    return CFG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- sweepCurrent

namespace cfg {
namespace {

// ionicVariableCompatibility::canonicalName (ionicVariableCompatibility.C:37-59):
// lower case, separators dropped, an "av" prefix stripped
std::string canonical_name(const char* raw)
{
    std::string out;
    for (const char* p = raw; *p; ++p) {
        char c = *p;
        if (c >= 'A' && c <= 'Z') c = char(c - 'A' + 'a');
        if (c == '_' || c == '-' || c == ' ') continue;
        out.push_back(c);
    }
    if (out.size() > 2 && out[0] == 'a' && out[1] == 'v') return out.substr(2);
    return out;
}

bool same_name(const std::string& name, const char* table_entry)
{
    return name == table_entry || canonical_name(name.c_str()) == canonical_name(table_entry);
}

// resolveVariable (ionicVariableCompatibility.C:215-275): Vm, a state, an
// algebraic, or RATES_<state> (prefix case-insensitive).  The column is an
// index into a sweep row [states | algebraic | rates].
bool resolve_column(const IonicModelOps* m, const std::string& name, int* col)
{
    if (name == "Vm" || canonical_name(name.c_str()) == "vm") {
        *col = 0;
        return true;
    }
    for (int s = 0; s < m->ns; ++s)
        if (same_name(name, m->state_strings[s])) { *col = s; return true; }
    for (int a = 0; a < m->na; ++a)
        if (m->alg_strings[a][0] && same_name(name, m->alg_strings[a])) { *col = m->ns + a; return true; }
    static const char prefix[] = "RATES_";
    if (name.size() > 6) {
        bool ok = true;
        for (int i = 0; i < 6; ++i) {
            char c = name[size_t(i)];
            if (c >= 'A' && c <= 'Z') c = char(c - 'A' + 'a');
            char q = prefix[i];
            if (q >= 'A' && q <= 'Z') q = char(q - 'A' + 'a');
            ok = ok && c == q;
        }
        if (ok) {
            const std::string st = name.substr(6);
            for (int s = 0; s < m->ns; ++s)
                if (same_name(st, m->state_strings[s])) { *col = m->ns + m->na + s; return true; }
        }
    }
    return false;
}

std::vector<std::string> split_commas(const char* s)
{
    std::vector<std::string> out;
    std::string cur;
    for (const char* p = s; *p; ++p) {
        if (*p == ',') { out.push_back(cur); cur.clear(); }
        else cur.push_back(*p);
    }
    if (!cur.empty()) out.push_back(cur);
    return out;
}

// The states (FP64; the mixed form's pairs summed), constants and tissue of
// integration point `cell`.
int cell_snapshot(cfg_ionic* ion, long long cell, std::vector<double>& y0, std::vector<double>& C,
                  int* tissue_out)
{
    const IonicModelOps* m = ion->ops;
    const long long n = ion->n;
    long long k0 = cell;
    if (!ion->h_perm.empty())
        for (size_t k = 0; k < ion->h_perm.size(); ++k)
            if (ion->h_perm[k] == cell) { k0 = (long long)k; break; }
    const int p = ion->precision, ns = m->ns;
    y0.assign(size_t(ns), 0.0);
    for (int i = 0; i < ns; ++i) {
        const int w = m->wide_of[p * ns + i], s = m->slot_of[p * ns + i];
        if (w) {
            double v = 0.0;
            CFG_CUDA_TRY(cudaMemcpy(&v, ion->d_yw + size_t(s) * n + k0, sizeof v,
                                    cudaMemcpyDeviceToHost));
            if (p == CFG_PRECISION_MIXED) {
                float hl[2];
                std::memcpy(hl, &v, sizeof hl);
                v = double(hl[0]) + double(hl[1]);
            }
            y0[size_t(i)] = v;
        } else {
            float v = 0.0f;
            CFG_CUDA_TRY(cudaMemcpy(&v, ion->d_yn + size_t(s) * n + k0, sizeof v,
                                    cudaMemcpyDeviceToHost));
            y0[size_t(i)] = v;
        }
    }
    int tissue = ion->tissue;
    if (ion->d_tissue) {
        unsigned char t = 0;
        CFG_CUDA_TRY(cudaMemcpy(&t, ion->d_tissue + k0, 1, cudaMemcpyDeviceToHost));
        tissue = t;
    }
    double sc[6];
    const double* scp = nullptr;
    if (ion->d_scales) {
        for (int j = 0; j < 6; ++j)
            CFG_CUDA_TRY(cudaMemcpy(&sc[j], ion->d_scales + size_t(j) * n + k0, sizeof(double),
                                    cudaMemcpyDeviceToHost));
        scp = sc;
    }
    C.assign(size_t(m->nc), 0.0);
    std::vector<double> yinit(size_t(ns), 0.0);
    m->host_init(C.data(), yinit.data(), tissue, scp);
    *tissue_out = tissue;
    return CFG_OK;
}

// [states | algebraic | rates] of one cell at model time t (clamp = 0) or of
// a clamped-voltage sweep (clamp = 1, n_points rows).
int evaluate_rows(cfg_ionic* ion, const std::vector<double>& y0, const std::vector<double>& C,
                  int tissue, double vmin, double vmax, int n_points, double t, int clamp,
                  std::vector<double>& rows)
{
    const IonicModelOps* m = ion->ops;
    const int width = 2 * m->ns + m->na;
    double *d_y = nullptr, *d_c = nullptr, *d_out = nullptr;
    cudaError_t e = dmalloc(&d_y, y0.size());
    if (!e) e = dmalloc(&d_c, C.size());
    if (!e) e = dmalloc(&d_out, size_t(n_points) * width);
    if (!e) e = cudaMemcpy(d_y, y0.data(), sizeof(double) * y0.size(), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d_c, C.data(), sizeof(double) * C.size(), cudaMemcpyHostToDevice);
    if (!e) e = m->sweep(d_y, d_c, tissue, ion->solve_vm ? 1 : 0, ion->stim, vmin, vmax, n_points,
                         t, clamp, d_out, ion->stream);
    rows.assign(size_t(n_points) * width, 0.0);
    if (!e) e = cudaMemcpyAsync(rows.data(), d_out, sizeof(double) * rows.size(),
                                cudaMemcpyDeviceToHost, ion->stream);
    if (!e) e = cudaStreamSynchronize(ion->stream);
    dfree(d_y);
    dfree(d_c);
    dfree(d_out);
    if (e) return fail(CFG_ERR_CUDA, "variable evaluation failed: %s", cudaGetErrorString(e));
    return CFG_OK;
}

// ionicModelIO's write plan: Vm (transformed state 0), the other states,
// the algebraics, RATES_<state> (fullPlan, ionicModelIO.C:169-232), or the
// requested names that resolve (exportedFieldNamesRef: unknown names are
// ignored).  Column -1 is Vm.
std::vector<std::pair<std::string, int>> trace_plan(const IonicModelOps* m, const char* columns)
{
    std::vector<std::pair<std::string, int>> plan;
    if (!columns || !*columns) {
        plan.push_back({"Vm", -1});
        for (int s = 1; s < m->ns; ++s) plan.push_back({m->state_strings[s], s});
        for (int a = 0; a < m->na; ++a) plan.push_back({m->alg_strings[a], m->ns + a});
        for (int s = 0; s < m->ns; ++s)
            plan.push_back({std::string("RATES_") + m->state_strings[s], m->ns + m->na + s});
        return plan;
    }
    std::string cur;
    auto flush = [&]() {
        if (cur.empty()) return;
        int col = 0;
        if (cur == "Vm" || canonical_name(cur.c_str()) == "vm") plan.push_back({cur, -1});
        else if (resolve_column(m, cur, &col)) plan.push_back({cur, col});
        cur.clear();
    };
    for (const char* p = columns; *p; ++p) {
        if (*p == ' ' || *p == ',' || *p == '\t' || *p == '(' || *p == ')') flush();
        else cur.push_back(*p);
    }
    flush();
    return plan;
}

// getter of the transformed membrane potential (AlievPanfilov.H:78-81,
// BuenoOrovio.H:78-81; otherwise state 0)
double transformed_vm(int vm_map, double s0)
{
    if (vm_map == CFG_VM_ALIEV) return s0 * 100 - 80;
    if (vm_map == CFG_VM_BUENO) return s0 * 85.7 - 84.0;
    return s0;
}

}  // namespace
}  // namespace cfg

extern "C" {

int cfg_ionic_sweep_currents(const cfg_ionic* ion, char* buf, size_t len)
{
    if (!ion || !buf || !len) return fail(CFG_ERR_INVALID, "null argument");
    std::string s;
    for (const char* const* c = ion->ops->sweep_currents; *c; ++c) {
        if (!s.empty()) s += ' ';
        s += *c;
    }
    std::snprintf(buf, len, "%s", s.c_str());
    return CFG_OK;
}

int cfg_ionic_sweep_current(cfg_ionic* ion, const char* current, double v_min, double v_max,
                            int n_points, double* out, int* n_columns, char* header,
                            size_t header_len)
{
    if (!ion || !current) return fail(CFG_ERR_INVALID, "null argument");
    const IonicModelOps* m = ion->ops;
    const char* deps = nullptr;
    std::string avail;
    for (int k = 0; m->sweep_currents[k]; ++k) {
        if (!std::strcmp(m->sweep_currents[k], current)) deps = m->sweep_deps[k];
        avail += std::string(avail.empty() ? "" : " ") + m->sweep_currents[k];
    }
    if (!deps)
        return fail(CFG_ERR_INVALID, "Unknown current: %s\nAvailable currents: (%s)", current,
                    avail.c_str());
    const std::vector<std::string> names = split_commas(deps);
    std::vector<int> cols(names.size());
    for (size_t k = 0; k < names.size(); ++k)
        if (!resolve_column(m, names[k], &cols[k]))
            return fail(CFG_ERR_INVALID, "Unknown debug variable: %s. Expected Vm, one of the "
                        "STATE names, one of the ALGEBRAIC names, or a rate name of the form "
                        "RATES_<stateName>.", names[k].c_str());
    const int nc = 1 + int(names.size());
    if (n_columns) *n_columns = nc;
    if (header && header_len) {
        std::string h = "V";
        for (const std::string& s : names) h += "," + s;
        std::snprintf(header, header_len, "%s", h.c_str());
    }
    if (!out) return CFG_OK;
    if (n_points < 2) return fail(CFG_ERR_INVALID, "a sweep needs at least 2 points");

    // states of integration point 0 and the model's constants
    std::vector<double> y0, C, rows;
    int tissue = 0;
    if (int rc = cell_snapshot(ion, 0, y0, C, &tissue)) return rc;
    if (int rc = evaluate_rows(ion, y0, C, tissue, v_min, v_max, n_points, 0.0, 1, rows)) return rc;
    const int width = 2 * m->ns + m->na;
    for (int i = 0; i < n_points; ++i) {
        const double* row = &rows[size_t(i) * width];
        double* o = out + size_t(i) * nc;
        o[0] = row[0];
        for (size_t k = 0; k < cols.size(); ++k) o[1 + k] = row[cols[k]];
    }
    return CFG_OK;
}

int cfg_ionic_trace_header(const cfg_ionic* ion, const char* columns, char* buf, size_t len)
{
    if (!ion || !buf || !len) return fail(CFG_ERR_INVALID, "null argument");
    std::string h = "time";
    for (const auto& c : trace_plan(ion->ops, columns)) h += " " + c.first;
    h += "\n";
    if (h.size() + 1 > len) return fail(CFG_ERR_INVALID, "trace header needs %zu bytes", h.size() + 1);
    std::memcpy(buf, h.c_str(), h.size() + 1);
    return CFG_OK;
}

int cfg_ionic_trace_row(cfg_ionic* ion, long long cell, double t, const char* columns, char* buf,
                        size_t len)
{
    if (!ion || !buf || !len) return fail(CFG_ERR_INVALID, "null argument");
    if (cell < 0 || cell >= ion->n) return fail(CFG_ERR_INVALID, "cell %lld outside the model", cell);
    const IonicModelOps* m = ion->ops;
    std::vector<double> y0, C, rows;
    int tissue = 0;
    if (int rc = cell_snapshot(ion, cell, y0, C, &tissue)) return rc;
    // the variables of the last solveODE: computeVariables at tEnd, model time
    const double tm = m->time_scale == 1000.0 ? t : t * 1000.0 / m->time_scale;
    if (int rc = evaluate_rows(ion, y0, C, tissue, 0.0, 0.0, 1, tm, 0, rows)) return rc;
    // OFstream with std::ios::fixed and precision 7 (singleCellSolver.C:117-118)
    std::string r;
    char tmp[64];
    std::snprintf(tmp, sizeof tmp, "%.7f", t);
    r += tmp;
    for (const auto& c : trace_plan(m, columns)) {
        const double v = c.second < 0 ? transformed_vm(m->vm_map, rows[0]) : rows[size_t(c.second)];
        std::snprintf(tmp, sizeof tmp, " %.7f", v);
        r += tmp;
    }
    r += "\n";
    if (r.size() + 1 > len) return fail(CFG_ERR_INVALID, "trace row needs %zu bytes", r.size() + 1);
    std::memcpy(buf, r.c_str(), r.size() + 1);
    return CFG_OK;
}

}  // extern "C"
