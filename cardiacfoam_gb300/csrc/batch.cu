// Host side of the batched single-cell solver: buffers, the launch loop of
// the work-stealing kernels and the C ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "host_common.h"
#include "ionic_host.h"

struct cfg_batch {
    const cfg::IonicModelOps* ops = nullptr;
    long long n = 0;
    int precision = CFG_PRECISION_FP64;
    int tissue = 0;
    double dt = 0.0;
    cfg::BatchLaunch L{};
    long long total_steps = 0;
    long long launches = 0;
    cudaStream_t stream = nullptr;
    // device buffers
    cfg::CfgStimulus* d_stim = nullptr;
    long long *d_n_steps = nullptr, *d_done = nullptr, *d_active = nullptr;
    double *d_t = nullptr, *d_yw = nullptr, *d_step = nullptr, *d_dep = nullptr;
    float* d_yn = nullptr;
    cfg::ApdTracker* d_apd = nullptr;
    double *d_ring_t = nullptr, *d_ring_v = nullptr, *d_trace = nullptr, *d_scales = nullptr;
    double* d_fail = nullptr;
    unsigned long long *d_queue = nullptr, *d_evals = nullptr;
    int* d_status = nullptr;
};

namespace cfg {
namespace {

void batch_free(cfg_batch* b)
{
    if (!b) return;
    dfree(b->d_stim); dfree(b->d_n_steps); dfree(b->d_done); dfree(b->d_active);
    dfree(b->d_t); dfree(b->d_yw); dfree(b->d_step); dfree(b->d_dep); dfree(b->d_yn);
    dfree(b->d_apd); dfree(b->d_ring_t); dfree(b->d_ring_v); dfree(b->d_trace);
    dfree(b->d_scales); dfree(b->d_fail); dfree(b->d_queue); dfree(b->d_evals);
    dfree(b->d_status);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int batch_create(const cfg_batch_desc* d, cfg_batch** out)
{
    if (!d || !out) return fail(CFG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (d->n_cells <= 0) return fail(CFG_ERR_INVALID, "no cells");
    if (!d->stimulus || !d->end_time)
        return fail(CFG_ERR_INVALID, "stimulus and end_time are required");
    if (!(d->delta_t > 0)) return fail(CFG_ERR_INVALID, "deltaT must be positive");
    const ApdParams apdp = apd_defaults(d->delta_t);
    if (apdp.ring > 4096)
        return fail(CFG_ERR_UNSUPPORTED, "deltaT %g s leaves %d samples in the 2 ms APD baseline "
                    "window (at most 4096 are kept)", d->delta_t, apdp.ring);
    if (d->trace_cells < 0 || d->trace_samples < 0 || d->trace_cells > d->n_cells)
        return fail(CFG_ERR_INVALID, "bad trace size");
    // model, tissue and ODE settings through the ionic model's own checks
    cfg_ionic_desc id{};
    id.ionic_model = d->ionic_model;
    id.tissue = d->tissue;
    id.n_cells = d->n_cells;
    id.initial_delta_t = d->delta_t;
    id.solve_vm_within_ode = 1;
    id.precision = d->precision;
    id.ode = d->ode;
    id.stimulus = d->stimulus[0];
    id.scales = d->scales;
    const IonicModelOps* ops = nullptr;
    int tissue = 0;
    if (int rc = ionic_validate(&id, &ops, &tissue)) return rc;
    if (d->precision != CFG_PRECISION_FP64 && d->precision != CFG_PRECISION_MIXED)
        return fail(CFG_ERR_INVALID, "unknown precision %d", d->precision);
    // per-cell protocol and length: runTime runs deltaT steps to endTime
    const long long n = d->n_cells;
    std::vector<CfgStimulus> stim(static_cast<size_t>(n));
    std::vector<long long> steps(static_cast<size_t>(n));
    long long total = 0, with_work = 0;
    for (long long c = 0; c < n; ++c) {
        const cfg_stimulus_desc& s = d->stimulus[c];
        stim[size_t(c)] = CfgStimulus{s.stim_start, s.stim_period_s1, s.stim_duration,
                                      s.stim_amplitude, s.nstim1, s.stim_period_s2, s.nstim2};
        if (!(d->end_time[c] >= 0))
            return fail(CFG_ERR_INVALID, "cell %lld: negative end time", c);
        steps[size_t(c)] = (long long)std::llround(d->end_time[c] / d->delta_t);
        total += steps[size_t(c)];
        with_work += steps[size_t(c)] > 0 ? 1 : 0;
    }

    cfg_batch* b = new cfg_batch;
    b->ops = ops;
    b->n = n;
    b->precision = d->precision;
    b->tissue = tissue;
    b->dt = d->delta_t;
    b->total_steps = total;
    const int p = d->precision;
    const int nw = ops->n_wide[p], nn = ops->ns - nw;
    auto bail = [&](int rc) { batch_free(b); return rc; };
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (!e) e = dmalloc(&b->d_stim, size_t(n));
    if (!e) e = dmalloc(&b->d_n_steps, size_t(n));
    if (!e) e = dmalloc(&b->d_done, size_t(n));
    if (!e) e = dmalloc(&b->d_active, 1);
    if (!e) e = dmalloc(&b->d_t, size_t(n));
    if (!e) e = dmalloc(&b->d_yw, size_t(nw) * n);
    if (!e && nn) e = dmalloc(&b->d_yn, size_t(nn) * n);
    if (!e) e = dmalloc(&b->d_step, size_t(n));
    if (!e && ops->nsd) e = dmalloc(&b->d_dep, size_t(ops->nsd) * n);
    if (!e) e = dmalloc(&b->d_apd, size_t(n));
    if (!e) e = dmalloc(&b->d_ring_t, size_t(apdp.ring) * n);
    if (!e) e = dmalloc(&b->d_ring_v, size_t(apdp.ring) * n);
    if (!e && d->trace_cells && d->trace_samples)
        e = dmalloc(&b->d_trace, size_t(2) * d->trace_cells * d->trace_samples);
    if (!e && d->scales) e = dmalloc(&b->d_scales, size_t(6) * n);
    if (!e) e = dmalloc(&b->d_fail, 8);
    if (!e) e = dmalloc(&b->d_queue, 1);
    if (!e) e = dmalloc(&b->d_evals, 1);
    if (!e) e = dmalloc(&b->d_status, 1);
    if (e) return bail(fail(CFG_ERR_CUDA, "device allocation failed: %s", cudaGetErrorString(e)));
    e = cudaMemcpy(b->d_stim, stim.data(), sizeof(CfgStimulus) * n, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(b->d_n_steps, steps.data(), sizeof(long long) * n, cudaMemcpyHostToDevice);
    if (!e && d->scales)
        e = cudaMemcpy(b->d_scales, d->scales, sizeof(double) * 6 * n, cudaMemcpyHostToDevice);
    const long long active = with_work;   // zero-length cells are done at set-up
    if (!e) e = cudaMemcpy(b->d_active, &active, sizeof active, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemset(b->d_evals, 0, sizeof(unsigned long long));
    if (!e) e = cudaMemset(b->d_status, 0, sizeof(int));
    if (!e) e = cudaMemset(b->d_fail, 0, 8 * sizeof(double));
    if (!e && b->d_trace)   // NaN where no sample was written
        e = cudaMemset(b->d_trace, 0xff, sizeof(double) * 2 * d->trace_cells * d->trace_samples);
    if (e) return bail(fail(CFG_ERR_CUDA, "device initialisation failed: %s", cudaGetErrorString(e)));

    BatchLaunch& L = b->L;
    L.n = n;
    L.dt = d->delta_t;
    L.chunk = d->chunk > 0 ? d->chunk : 2000;
    L.ode = make_ode(d->ode);
    L.stim = b->d_stim;
    L.n_steps = b->d_n_steps;
    L.done = b->d_done;
    L.t = b->d_t;
    L.yw = b->d_yw;
    L.yn = b->d_yn;
    L.step = b->d_step;
    L.dep = b->d_dep;
    L.apd = b->d_apd;
    L.ring_t = b->d_ring_t;
    L.ring_v = b->d_ring_v;
    L.apdp = apdp;
    L.trace = b->d_trace;
    L.trace_cells = b->d_trace ? d->trace_cells : 0;
    L.trace_cap = b->d_trace ? d->trace_samples : 0;
    L.queue = b->d_queue;
    L.active = b->d_active;
    L.status = b->d_status;
    L.rhs_evals = b->d_evals;
    L.fail_record = b->d_fail;
    // initConsts per cell; the first ODE step is initialDeltaT taken as a
    // model-time value, as ionicModel's step_ (ionicModel.C:35-38)
    e = ops->batch_init[p](L, b->d_scales, tissue, d->delta_t, b->stream);
    if (!e) e = cudaStreamSynchronize(b->stream);
    if (e) return bail(fail(CFG_ERR_CUDA, "batch set-up failed: %s", cudaGetErrorString(e)));
    *out = b;
    return CFG_OK;
}

int batch_check(cfg_batch* b)
{
    int st = 0;
    CFG_CUDA_TRY(cudaMemcpy(&st, b->d_status, sizeof st, cudaMemcpyDeviceToHost));
    if (st & CFG_ERR_ODE_STEPS) {
        double r[8];
        CFG_CUDA_TRY(cudaMemcpy(r, b->d_fail, sizeof r, cudaMemcpyDeviceToHost));
        const int worst = int(r[4]);
        return fail(CFG_ERR_ODE_STEPS,
                    "%s: cell %lld: %s at x = %.17g, dx = %.6g after %lld substeps; worst state "
                    "%s = %.9g with normalised error %.6g",
                    b->ops->name, (long long)r[0],
                    r[1] == 2 ? "stepsize underflow" : "Integration steps greater than maximum",
                    r[2], r[3], (long long)r[7],
                    worst >= 0 && worst < b->ops->ns ? b->ops->state_names[worst] : "?", r[6],
                    r[5]);
    }
    return CFG_OK;
}

}  // namespace
}  // namespace cfg

using namespace cfg;

extern "C" {

int cfg_batch_create(const cfg_batch_desc* desc, cfg_batch** out)
{
    clear_error();
    return batch_create(desc, out);
}

int cfg_batch_run(cfg_batch* b)
{
    if (!b) return fail(CFG_ERR_INVALID, "null batch");
    // each launch hands every cell out once and advances it by up to `chunk`
    // steps, so the longest remaining cell bounds the number of launches
    long long max_steps = 0;
    {
        std::vector<long long> steps(static_cast<size_t>(b->n)), done(static_cast<size_t>(b->n));
        CFG_CUDA_TRY(cudaMemcpy(steps.data(), b->L.n_steps, sizeof(long long) * b->n,
                                cudaMemcpyDeviceToHost));
        CFG_CUDA_TRY(cudaMemcpy(done.data(), b->L.done, sizeof(long long) * b->n,
                                cudaMemcpyDeviceToHost));
        for (long long c = 0; c < b->n; ++c)
            max_steps = std::max(max_steps, steps[size_t(c)] - done[size_t(c)]);
    }
    const long long bound = (max_steps + b->L.chunk - 1) / b->L.chunk + 1;
    for (long long k = 0; k < bound; ++k) {
        long long active = 0;
        CFG_CUDA_TRY(cudaMemcpyAsync(&active, b->d_active, sizeof active, cudaMemcpyDeviceToHost,
                                     b->stream));
        CFG_CUDA_TRY(cudaStreamSynchronize(b->stream));
        if (active <= 0) break;
        CFG_CUDA_TRY(cudaMemsetAsync(b->d_queue, 0, sizeof(unsigned long long), b->stream));
        CFG_CUDA_TRY(b->ops->batch_step[b->precision](b->L, b->tissue, b->stream));
        b->launches += 1;
    }
    CFG_CUDA_TRY(cudaStreamSynchronize(b->stream));
    if (int rc = batch_check(b)) return rc;
    long long active = 0;
    CFG_CUDA_TRY(cudaMemcpy(&active, b->d_active, sizeof active, cudaMemcpyDeviceToHost));
    if (active > 0) return fail(CFG_ERR_CUDA, "%lld cells did not finish", active);
    return CFG_OK;
}

int cfg_batch_results(cfg_batch* b, int* n_beats, double* apd90_ms, double* t_up,
                      double* peak_ca)
{
    if (!b) return fail(CFG_ERR_INVALID, "null batch");
    std::vector<ApdTracker> a(static_cast<size_t>(b->n));
    CFG_CUDA_TRY(cudaMemcpy(a.data(), b->d_apd, sizeof(ApdTracker) * b->n, cudaMemcpyDeviceToHost));
    for (long long c = 0; c < b->n; ++c) {
        const ApdTracker& t = a[size_t(c)];
        if (n_beats) n_beats[c] = t.n_beats;
        if (apd90_ms) apd90_ms[c] = t.last_apd * 1000.0;
        if (t_up) t_up[c] = t.last_t_up;
        if (peak_ca) peak_ca[c] = t.last_ca;
    }
    return CFG_OK;
}

int cfg_batch_trace(cfg_batch* b, double* host)
{
    if (!b || !host) return fail(CFG_ERR_INVALID, "null argument");
    if (!b->d_trace) return fail(CFG_ERR_INVALID, "no traces were requested");
    CFG_CUDA_TRY(cudaMemcpy(host, b->d_trace,
                            sizeof(double) * 2 * b->L.trace_cells * b->L.trace_cap,
                            cudaMemcpyDeviceToHost));
    return CFG_OK;
}

int cfg_batch_get_states(cfg_batch* b, double* host)
{
    if (!b || !host) return fail(CFG_ERR_INVALID, "null argument");
    const long long n = b->n;
    const int p = b->precision, ns = b->ops->ns;
    std::vector<double> wide(size_t(b->ops->n_wide[p]) * n);
    std::vector<float> narrow(size_t(ns - b->ops->n_wide[p]) * n);
    CFG_CUDA_TRY(cudaMemcpy(wide.data(), b->d_yw, sizeof(double) * wide.size(),
                            cudaMemcpyDeviceToHost));
    if (!narrow.empty())
        CFG_CUDA_TRY(cudaMemcpy(narrow.data(), b->d_yn, sizeof(float) * narrow.size(),
                                cudaMemcpyDeviceToHost));
    for (int i = 0; i < ns; ++i) {
        const int w = b->ops->wide_of[p * ns + i], s = b->ops->slot_of[p * ns + i];
        for (long long c = 0; c < n; ++c) {
            double v;
            if (w && p == CFG_PRECISION_MIXED) {
                float hl[2];
                std::memcpy(hl, &wide[size_t(s) * n + c], sizeof hl);
                v = double(hl[0]) + double(hl[1]);
            } else if (w) {
                v = wide[size_t(s) * n + c];
            } else {
                v = narrow[size_t(s) * n + c];
            }
            host[size_t(i) * n + c] = v;
        }
    }
    return CFG_OK;
}

int cfg_batch_stats(const cfg_batch* b, unsigned long long* rhs_evaluations,
                    long long* solver_steps, long long* launches)
{
    if (!b) return fail(CFG_ERR_INVALID, "null batch");
    if (rhs_evaluations)
        CFG_CUDA_TRY(cudaMemcpy(rhs_evaluations, b->d_evals, sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost));
    if (solver_steps) {
        std::vector<long long> done(static_cast<size_t>(b->n));
        CFG_CUDA_TRY(cudaMemcpy(done.data(), b->d_done, sizeof(long long) * b->n,
                                cudaMemcpyDeviceToHost));
        long long s = 0;
        for (long long v : done) s += v;
        *solver_steps = s;
    }
    if (launches) *launches = b->launches;
    return CFG_OK;
}

void* cfg_batch_stream(cfg_batch* b) { return b ? static_cast<void*>(b->stream) : nullptr; }

int cfg_batch_destroy(cfg_batch* b)
{
    batch_free(b);
    return CFG_OK;
}

}  // extern "C"
