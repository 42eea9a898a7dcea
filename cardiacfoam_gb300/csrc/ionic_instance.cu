// One ionic model in one precision form.  Compiled once per (model,
// precision) with -DCFG_MODEL=<namespace> -DCFG_FP64=<0|1>; the plain form is
// built with --fmad=false so FP64 rounding follows the host evaluation order.
#include <cuda_runtime.h>

#include "ionic_kernels.cuh"
#include "ionic_mixed.cuh"
#include "ionic_batch.cuh"

#define CFG_STR2(x) #x
#define CFG_STR(x) CFG_STR2(x)
#define CFG_CAT3_(a, b, c) a##b##c
#define CFG_CAT3(a, b, c) CFG_CAT3_(a, b, c)
#include CFG_STR(models/CFG_MODEL.cuh)

#if CFG_FP64
#define CFG_PREC_TAG _fp64
#else
#define CFG_PREC_TAG _mixed
#endif

using M = cfg::CFG_MODEL::Model;
static constexpr bool kFP64 = CFG_FP64 != 0;

using cfg::TissueList;
using Tissues = cfg::CFG_MODEL::TissueSet;

// The plain form runs ionic_step_kernel (one cell per thread, stage arrays
// per thread); the mixed form runs ionic_mixed_kernel (stage data in shared
// memory, block size fixed by the model's slice length).
// `block` threads per block (the plain form: at most 128; the mixed form:
// at most the model's slice block, 0 = that block) and p.cells_per_thread
// slots per thread; every slot's arithmetic is independent of both, so the
// results are too.
template <bool SV, int T>
static void launch_one(const cfg::IonicLaunch& p, cudaStream_t s, int block)
{
    const long long cpt = p.cells_per_thread > 0 ? p.cells_per_thread : 1;
    if constexpr (kFP64) {
        const int b = (block > 0 && block <= 128) ? block : 128;
        const unsigned grid = unsigned((p.count + b * cpt - 1) / (b * cpt));
        cfg::ionic_step_kernel<M, true, SV, T><<<grid, b, 0, s>>>(p);
    } else {
        using S = cfg::mixed::Slice<M>;
        const int b = (block > 0 && block <= S::block && block % 32 == 0) ? block : S::block;
        const unsigned grid = unsigned((p.count + b * cpt - 1) / (b * cpt));
        cfg::ionic_mixed_kernel<M, SV, T><<<grid, b, size_t(b) * S::len * 4, s>>>(p);
    }
}

extern "C" int CFG_CAT3(cfg_ionic_max_block_, CFG_MODEL, CFG_PREC_TAG)()
{
    if constexpr (kFP64) return 128;
    else return cfg::mixed::Slice<M>::block;
}

// Opt the mixed kernels into their dynamic shared memory (above the 48 KB
// default) on the current device; runs when a model is created, before any
// launch can be captured into a graph.
template <bool SV, int T>
static cudaError_t prepare_one()
{
    if constexpr (kFP64) {
        return cudaSuccess;
    } else {
        return cudaFuncSetAttribute(&cfg::ionic_mixed_kernel<M, SV, T>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    cfg::mixed::Slice<M>::smem_bytes);
    }
}

template <int... TS>
static cudaError_t prepare_all(TissueList<TS...>)
{
    cudaError_t e = prepare_one<true, 0>();
    if (e == cudaSuccess) e = prepare_one<false, 0>();
    cudaError_t r[] = {cudaSuccess, prepare_one<false, TS>()...};
    for (cudaError_t x : r)
        if (e == cudaSuccess) e = x;
    return e;
}

template <int T0, int... TR>
static bool launch_uniform(const cfg::IonicLaunch& p, cudaStream_t s, int block,
                           TissueList<T0, TR...>)
{
    if (p.tissue == T0) {
        launch_one<false, T0>(p, s, block);
        return true;
    }
    if constexpr (sizeof...(TR) > 0) return launch_uniform(p, s, block, TissueList<TR...>{});
    return false;
}

extern "C" cudaError_t CFG_CAT3(cfg_ionic_step_, CFG_MODEL, CFG_PREC_TAG)(
    const cfg::IonicLaunch& p, int solve_vm, cudaStream_t stream, int block)
{
    if (p.n <= 0 || p.count <= 0) return cudaSuccess;
    const bool uniform = !p.tissue_cell && !p.scales;
    if (solve_vm) {
        launch_one<true, 0>(p, stream, block);
    } else if (uniform && launch_uniform(p, stream, block, Tissues{})) {
        // tissue-specialised kernel launched
    } else {
        launch_one<false, 0>(p, stream, block);
    }
    return cudaGetLastError();
}

extern "C" cudaError_t CFG_CAT3(cfg_ionic_init_, CFG_MODEL, CFG_PREC_TAG)(
    long long n, int tissue, const unsigned char* tissue_cell, const double* scales,
    long long stride, double init_step, double* yw, float* yn, double* step,
    cudaStream_t stream)
{
    if (cudaError_t e = prepare_all(Tissues{})) return e;
    if (n <= 0) return cudaSuccess;
    const int block = 128;
    const unsigned grid = unsigned((n + block - 1) / block);
    cfg::ionic_init_kernel<M, kFP64><<<grid, block, 0, stream>>>(n, tissue, tissue_cell, scales,
                                                                stride, init_step, yw, yn, step);
    return cudaGetLastError();
}

#if CFG_FP64
// host-side initConsts of this model (compiled once, in the plain TU)
extern "C" void CFG_CAT3(cfg_ionic_host_init_, CFG_MODEL, )(double* C, double* y, int tissue,
                                                             const double* scale)
{
    M::init(C, y, tissue, scale);
}
#endif

// ---------------------------------------------------------------- batched single cells

template <int T>
static void* batch_kernel_ptr()
{
    if constexpr (kFP64) return reinterpret_cast<void*>(&cfg::batch_fp64_kernel<M, T>);
    else return reinterpret_cast<void*>(&cfg::batch_mixed_kernel<M, T>);
}

template <int T>
static cudaError_t batch_launch(const cfg::BatchLaunch& p, cudaStream_t s)
{
    int block, smem;
    if constexpr (kFP64) {
        block = 128;
        smem = 0;
    } else {
        block = cfg::mixed::Slice<M>::block;
        smem = cfg::mixed::Slice<M>::smem_bytes;
    }
    // persistent grid: every block resident, cells handed out by the queue
    static int per_sm = 0, sms = 0;
    if (!per_sm) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (!e) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel_ptr<T>(),
                                                                  block, smem);
        if (e) return e;
        if (per_sm < 1) per_sm = 1;
    }
    const long long want = (p.n + block - 1) / block;
    const long long cap = (long long)sms * per_sm;
    const unsigned grid = unsigned(want < cap ? want : cap);
    if constexpr (kFP64) cfg::batch_fp64_kernel<M, T><<<grid, block, 0, s>>>(p);
    else cfg::batch_mixed_kernel<M, T><<<grid, block, smem, s>>>(p);
    return cudaGetLastError();
}

template <int T0, int... TR>
static cudaError_t batch_dispatch(const cfg::BatchLaunch& p, int tissue, cudaStream_t s,
                                  TissueList<T0, TR...>)
{
    if (tissue == T0) return batch_launch<T0>(p, s);
    if constexpr (sizeof...(TR) > 0) return batch_dispatch(p, tissue, s, TissueList<TR...>{});
    return cudaErrorInvalidValue;
}

template <int... TS>
static cudaError_t batch_prepare(TissueList<TS...>)
{
    if constexpr (kFP64) {
        return cudaSuccess;
    } else {
        cudaError_t r[] = {cudaSuccess,
                           cudaFuncSetAttribute(&cfg::batch_mixed_kernel<M, TS>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                cfg::mixed::Slice<M>::smem_bytes)...};
        for (cudaError_t x : r)
            if (x) return x;
        return cudaSuccess;
    }
}

extern "C" cudaError_t CFG_CAT3(cfg_batch_init_, CFG_MODEL, CFG_PREC_TAG)(
    const cfg::BatchLaunch& p, const double* scales, int tissue, double init_step,
    cudaStream_t stream)
{
    if (cudaError_t e = batch_prepare(Tissues{})) return e;
    if (p.n <= 0) return cudaSuccess;
    const int block = 128;
    const unsigned grid = unsigned((p.n + block - 1) / block);
    cfg::batch_init_kernel<M, kFP64><<<grid, block, 0, stream>>>(p, scales, tissue, init_step);
    return cudaGetLastError();
}

extern "C" cudaError_t CFG_CAT3(cfg_batch_step_, CFG_MODEL, CFG_PREC_TAG)(
    const cfg::BatchLaunch& p, int tissue, cudaStream_t stream)
{
    if (p.n <= 0) return cudaSuccess;
    return batch_dispatch(p, tissue, stream, Tissues{});
}

#if CFG_FP64
// ---------------------------------------------------------------- sweepCurrent
// <Model>::sweepCurrent (e.g. TNNP.C:208-272): the states of one cell with
// state 0 clamped to V = vmin + (vmax - vmin) i / (npts - 1), the first
// variables function at VOI = 0, one thread per voltage.  Row i of `out` is
// [states | algebraic | rates] (2 NS + NA doubles).
// With clamp = 0 the states are taken as they are (one row: the variables
// of a cell at model time t, as a trace row of ionicModelIO::write holds).
template <bool SV>
__global__ void sweep_kernel(const double* y0, const double* C, int tissue, cfg::CfgStimulus stim,
                             double vmin, double vmax, int npts, double t, int clamp, double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npts) return;
    constexpr int NS = M::NS, NA = M::NA;
    double y[NS];
    for (int k = 0; k < NS; ++k) y[k] = y0[k];
    if (clamp) {
        const double denom = double(npts - 1);
        y[0] = vmin + (vmax - vmin) * double(i) / denom;
    }
    double A[NA > 0 ? NA : 1] = {};
    double R[NS] = {};
    const cfg::ConstView<double> K{C};
    M::template all_variables<double, SV>(t, cfg::ArrayView<double>{y}, K, A, R, tissue, stim);
    double* row = out + (long long)i * (2 * NS + NA);
    for (int k = 0; k < NS; ++k) row[k] = y[k];
    for (int k = 0; k < NA; ++k) row[NS + k] = A[k];
    for (int k = 0; k < NS; ++k) row[NS + NA + k] = R[k];
}

extern "C" cudaError_t CFG_CAT3(cfg_ionic_sweep_, CFG_MODEL, )(
    const double* y0, const double* C, int tissue, int solve_vm, const cfg::CfgStimulus& stim,
    double vmin, double vmax, int npts, double t, int clamp, double* out, cudaStream_t s)
{
    if (npts <= 0) return cudaSuccess;
    const int block = 64;
    const unsigned grid = unsigned((npts + block - 1) / block);
    if (solve_vm)
        sweep_kernel<true><<<grid, block, 0, s>>>(y0, C, tissue, stim, vmin, vmax, npts, t, clamp,
                                                  out);
    else
        sweep_kernel<false><<<grid, block, 0, s>>>(y0, C, tissue, stim, vmin, vmax, npts, t, clamp,
                                                   out);
    return cudaGetLastError();
}
#endif
