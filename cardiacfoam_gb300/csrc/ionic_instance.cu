// One ionic model in one precision form.  Compiled once per (model,
// precision) with -DCFG_MODEL=<namespace> -DCFG_FP64=<0|1>; the plain form is
// built with --fmad=false so FP64 rounding follows the host evaluation order.
#include <cuda_runtime.h>

#include "ionic_kernels.cuh"

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

template <int T0, int... TR>
static bool launch_uniform(const cfg::IonicLaunch& p, cudaStream_t s, unsigned grid, int block,
                           TissueList<T0, TR...>)
{
    if (p.tissue == T0) {
        cfg::ionic_step_kernel<M, kFP64, false, T0><<<grid, block, 0, s>>>(p);
        return true;
    }
    if constexpr (sizeof...(TR) > 0) return launch_uniform(p, s, grid, block, TissueList<TR...>{});
    return false;
}

extern "C" cudaError_t CFG_CAT3(cfg_ionic_step_, CFG_MODEL, CFG_PREC_TAG)(
    const cfg::IonicLaunch& p, int solve_vm, cudaStream_t stream, int block)
{
    if (p.n <= 0) return cudaSuccess;
    const unsigned grid = unsigned((p.n + block - 1) / block);
    const bool uniform = !p.tissue_cell && !p.scales;
    if (solve_vm) {
        cfg::ionic_step_kernel<M, kFP64, true, 0><<<grid, block, 0, stream>>>(p);
    } else if (uniform && launch_uniform(p, stream, grid, block, Tissues{})) {
        // tissue-specialised kernel launched
    } else {
        cfg::ionic_step_kernel<M, kFP64, false, 0><<<grid, block, 0, stream>>>(p);
    }
    return cudaGetLastError();
}

extern "C" cudaError_t CFG_CAT3(cfg_ionic_init_, CFG_MODEL, CFG_PREC_TAG)(
    long long n, int tissue, const unsigned char* tissue_cell, const double* scales,
    long long stride, double init_step, double* yw, float* yn, double* step,
    cudaStream_t stream)
{
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
