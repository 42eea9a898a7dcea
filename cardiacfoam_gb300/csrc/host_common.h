// Host-side helpers shared by the C-ABI implementation files.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/cardiac_gpu.h"

namespace cfg {

// Record the message of a failure for cfg_last_error() and return `code`.
int fail(int code, const char* fmt, ...);
void clear_error();

// tissue key -> flag (ionicSelector::tissueFlag, ionicSelector.C:56-63)
int tissue_flag(const char* name);

#define CFG_CUDA_TRY(expr)                                                                    \
    do {                                                                                      \
        cudaError_t e_ = (expr);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return ::cfg::fail(CFG_ERR_CUDA, "%s failed: %s (%s:%d)", #expr,                  \
                               cudaGetErrorString(e_), __FILE__, __LINE__);                   \
    } while (0)

template <class T>
cudaError_t dmalloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
}

template <class T>
void dfree(T*& p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

}  // namespace cfg
