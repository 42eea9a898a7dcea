// Grid-wide synchronisation and deterministic reductions for persistent
// cooperative kernels (every block resident).  A barrier counts arrivals on a
// monotonic counter that the caller resets before the launch, and its spin
// is bounded: a block that waits longer than the spin limit (by default
// about a second) sets an abort flag and every block leaves at its next
// barrier.
#pragma once

#include <cuda_runtime.h>

#include "float_pair.cuh"

namespace cfg {
namespace gsync {

constexpr long long kSpinLimit = 1LL << 25;   // x >= 32 ns per spin: about a second

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_relaxed_int(const int* p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// count += 1 with release semantics at GPU scope: the block's writes, made
// visible to thread 0 by the block barrier before it, are visible to any
// thread whose acquire load reads this arrival or a later one
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

// Each block adds one arrival and waits until all gridDim.x arrivals of this
// barrier are in; `epoch` counts the arrivals expected so far.  The arrival
// is a release and the wait an acquire on the same counter, which orders the
// blocks' writes before the barrier against their reads after it without a
// full fence.  Returns false when the launch was aborted (some block waited
// more than `spin_limit` spins).
__device__ __forceinline__ bool grid_barrier(unsigned* count, int* abort, unsigned& epoch,
                                             long long spin_limit = kSpinLimit)
{
    __shared__ int ok;
    epoch += gridDim.x;
    __syncthreads();
    if (threadIdx.x == 0) {
        red_release_add(count, 1u);
        int good = 1;
        long long spins = 0;
        while (ld_acquire(count) < epoch) {
            if (ld_relaxed_int(abort)) { good = 0; break; }
            if (++spins > spin_limit) {
                atomicExch(abort, 1);
                good = 0;
                break;
            }
            // short waits spin; long ones back off (a waiting block then
            // polls L2 less often)
            if (spins > 4096) __nanosleep(64);
        }
        if (ld_relaxed_int(abort)) good = 0;
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Block sums of K per-thread values into partial[set][k][blockIdx.x]
// (sets of two slots, alternated between consecutive reductions).
template <int kBlock, int K>
__device__ __forceinline__ void block_sums(double* partial, int set, double (&v)[K])
{
    constexpr int kWarps = kBlock / 32;
    __shared__ double sh[K][kWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = v[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) sh[k][w] = s;
    }
    __syncthreads();
    if (threadIdx.x < 32 * K && (threadIdx.x & 31) == 0) {
        const int k = threadIdx.x >> 5;
        double s = 0.0;
        for (int j = 0; j < kWarps; ++j) s += sh[k][j];
        __stcg(&partial[(size_t(set) * 2 + k) * gridDim.x + blockIdx.x], s);
    }
}

// Sum of partial[set][k][0..gridDim.x) in a fixed order; every block gets
// the same value.  Called after a grid barrier, by all threads.
template <int K>
__device__ __forceinline__ void grid_sums(const double* partial, int set, double (&out)[K])
{
    __shared__ double sh[K];
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const double* src = partial + (size_t(set) * 2 + k) * gridDim.x;
            double s = 0.0;
            for (unsigned i = threadIdx.x; i < gridDim.x; i += 32) s += __ldcg(&src[i]);
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (threadIdx.x == 0) sh[k] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = sh[k];
    __syncthreads();
}

// K scalars derived from reduction results (ratios of sums), computed by
// thread 0 and read by every thread of the block.  Every thread holds the
// same sums, so every block gets the same values; doing the arithmetic once
// per block instead of once per thread matters because an FP64 division is a
// few tens of instructions on GB300's FP64 pipe, which the row work shares.
template <int K, class F>
__device__ __forceinline__ void block_scalars(double (&out)[K], F f)
{
    __shared__ double v[K];
    if (threadIdx.x == 0) f(v);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = v[k];
    __syncthreads();   // v is written again by the next call
}

// Float-pair forms of block_sums / grid_sums (partial slots of 8 bytes hold
// one pair; a set has S slots of gridDim.x, so a kernel whose reductions
// alternate between two sets needs 2 S gridDim.x pairs).  Warp k adds the
// block's warp sums of value k in a fixed tree; every block then adds the
// block sums in the same fixed order, so all blocks hold bitwise the same
// totals.
template <int kBlock, int K, int S = 2>
__device__ __forceinline__ void block_sums_pair(float2* partial, int set, fp::P (&v)[K])
{
    constexpr int kWarps = kBlock / 32;
    static_assert(kWarps <= 32 && K <= kWarps && K <= S, "one warp per value");
    __shared__ float2 sh[K][kWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const fp::P s = fp::warp_sum(v[k]);
        if (lane == 0) sh[k][w] = s;
    }
    __syncthreads();
    if (w < K) {
        fp::P s = lane < kWarps ? sh[w][lane] : fp::make(0.0f);
        s = fp::warp_sum(s);
        if (lane == 0) __stcg(&partial[(size_t(set) * S + w) * gridDim.x + blockIdx.x], s);
    }
}

template <int K, int S = 2>
__device__ __forceinline__ void grid_sums_pair(const float2* partial, int set, fp::P (&out)[K])
{
    __shared__ float2 sh[K];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (w < K) {
        const float2* src = partial + (size_t(set) * S + w) * gridDim.x;
        fp::P s = fp::make(0.0f);
        for (unsigned i = lane; i < gridDim.x; i += 32) s = fp::add(s, __ldcg(&src[i]));
        s = fp::warp_sum(s);
        if (lane == 0) sh[w] = s;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = sh[k];
    __syncthreads();
}

}  // namespace gsync
}  // namespace cfg
