// Pseudo-ECG (PseudoECGSolver::compute, pseudoECGSolver.C:34-87) on the GPU.
//
//   phi(P_e) = sum_c ((sigma_c grad(Vm)_c) V_c) . r_ec / |r_ec|^3,  r_ec = C_c - P_e
//
// The gradient is linear in Vm (fvc::grad with zeroGradient walls) and the
// mesh, the conductivity and the electrodes do not change during a run, so
// phi is a fixed linear functional of Vm.  Creation folds the gradient
// scheme's per-face weights and each cell's dipole geometry
// z_ec = V_c sigma_c r_ec / |r_ec|^3 into one lead row L[e][0..n) per
// electrode; an evaluation is phi_e = sum_c L[e][c] Vm_c, one streaming
// pass over the rows (8 bytes per cell and electrode) and over Vm, bound by
// HBM bandwidth.  Block partial sums are combined in block order by the
// last block to finish, so the values do not depend on scheduling.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "geometry.h"
#include "host_common.h"
#include "monodomain_host.h"

namespace {

constexpr int kEcgBlock = 256;
constexpr int kEcgChunk = 8;      // electrodes of one launch
constexpr int kEcgBlocksPerSm = 8;
#ifndef CFG_ECG_TILE
#define CFG_ECG_TILE 2048
#endif
#ifndef CFG_ECG_STAGED_PER_SM
#define CFG_ECG_STAGED_PER_SM 1
#endif
constexpr int kTile = CFG_ECG_TILE;             // cells per tile (a multiple of 2 * kEcgBlock)
// Tile of a launch of ne electrodes: kTile while two stages of Vm and ne rows
// fit in 216 KB of shared memory, else half of it.
constexpr int tile_of(int ne)
{
    return 2 * (ne + 1) * kTile * 8 <= 216 * 1024 ? kTile : kTile / 2;
}
constexpr int kStagedPerSm = CFG_ECG_STAGED_PER_SM;
constexpr int kMaxStages = 8;
static_assert(kTile % (4 * kEcgBlock) == 0, "a tile is whole pairs of cells per thread");

struct EcgArgs {
    const void* lead;     // tile-blocked rows (below): doubles, or (hi, lo) float pairs
    const double* scale;  // pairs: the power of two each row was scaled by
    const double* vm;     // [n]
    long long n, ld;      // cells; row length padded with zeros to whole tiles
    int n_el, e0;         // all electrodes; the first of this launch
    double* partial;      // [gridDim.x][n_el]
    unsigned* ticket;     // this launch's
    double* out;          // [n_el]
    long long wait_cycles;  // staged form: clock cycles a copy wait may take
};

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Accumulators: FP64 multiply-add, or a float pair (ch + cl) fed by the
// error-free product of two float pairs (Dekker's product with fmaf for the
// rounding error, the low-order cross terms added into it) and Knuth's
// two-sum; the rounded operations are the _rn intrinsics so that no
// multiply-add contraction changes them.
template <bool PAIR>
struct Acc;

template <>
struct Acc<false> {
    double a = 0.0;
    __device__ __forceinline__ void add(double l, double v) { a = fma(l, v, a); }
    __device__ __forceinline__ double value() const { return a; }
    static __device__ __forceinline__ Acc nan()
    {
        Acc r;
        r.a = __longlong_as_double(0x7ff8000000000000LL);
        return r;
    }
};

template <>
struct Acc<true> {
    float h = 0.0f, l = 0.0f;
    __device__ __forceinline__ void add(float2 a, float bh, float bl)
    {
        const float p = __fmul_rn(a.x, bh);
        float e = fmaf(a.x, bh, -p);
        e = fmaf(a.x, bl, e);
        e = fmaf(a.y, bh, e);
        const float s = __fadd_rn(h, p);
        const float z = __fsub_rn(s, h);
        const float t = __fadd_rn(__fsub_rn(h, __fsub_rn(s, z)), __fsub_rn(p, z));
        l = __fadd_rn(l, __fadd_rn(t, e));
        h = s;
    }
    __device__ __forceinline__ void renormalize()
    {
        const float s = __fadd_rn(h, l);
        l = __fsub_rn(l, __fsub_rn(s, h));
        h = s;
    }
    __device__ __forceinline__ double value() const { return double(h) + double(l); }
    static __device__ __forceinline__ Acc nan()
    {
        Acc r;
        r.h = __uint_as_float(0x7fc00000u);
        return r;
    }
};

// Adds the block's sums to the partial sums and, in the last block to
// finish, the blocks' sums in block order into out (divided by the row
// scale for pairs).
template <int NE, bool PAIR>
__device__ __forceinline__ void finish(const EcgArgs& a, const Acc<PAIR> (&acc)[NE],
                                       double (&red)[kEcgBlock / 32][NE], bool& last)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double sum[NE];
#pragma unroll
    for (int j = 0; j < NE; ++j) sum[j] = warp_sum(acc[j].value());
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < NE; ++j) red[warp][j] = sum[j];
    __syncthreads();
    if (threadIdx.x < NE) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kEcgBlock / 32; ++w) s += red[w][threadIdx.x];
        a.partial[(long long)blockIdx.x * a.n_el + a.e0 + threadIdx.x] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(a.ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int e = warp; e < NE; e += kEcgBlock / 32) {
        double s = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32)
            s += __ldcg(&a.partial[(long long)b * a.n_el + a.e0 + e]);
        s = warp_sum(s);
        if (lane == 0) a.out[a.e0 + e] = PAIR ? s / a.scale[a.e0 + e] : s;
    }
    if (threadIdx.x == 0) *a.ticket = 0u;
}

// One cell's terms: entry l of each row, Vm value v.
// Rows of one launch's NE electrodes are stored tile-blocked: tile t of
// T = tile_of(NE) cells holds row 0's T entries, then row 1's, ..., so that
// a tile of all NE rows is one contiguous block (one bulk copy).  Entry
// (j, c) is at (c / T) NE T + j T + c % T.
template <int NE, bool PAIR, class Entry>
__device__ __forceinline__ void cell_terms(Acc<PAIR> (&acc)[NE], const Entry* lead, long long c,
                                           double v)
{
    constexpr int T = tile_of(NE);
    const Entry* e = lead + (c / T) * NE * T + c % T;
    if constexpr (PAIR) {
        // Vm as a float pair from its bit pattern (no FP64 operation)
        const float2 vp = cfg::fp::split(v);
#pragma unroll
        for (int j = 0; j < NE; ++j) acc[j].add(e[j * T], vp.x, vp.y);
    } else {
#pragma unroll
        for (int j = 0; j < NE; ++j) acc[j].add(e[j * T], v);
    }
}

template <int NE, bool PAIR>
__device__ __forceinline__ void renormalize(Acc<PAIR> (&acc)[NE])
{
    if constexpr (PAIR) {
#pragma unroll
        for (int j = 0; j < NE; ++j) acc[j].renormalize();
    }
}

// Grid-stride form, one cell per load: for a Vm that is not 16-byte aligned.
template <int NE, bool PAIR>
__global__ void __launch_bounds__(kEcgBlock) k_pseudo_ecg(EcgArgs a)
{
    __shared__ double red[kEcgBlock / 32][NE];
    __shared__ bool last;
    using Entry = typename std::conditional<PAIR, float2, double>::type;
    const Entry* lead = static_cast<const Entry*>(a.lead) + (long long)a.e0 * a.ld;
    const long long stride = (long long)gridDim.x * kEcgBlock;
    Acc<PAIR> acc[NE];
    for (long long c = (long long)blockIdx.x * kEcgBlock + threadIdx.x; c < a.n; c += stride) {
        cell_terms<NE, PAIR>(acc, lead, c, a.vm[c]);
        renormalize<NE, PAIR>(acc);
    }
    finish<NE, PAIR>(a, acc, red, last);
}

// ---------------------------------------------------------------- staged
// Persistent form, one block per SM over a contiguous range of tiles of
// tile_of(NE) cells: thread 0 moves each tile of Vm and of the NE rows into a ring
// of shared-memory stages with bulk asynchronous copies (cp.async.bulk,
// completion counted on the stage's mbarrier), keeping up to `stages` tiles
// in flight while the block consumes the oldest.  Every wait is bounded: a
// wait that runs out (after EcgArgs::wait_cycles, by default kWaitCycles)
// sets *error, the block waits for the copies it issued (bounded by
// kWaitCycles whatever the launch's limit, so that no copy lands in the
// shared memory of a block that has left), and its sums become NaN.
constexpr long long kWaitCycles = 1LL << 31;    // about a second

__device__ __forceinline__ unsigned smem_u32(const void* p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy(unsigned dst, const void* src, unsigned bytes,
                                          unsigned bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, long long limit)
{
    const long long t0 = clock64();
    for (;;) {
        unsigned ok;
        // test_wait does not suspend the thread, so the clock limit alone
        // bounds the wait (a limit of zero gives up unless the copy landed)
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > limit) return false;
    }
}

template <int NE>
constexpr unsigned stage_bytes()
{
    return unsigned(NE + 1) * unsigned(tile_of(NE)) * 8u;
}

template <int NE, bool PAIR>
__global__ void __launch_bounds__(kEcgBlock, kStagedPerSm) k_pseudo_ecg_staged(EcgArgs a, int stages,
                                                                  unsigned* error)
{
    extern __shared__ __align__(128) unsigned char stage_mem[];
    __shared__ __align__(8) unsigned long long full[kMaxStages];
    __shared__ double red[kEcgBlock / 32][NE];
    __shared__ bool last;
    __shared__ int failed;
    using Entry = typename std::conditional<PAIR, float2, double>::type;
    constexpr int T = tile_of(NE);
    constexpr unsigned kRow = T * 8u;
    const long long n_even = a.n & ~1LL;
    const long long tiles = (n_even + T - 1) / T;
    const long long per = (tiles + gridDim.x - 1) / gridDim.x;
    const long long t_begin = min(tiles, (long long)blockIdx.x * per);
    const long long t_end = min(tiles, t_begin + per);
    const char* lead = static_cast<const char*>(a.lead) + (long long)a.e0 * a.ld * 8;
    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) mbar_init(smem_u32(&full[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        failed = 0;
    }
    __syncthreads();
    long long issued = 0;    // thread 0: tiles whose copies were issued
    auto issue = [&](long long t, int s) {
        const long long c0 = t * T;
        const unsigned bytes = unsigned(min((long long)T, n_even - c0) * 8);
        const unsigned bar = smem_u32(&full[s]);
        const unsigned dst = smem_u32(stage_mem + (size_t)s * stage_bytes<NE>());
        mbar_expect_tx(bar, bytes + unsigned(NE) * kRow);
        bulk_copy(dst, a.vm + c0, bytes, bar);
        bulk_copy(dst + kRow, lead + t * NE * (long long)kRow, unsigned(NE) * kRow, bar);
        ++issued;
    };
    if (threadIdx.x == 0)
        for (int k = 0; k < stages && t_begin + k < t_end; ++k) issue(t_begin + k, k);
    Acc<PAIR> acc[NE];
    long long k = 0;
    for (long long t = t_begin; t < t_end; ++t, ++k) {
        const int s = int(k % stages);
        if (!mbar_wait(smem_u32(&full[s]), unsigned((k / stages) & 1), a.wait_cycles))
            atomicOr(&failed, 1);
        __syncthreads();
        if (failed) break;
        const unsigned char* st = stage_mem + (size_t)s * stage_bytes<NE>();
        const double* vs = reinterpret_cast<const double*>(st);
        const Entry* rows = reinterpret_cast<const Entry*>(st + kRow);
        const int m = int(min((long long)T, n_even - t * T));
#pragma unroll
        for (int q = 0; q < T / kEcgBlock; ++q) {
            const int i = threadIdx.x + q * kEcgBlock;
            if (i < m) cell_terms<NE, PAIR>(acc, rows, i, vs[i]);
        }
        renormalize<NE, PAIR>(acc);
        __syncthreads();    // stage s read by every thread: refill it
        if (threadIdx.x == 0 && t + stages < t_end) issue(t + stages, s);
    }
    if (failed) {
        if (threadIdx.x == 0) {
            // let the copies still in flight land before the block leaves
            for (long long q = k; q < issued; ++q)
                mbar_wait(smem_u32(&full[int(q % stages)]), unsigned((q / stages) & 1),
                          kWaitCycles);
            atomicOr(error, 1u);
        }
#pragma unroll
        for (int j = 0; j < NE; ++j) acc[j] = Acc<PAIR>::nan();
    }
    // the odd last cell
    if ((a.n & 1) && blockIdx.x == 0 && threadIdx.x == 0)
        cell_terms<NE, PAIR>(acc, reinterpret_cast<const Entry*>(lead), a.n - 1, a.vm[a.n - 1]);
    finish<NE, PAIR>(a, acc, red, last);
}

template <int NE, bool PAIR>
int stages_for()
{
    return std::max(2, std::min(kMaxStages, int((216u * 1024u / kStagedPerSm) / stage_bytes<NE>())));
}

template <int NE, bool PAIR>
cudaError_t launch_typed(const EcgArgs& a, bool staged, int blocks, unsigned* error, cudaStream_t s)
{
    if (staged) {
        const int st = stages_for<NE, PAIR>();
        const size_t smem = size_t(st) * stage_bytes<NE>();
        cudaError_t e = cudaFuncSetAttribute(k_pseudo_ecg_staged<NE, PAIR>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e) return e;
        k_pseudo_ecg_staged<NE, PAIR><<<blocks, kEcgBlock, smem, s>>>(a, st, error);
    } else {
        k_pseudo_ecg<NE, PAIR><<<blocks, kEcgBlock, 0, s>>>(a);
    }
    return cudaGetLastError();
}

template <int NE>
cudaError_t launch_chunk(const EcgArgs& a, bool staged, bool pair, int blocks, unsigned* error,
                         cudaStream_t s)
{
    return pair ? launch_typed<NE, true>(a, staged, blocks, error, s)
                : launch_typed<NE, false>(a, staged, blocks, error, s);
}

cudaError_t launch_any(const EcgArgs& a, int ne, bool staged, bool pair, int blocks,
                       unsigned* error, cudaStream_t s)
{
    switch (ne) {
    case 1: return launch_chunk<1>(a, staged, pair, blocks, error, s);
    case 2: return launch_chunk<2>(a, staged, pair, blocks, error, s);
    case 3: return launch_chunk<3>(a, staged, pair, blocks, error, s);
    case 4: return launch_chunk<4>(a, staged, pair, blocks, error, s);
    case 5: return launch_chunk<5>(a, staged, pair, blocks, error, s);
    case 6: return launch_chunk<6>(a, staged, pair, blocks, error, s);
    case 7: return launch_chunk<7>(a, staged, pair, blocks, error, s);
    default: return launch_chunk<8>(a, staged, pair, blocks, error, s);
    }
}

template <int NE>
int resident_blocks(bool pair)
{
    int per_sm = 0;
    if (pair)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pseudo_ecg<NE, true>, kEcgBlock, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pseudo_ecg<NE, false>, kEcgBlock,
                                                      0);
    return per_sm;
}

int resident_blocks_any(int ne, bool pair)
{
    switch (ne) {
    case 1: return resident_blocks<1>(pair);
    case 2: return resident_blocks<2>(pair);
    case 3: return resident_blocks<3>(pair);
    case 4: return resident_blocks<4>(pair);
    case 5: return resident_blocks<5>(pair);
    case 6: return resident_blocks<6>(pair);
    case 7: return resident_blocks<7>(pair);
    default: return resident_blocks<8>(pair);
    }
}

}  // namespace

struct cfg_pseudo_ecg {
    long long n = 0, ld = 0;
    int n_el = 0;
    std::vector<int> blocks;        // grid of each grid-stride launch
    std::vector<int> staged_blocks; // grid of each staged launch
    unsigned* d_error = nullptr;    // set by a staged launch whose copy wait ran out
    unsigned* h_error = nullptr;    // pinned mirror
    bool pair = false;              // float-pair arithmetic on scaled rows
    void* d_lead = nullptr;         // tile-blocked rows per launch, doubles or float pairs
    double* d_scale = nullptr;      // [n_el] row scales (pairs)
    double* d_partial = nullptr;
    unsigned* d_ticket = nullptr;   // one per launch of kEcgChunk electrodes
    double* d_values = nullptr;     // compute()
    double* h_values = nullptr;     // pinned mirror
    double* d_series = nullptr;     // [max_rows][n_el]
    long long max_rows = 0, rows = 0;
    std::vector<double> times;
    cudaStream_t last_stream = nullptr;   // stream of the last launch (the caller's)
    cudaEvent_t done = nullptr;           // recorded after each launch: the object's
                                          // own handle on its work, whatever the stream
    bool launched = false;
    long long wait_cycles = kWaitCycles;   // limit of the staged form's copy waits
};

using namespace cfg;

namespace {

// Lead rows L[e][c] of the pseudo-ECG: for each face the owner's gradient
// gains g_own (phi_N - phi_P) and the neighbour's g_nei (phi_P - phi_N)
// (the difference form of leastSquaresGrad / gaussGrad with zeroGradient
// walls, built by assemble_corrected), so z_eP.g_own moves to N from P and
// z_eN.g_nei to P from N.
int fold_lead(const cfg_mesh_desc* m, const cfg_pseudo_ecg_desc* d, const CorrectedOperator& op,
              std::vector<double>& lead)
{
    const long long n = m->n_cells, nf = m->n_faces;
    const int ne = d->n_electrodes;
    lead.assign(size_t(ne) * size_t(n), 0.0);
    std::vector<double> z(size_t(3) * size_t(n));
    for (int e = 0; e < ne; ++e) {
        const double* P = d->electrodes + 3 * e;
        for (long long c = 0; c < n; ++c) {
            const double* C = m->centres + 3 * c;
            const double r[3] = {C[0] - P[0], C[1] - P[1], C[2] - P[2]};
            const double mag = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            double* zc = z.data() + 3 * c;
            if (!(mag > 1e-300)) {   // VSMALL
                zc[0] = zc[1] = zc[2] = 0.0;
                continue;
            }
            const double* s = d->conductivity_per_cell ? d->conductivity_per_cell + 6 * c
                                                       : d->conductivity;
            const double k = m->volumes[c] / (mag * mag * mag);
            // (sigma g) . r = g . (sigma r) for the symmetric sigma
            zc[0] = k * (s[0] * r[0] + s[1] * r[1] + s[2] * r[2]);
            zc[1] = k * (s[1] * r[0] + s[3] * r[1] + s[4] * r[2]);
            zc[2] = k * (s[2] * r[0] + s[4] * r[1] + s[5] * r[2]);
        }
        double* L = lead.data() + size_t(e) * size_t(n);
        for (long long f = 0; f < nf; ++f) {
            const long long own = m->owner[f], nei = m->neighbour[f];
            const double* go = op.g_own.data() + 3 * f;
            const double* gn = op.g_nei.data() + 3 * f;
            const double* zp = z.data() + 3 * own;
            const double* zn = z.data() + 3 * nei;
            const double a = zp[0] * go[0] + zp[1] * go[1] + zp[2] * go[2];
            const double b = zn[0] * gn[0] + zn[1] * gn[1] + zn[2] * gn[2];
            L[nei] += a - b;
            L[own] += b - a;
        }
    }
    return CFG_OK;
}

// The partial sums and the ticket are the object's own: a launch on another
// stream than the last one waits for that one first.
int launch(cfg_pseudo_ecg* ecg, const double* vm, cudaStream_t s, double* out)
{
    if (ecg->launched && s != ecg->last_stream) CFG_CUDA_TRY(cudaStreamWaitEvent(s, ecg->done, 0));
    // the staged form copies whole 16-byte units of Vm
    const bool staged = (reinterpret_cast<uintptr_t>(vm) & 15) == 0;
    for (int e0 = 0, k = 0; e0 < ecg->n_el; e0 += kEcgChunk, ++k) {
        EcgArgs a{ecg->d_lead, ecg->d_scale, vm, ecg->n, ecg->ld, ecg->n_el, e0,
                  ecg->d_partial, ecg->d_ticket + k, out, ecg->wait_cycles};
        const int blocks = staged ? ecg->staged_blocks[size_t(k)] : ecg->blocks[size_t(k)];
        CFG_CUDA_TRY(launch_any(a, std::min(kEcgChunk, ecg->n_el - e0), staged, ecg->pair,
                                blocks, ecg->d_error, s));
    }
    CFG_CUDA_TRY(cudaEventRecord(ecg->done, s));
    ecg->last_stream = s;
    ecg->launched = true;
    return CFG_OK;
}

// Waits for the object's last launch and reports a staged launch whose copy
// wait ran out (the flag is cleared).
int check_error(cfg_pseudo_ecg* ecg)
{
    CFG_CUDA_TRY(cudaEventSynchronize(ecg->done));
    CFG_CUDA_TRY(cudaMemcpy(ecg->h_error, ecg->d_error, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (*ecg->h_error) {
        CFG_CUDA_TRY(cudaMemset(ecg->d_error, 0, sizeof(unsigned)));
        return fail(CFG_ERR_CUDA, "a pseudo-ECG tile copy did not complete within its wait limit");
    }
    return CFG_OK;
}

}  // namespace

extern "C" int cfg_pseudo_ecg_create(const cfg_pseudo_ecg_desc* d, const cfg_mesh_desc* m,
                                     cfg_pseudo_ecg** out)
{
    clear_error();
    if (!d || !m || !out) return fail(CFG_ERR_INVALID, "null argument");
    *out = nullptr;
    if (!m->face_centres || !m->centres || !m->volumes || !m->face_sf)
        return fail(CFG_ERR_INVALID, "the pseudo-ECG needs the mesh's full geometry");
    if (d->n_electrodes <= 0 || !d->electrodes)
        return fail(CFG_ERR_INVALID, "no electrodes");
    if (d->max_rows < 0) return fail(CFG_ERR_INVALID, "max_rows must be non-negative");
    if (d->grad_scheme != CFG_GRAD_LEAST_SQUARES && d->grad_scheme != CFG_GRAD_GAUSS_LINEAR)
        return fail(CFG_ERR_INVALID, "unknown gradient scheme %d", d->grad_scheme);
    if (d->arithmetic != CFG_ECG_FP64 && d->arithmetic != CFG_ECG_FLOAT_PAIRS)
        return fail(CFG_ERR_INVALID, "unknown arithmetic %d", d->arithmetic);
    const long long n = m->n_cells;
    for (long long f = 0; f < m->n_faces; ++f) {
        const int l = m->owner[f], u = m->neighbour[f];
        if (l < 0 || u < 0 || l >= n || u >= n || l == u)
            return fail(CFG_ERR_INVALID, "face %lld has invalid owner/neighbour %d/%d", f, l, u);
    }
    if (n <= 0) return fail(CFG_ERR_INVALID, "the mesh has no cells");
    const long long ld = (n + kTile - 1) / kTile * kTile;   // whole tiles of either size
    const size_t lead_bytes = size_t(d->n_electrodes) * size_t(ld) * sizeof(double);
    size_t free_b = 0, total_b = 0;
    CFG_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    if (lead_bytes > free_b / 2)
        return fail(CFG_ERR_INVALID, "the lead rows (%zu bytes) exceed half the free device memory",
                    lead_bytes);
    CorrectedOperator op;
    if (int rc = assemble_corrected(m, d->conductivity, d->conductivity_per_cell, d->grad_scheme,
                                    0, op))
        return rc;
    std::vector<double> lead;
    if (int rc = fold_lead(m, d, op, lead)) return rc;

    auto* ecg = new cfg_pseudo_ecg();
    ecg->n = n;
    ecg->ld = ld;
    ecg->n_el = d->n_electrodes;
    ecg->pair = d->arithmetic == CFG_ECG_FLOAT_PAIRS;
    // staged form: one block per SM (at most one per tile); grid-stride form:
    // per launch one wave of resident blocks
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    for (int e0 = 0; e0 < ecg->n_el; e0 += kEcgChunk) {
        const long long T = tile_of(std::min(kEcgChunk, ecg->n_el - e0));
        ecg->staged_blocks.push_back(int(std::max(
            1LL, std::min<long long>(std::max(sms, 1) * kStagedPerSm, ((n & ~1LL) + T - 1) / T))));
    }
    const long long need = (n + kEcgBlock - 1) / kEcgBlock;
    for (int e0 = 0; e0 < ecg->n_el; e0 += kEcgChunk) {
        const int per_sm = std::max(1, std::min(resident_blocks_any(std::min(kEcgChunk,
                                                                             ecg->n_el - e0),
                                                                    ecg->pair),
                                                kEcgBlocksPerSm));
        ecg->blocks.push_back(int(std::max(1LL, std::min<long long>(
                                                    need, (long long)std::max(sms, 1) * per_sm))));
    }
    const int max_blocks = std::max(
        *std::max_element(ecg->staged_blocks.begin(), ecg->staged_blocks.end()),
        *std::max_element(ecg->blocks.begin(), ecg->blocks.end()));
    auto bail = [&](int rc) {
        cfg_pseudo_ecg_destroy(ecg);
        return rc;
    };
    cudaError_t e = cudaMalloc(&ecg->d_lead, lead_bytes);
    // pairs: each row scaled by a power of two to a largest magnitude in
    // [0.5, 1) (exact), then split into the nearest float and the float
    // nearest to the rest
    std::vector<double> scale(size_t(ecg->n_el), 1.0);
    if (ecg->pair)
        for (int r = 0; r < ecg->n_el; ++r) {
            const double* row = lead.data() + size_t(r) * size_t(n);
            double mx = 0.0;
            for (long long c = 0; c < n; ++c) mx = std::max(mx, std::fabs(row[c]));
            int ex = 0;
            if (mx > 0.0) std::frexp(mx, &ex);
            scale[size_t(r)] = std::ldexp(1.0, -ex);
        }
    // tile-blocked order per launch of up to kEcgChunk electrodes, zero padded
    auto blocked = [&](auto put) {
        for (int e0 = 0; e0 < ecg->n_el; e0 += kEcgChunk) {
            const int ne = std::min(kEcgChunk, ecg->n_el - e0);
            const long long T = tile_of(ne);
            for (long long t = 0; t < ld / T; ++t)
                for (int j = 0; j < ne; ++j)
                    for (long long i = 0; i < T; ++i) {
                        const long long c = t * T + i;
                        const size_t at = size_t(e0) * size_t(ld) +
                                          size_t((t * ne + j) * T + i);
                        put(at, e0 + j, c < n ? lead[size_t(e0 + j) * size_t(n) + size_t(c)] : 0.0);
                    }
        }
    };
    if (!e && ecg->pair) {
        std::vector<float2> pairs(size_t(ecg->n_el) * size_t(ld));
        blocked([&](size_t at, int r, double x) {
            const double v = x * scale[size_t(r)];
            const float h = float(v);
            pairs[at] = make_float2(h, float(v - double(h)));
        });
        e = cudaMemcpy(ecg->d_lead, pairs.data(), lead_bytes, cudaMemcpyHostToDevice);
        if (!e) e = dmalloc(&ecg->d_scale, scale.size());
        if (!e) e = cudaMemcpy(ecg->d_scale, scale.data(), scale.size() * sizeof(double),
                               cudaMemcpyHostToDevice);
    } else if (!e) {
        std::vector<double> rows(size_t(ecg->n_el) * size_t(ld));
        blocked([&](size_t at, int, double x) { rows[at] = x; });
        e = cudaMemcpy(ecg->d_lead, rows.data(), lead_bytes, cudaMemcpyHostToDevice);
    }
    if (!e) e = dmalloc(&ecg->d_partial, size_t(max_blocks) * size_t(ecg->n_el));
    const int chunks = (ecg->n_el + kEcgChunk - 1) / kEcgChunk;
    if (!e) e = dmalloc(&ecg->d_ticket, size_t(chunks));
    if (!e) e = cudaMemset(ecg->d_ticket, 0, sizeof(unsigned) * size_t(chunks));
    if (!e) e = cudaEventCreateWithFlags(&ecg->done, cudaEventDisableTiming);
    if (!e) e = dmalloc(&ecg->d_error, 1);
    if (!e) e = cudaMemset(ecg->d_error, 0, sizeof(unsigned));
    if (!e) e = dmalloc(&ecg->d_values, size_t(ecg->n_el));
    if (!e) e = cudaMallocHost(reinterpret_cast<void**>(&ecg->h_values),
                               size_t(ecg->n_el) * sizeof(double));
    if (!e) e = cudaMallocHost(reinterpret_cast<void**>(&ecg->h_error), sizeof(unsigned));
    if (!e && d->max_rows > 0) e = dmalloc(&ecg->d_series, size_t(d->max_rows) * size_t(ecg->n_el));
    if (e) return bail(fail(CFG_ERR_CUDA, "pseudo-ECG allocation: %s", cudaGetErrorString(e)));
    ecg->max_rows = d->max_rows;
    ecg->times.reserve(size_t(d->max_rows));
    *out = ecg;
    return CFG_OK;
}

extern "C" int cfg_pseudo_ecg_compute(cfg_pseudo_ecg* ecg, const double* vm, void* stream,
                                      double* values)
{
    if (!ecg || !vm || !values) return fail(CFG_ERR_INVALID, "null argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (int rc = launch(ecg, vm, s, ecg->d_values)) return rc;
    CFG_CUDA_TRY(cudaMemcpyAsync(ecg->h_values, ecg->d_values, size_t(ecg->n_el) * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
    CFG_CUDA_TRY(cudaEventRecord(ecg->done, s));   // after the copy of the values
    if (int rc = check_error(ecg)) return rc;
    std::memcpy(values, ecg->h_values, size_t(ecg->n_el) * sizeof(double));
    return CFG_OK;
}

extern "C" int cfg_pseudo_ecg_compute_monodomain(cfg_pseudo_ecg* ecg, cfg_monodomain* md,
                                                 double* values)
{
    if (!ecg || !md) return fail(CFG_ERR_INVALID, "null argument");
    if (md->n != ecg->n) return fail(CFG_ERR_INVALID, "the context has %lld cells, the ECG %lld",
                                     md->n, ecg->n);
    return cfg_pseudo_ecg_compute(ecg, md->d_vm, md->stream, values);
}

extern "C" int cfg_pseudo_ecg_record_field(cfg_pseudo_ecg* ecg, const double* vm, void* stream,
                                           double t)
{
    if (!ecg || !vm) return fail(CFG_ERR_INVALID, "null argument");
    if (ecg->rows >= ecg->max_rows)
        return fail(CFG_ERR_INVALID, "the pseudo-ECG series is full (%lld rows)", ecg->max_rows);
    if (int rc = launch(ecg, vm, static_cast<cudaStream_t>(stream),
                        ecg->d_series + ecg->rows * ecg->n_el))
        return rc;
    ecg->times.push_back(t);
    ecg->rows++;
    return CFG_OK;
}

extern "C" int cfg_pseudo_ecg_record(cfg_pseudo_ecg* ecg, cfg_monodomain* md)
{
    if (!ecg || !md) return fail(CFG_ERR_INVALID, "null argument");
    if (md->n != ecg->n) return fail(CFG_ERR_INVALID, "the context has %lld cells, the ECG %lld",
                                     md->n, ecg->n);
    return cfg_pseudo_ecg_record_field(ecg, md->d_vm, md->stream, md->t_host);
}

extern "C" int cfg_pseudo_ecg_series(cfg_pseudo_ecg* ecg, double* times, double* values,
                                     long long max_rows, long long* n_rows)
{
    if (!ecg) return fail(CFG_ERR_INVALID, "null argument");
    if (n_rows) *n_rows = ecg->rows;
    const long long k = std::min(max_rows, ecg->rows);
    if (k <= 0) return CFG_OK;
    if (ecg->launched)
        if (int rc = check_error(ecg)) return rc;
    if (values)
        CFG_CUDA_TRY(cudaMemcpy(values, ecg->d_series, size_t(k) * size_t(ecg->n_el) * sizeof(double),
                                cudaMemcpyDeviceToHost));
    if (times) std::memcpy(times, ecg->times.data(), size_t(k) * sizeof(double));
    return CFG_OK;
}

extern "C" int cfg_pseudo_ecg_set_wait_limit(cfg_pseudo_ecg* ecg, long long cycles)
{
    if (!ecg) return fail(CFG_ERR_INVALID, "null argument");
    ecg->wait_cycles = cycles < 0 ? kWaitCycles : cycles;
    return CFG_OK;
}

extern "C" int cfg_pseudo_ecg_reset(cfg_pseudo_ecg* ecg)
{
    if (!ecg) return fail(CFG_ERR_INVALID, "null argument");
    ecg->rows = 0;
    ecg->times.clear();
    return CFG_OK;
}

extern "C" int cfg_pseudo_ecg_destroy(cfg_pseudo_ecg* ecg)
{
    if (!ecg) return CFG_OK;
    // the last launch ran on a caller's stream, which may be gone by now: wait
    // on the object's own event instead
    if (ecg->launched) cudaEventSynchronize(ecg->done);
    if (ecg->done) cudaEventDestroy(ecg->done);
    if (ecg->d_lead) cudaFree(ecg->d_lead);
    dfree(ecg->d_scale);
    dfree(ecg->d_partial);
    dfree(ecg->d_ticket);
    dfree(ecg->d_error);
    dfree(ecg->d_values);
    dfree(ecg->d_series);
    if (ecg->h_values) cudaFreeHost(ecg->h_values);
    if (ecg->h_error) cudaFreeHost(ecg->h_error);
    delete ecg;
    return CFG_OK;
}
