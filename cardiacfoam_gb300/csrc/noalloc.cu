// Implicit diffusion solve of the monodomain equation on a structured box
// that allocates no device memory.
//
// Some callers cannot call cudaMalloc when they need a solve: a coupled
// solver or host application that owns all device memory through its own
// pool and gives plug-ins a fixed budget, or one that overlaps work on
// several streams and cannot afford the device-wide synchronisation that
// cudaFree (and often cudaMalloc) implies in the middle of a time step.
// For them this entry point takes the fields as caller-owned device buffers
// and keeps every temporary of the solve (the matrix diagonal, the PCG
// vectors, the reduction partials and the solver state) in one file-scope
// device array of fixed size, CFG_NOALLOC_SCRATCH_BYTES, for boxes of at
// most CFG_NOALLOC_MAX_CELLS cells.  Every GPU that loads this code holds
// that array until the process exits.
//
// The solve runs the same kernels as the monodomain step's implicit
// diffusion (one PIMPLE corrector, PCG with the diagonal preconditioner),
// so its result is that of the step's first corrector for the same inputs.
//
// The array is shared by every call on a device and keeps the last call's
// contents; the solver state, including the counters of the last-block
// reductions, is cleared at the start of each call, and every vector is
// written before it is read.  Calls whose work overlaps on the GPU (two
// host threads, or two streams) race on the array: serialise them.
//
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture is begun on the device.  The cached
// address is that of the device's primary context at the first call: a
// cudaDeviceReset (or another reset of the primary context) invalidates it,
// and the entry point is not to be called after one in the same process.
#include <mutex>

#include "diffusion_kernels.cuh"
#include "host_common.h"

namespace cfg {

__global__ void k_prepare(DiffusionArgs a);
__global__ void k_solve_begin(DiffusionArgs a);
__global__ void k_solve_norm(DiffusionArgs a);
__global__ void k_pcg_p(DiffusionArgs a);
__global__ void k_pcg_update(DiffusionArgs a);

namespace {

constexpr long long kMaxCells = CFG_NOALLOC_MAX_CELLS;
constexpr int kMaxBlocks = int((kMaxCells + kDiffBlock - 1) / kDiffBlock);
constexpr size_t round256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kVecBytes = round256(size_t(kMaxCells) * sizeof(double));
// vol, lapdiag, b, r, z, ax, pA, pB, ap, and [2][n] diag2, rdiag2, sumA2
constexpr int kVectors = 9 + 2 * 3;
constexpr size_t kPartialBytes = round256(4 * size_t(kMaxBlocks) * sizeof(double));
constexpr size_t kStateBytes = round256(sizeof(PcgState));
constexpr size_t kScratchBytes = kVectors * kVecBytes + kPartialBytes + kStateBytes;
static_assert(kScratchBytes <= CFG_NOALLOC_SCRATCH_BYTES,
              "CFG_NOALLOC_SCRATCH_BYTES must cover the no-allocation scratch layout");

// In host code this name only stands for the device array: its address is
// taken with cudaGetSymbolAddress, never by '&' on the host.
static __device__ __align__(256) unsigned char g_noalloc_scratch[CFG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_base[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up on the
// first call per device).
int scratch_base(unsigned char** out)
{
    int dev = 0;
    CFG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(CFG_ERR_INVALID, "device %d is beyond the %d devices supported", dev,
                    kMaxDevices);
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_base[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(CFG_ERR_CUDA, "cudaGetSymbolAddress of the no-allocation scratch on "
                                      "device %d failed: %s", dev, cudaGetErrorString(e));
        g_base[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_base[dev];
    return CFG_OK;
}

// Cell volumes, the Laplacian row sums (minus the face coefficients of the
// present neighbours, in ascending neighbour order as the ELL build sums
// them) and a cleared solver state for one corrector.
__global__ void k_noalloc_begin(DiffusionArgs a, double* vol, double* lapdiag, double cell_volume,
                                int n_old, double tol, double rel_tol, int max_iter)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < a.n) {
        const long long nx = a.sx, nxy = (long long)a.sx * a.sy;
        const long long i = c % nx, j = (c / nx) % a.sy, k = c / nxy;
        double s = 0.0;
        if (k > 0) s -= a.cz;
        if (j > 0) s -= a.cy;
        if (i > 0) s -= a.cx;
        if (i + 1 < nx) s -= a.cx;
        if (j + 1 < a.sy) s -= a.cy;
        if (k + 1 < a.sz) s -= a.cz;
        vol[c] = cell_volume;
        lapdiag[c] = s;
    }
    if (c == 0) {
        PcgState* st = a.st;
        *st = PcgState{};
        st->n_old = n_old;
        st->corr = 1;
        st->outer_active = 1;
        st->tol = tol;
        st->rel_tol = rel_tol;
        st->outer_tol = 0.0;
        st->max_iter = max_iter;
        st->n_outer = 1;
    }
}

}  // namespace
}  // namespace cfg

using namespace cfg;

extern "C" int cfg_box_diffusion_solve_noalloc(const cfg_box_diffusion_desc* d, double delta_t,
                                               const double* vm_old, const double* vm_oldold,
                                               const double* iion, double* vm, void* stream,
                                               cfg_solve_result* result)
{
    clear_error();
    if (!d || !vm_old || !iion || !vm) return fail(CFG_ERR_INVALID, "null argument");
    if (d->nx < 1 || d->ny < 1 || d->nz < 1)
        return fail(CFG_ERR_INVALID, "box of %d x %d x %d cells", d->nx, d->ny, d->nz);
    const long long n = (long long)d->nx * d->ny * d->nz;
    if (n > kMaxCells)
        return fail(CFG_ERR_INVALID,
                    "box of %lld cells exceeds the no-allocation maximum of %lld cells "
                    "(CFG_NOALLOC_MAX_CELLS)", n, kMaxCells);
    if (!(delta_t > 0)) return fail(CFG_ERR_INVALID, "deltaT must be positive");
    if (!(d->chi > 0) || !(d->cm > 0)) return fail(CFG_ERR_INVALID, "chi and cm must be positive");
    if (!(d->cell_volume > 0)) return fail(CFG_ERR_INVALID, "cell volume must be positive");
    for (int k = 0; k < 3; ++k)
        if (!(d->face_coeff[k] >= 0))
            return fail(CFG_ERR_INVALID, "face coefficient %d must be non-negative", k);
    if (d->ddt_backward && !vm_oldold)
        return fail(CFG_ERR_INVALID, "backward ddt needs the old-old time level");
    if (d->pcg_max_iter < 0) return fail(CFG_ERR_INVALID, "maxIter must be non-negative");

    unsigned char* base = nullptr;
    if (int rc = scratch_base(&base)) return rc;
    auto vec = [base](int i) { return reinterpret_cast<double*>(base + size_t(i) * kVecBytes); };

    DiffusionArgs a{};
    a.n = n;
    a.sx = d->nx;
    a.sy = d->ny;
    a.sz = d->nz;
    a.cx = d->face_coeff[0];
    a.cy = d->face_coeff[1];
    a.cz = d->face_coeff[2];
    a.vol = vec(0);
    a.lapdiag = vec(1);
    a.b = vec(2);
    a.r = vec(3);
    a.z = vec(4);
    a.ax = vec(5);
    a.pA = vec(6);
    a.pB = vec(7);
    a.ap = vec(8);
    // [2][n] arrays over two vector slots each: v * n + c stays inside them
    a.diag2 = vec(9);
    a.rdiag2 = vec(11);
    a.sumA2 = vec(13);
    a.partial = reinterpret_cast<double*>(base + kVectors * kVecBytes);
    a.st = reinterpret_cast<PcgState*>(base + kVectors * kVecBytes + kPartialBytes);
    a.nblocks = int((n + kDiffBlock - 1) / kDiffBlock);
    // the solve reads the old time levels and never writes them
    a.vm = vm;
    a.vm_old = const_cast<double*>(vm_old);
    a.vm_oldold = const_cast<double*>(vm_oldold ? vm_oldold : vm_old);
    a.iion = iion;
    a.use_graph = 0;
    a.iter_cap = (long long)d->pcg_max_iter + 1;
    a.dt = delta_t;
    a.chicm = d->chi * d->cm;
    a.ddt_backward = d->ddt_backward ? 1 : 0;
    // EulerDdtScheme, or backwardDdtScheme with both old levels (deltaT0 = deltaT)
    a.rdt = 1.0 / delta_t;
    for (int v = 0; v < 2; ++v) {
        if (!a.ddt_backward) {
            a.cft[v] = 1.0; a.cft0[v] = 1.0; a.cft00[v] = 0.0;
            continue;
        }
        const double dt0 = v == 0 ? 1e15 : delta_t;
        a.cft[v] = 1 + delta_t / (delta_t + dt0);
        a.cft00[v] = delta_t * delta_t / (dt0 * (delta_t + dt0));
        a.cft0[v] = a.cft[v] + a.cft00[v];
    }

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned grid = unsigned(a.nblocks);
    k_noalloc_begin<<<grid, kDiffBlock, 0, s>>>(a, vec(0), vec(1), d->cell_volume,
                                                 a.ddt_backward ? 2 : 1, d->pcg_tol,
                                                 d->pcg_rel_tol, d->pcg_max_iter);
    k_prepare<<<grid, kDiffBlock, 0, s>>>(a);
    k_solve_begin<<<grid, kDiffBlock, 0, s>>>(a);
    k_solve_norm<<<grid, kDiffBlock, 0, s>>>(a);
    CFG_CUDA_TRY(cudaGetLastError());
    PcgState h;
    auto read = [&]() -> int {
        CFG_CUDA_TRY(cudaMemcpyAsync(&h, a.st, sizeof h, cudaMemcpyDeviceToHost, s));
        CFG_CUDA_TRY(cudaStreamSynchronize(s));
        return CFG_OK;
    };
    if (int rc = read()) return rc;
    constexpr int kChunk = 8;   // iterations enqueued per host check; surplus ones return at once
    for (long long guard = 0; h.solve_active; guard += kChunk) {
        if (guard > (long long)d->pcg_max_iter + kChunk)
            return fail(CFG_ERR_PCG, "PCG did not stop within maxIter = %d", d->pcg_max_iter);
        for (int k = 0; k < kChunk; ++k) {
            k_pcg_p<<<grid, kDiffBlock, 0, s>>>(a);
            k_pcg_update<<<grid, kDiffBlock, 0, s>>>(a);
        }
        CFG_CUDA_TRY(cudaGetLastError());
        if (int rc = read()) return rc;
    }
    if (result) {
        result->iterations = h.iters[0];
        result->converged = (h.status & CFG_ERR_PCG) ? 0 : 1;
        result->initial_residual = h.init_r[0];
        result->final_residual = h.final_r[0];
    }
    return CFG_OK;
}
