// One monodomain time step as a CUDA graph.  The PIMPLE corrector loop and
// the PCG iteration loop are conditional WHILE nodes whose conditions the
// kernels set from the device-side solver state, so a step needs no host
// round trip:
//
//   k_step_begin -> ionic step -> WHILE(outer) {
//       [k_grad_iterate] -> k_solve_begin -> k_solve_norm
//       -> WHILE(inner) { k_pcg_p -> k_pcg_update } -> k_outer_cond }
//   -> k_activation
//
// (k_grad_iterate only on general meshes, for the Laplacian's explicit
// correction.)
//
// Both loops are bounded: PCG stops at maxIter, the corrector loop at
// nOuterCorrectors, and a per-step iteration cap ends the step with an error.
#include "diffusion_kernels.cuh"
#include "host_common.h"
#include "ionic_host.h"
#include "monodomain_host.h"

namespace cfg {

__global__ void k_step_begin(DiffusionArgs a);
__global__ void k_solve_begin(DiffusionArgs a);
__global__ void k_solve_norm(DiffusionArgs a);
__global__ void k_pcg_p(DiffusionArgs a);
__global__ void k_pcg_update(DiffusionArgs a);
__global__ void k_outer_cond(DiffusionArgs a);
__global__ void k_activation(DiffusionArgs a);
__global__ void k_explicit(DiffusionArgs a);
__global__ void k_explicit_finish(PcgState* st, int ddt_backward);
__global__ void k_grad_iterate(DiffusionArgs a);
__global__ void k_grad_start(DiffusionArgs a);

namespace {

struct Builder {
    cudaGraph_t g;
    const DiffusionArgs* args;
    unsigned grid;

    cudaError_t kernel(void (*fn)(DiffusionArgs), cudaGraphNode_t* out,
                       const cudaGraphNode_t* deps, size_t ndeps, unsigned blocks = 0,
                       unsigned threads = kDiffBlock)
    {
        cudaKernelNodeParams p{};
        p.func = reinterpret_cast<void*>(fn);
        p.gridDim = dim3(blocks ? blocks : grid);
        p.blockDim = dim3(threads);
        void* kargs[] = {const_cast<DiffusionArgs*>(args)};
        p.kernelParams = kargs;
        return cudaGraphAddKernelNode(out, g, deps, ndeps, &p);
    }

    cudaError_t event(cudaEvent_t e, cudaGraphNode_t* out, const cudaGraphNode_t* deps,
                      size_t ndeps)
    {
        return cudaGraphAddEventRecordNode(out, g, deps, ndeps, e);
    }
};

// Capture the ionic launch (a host launcher picks the kernel) into a child graph.
cudaError_t capture_ionic(cfg_monodomain* md, double dt, cudaGraph_t* out)
{
    cudaStream_t s = md->stream;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e) return e;
    IonicLaunch L = ionic_launch_args(md->ion, 0.0, dt, &md->d_st->t0, md->d_vm, md->d_iion);
    cudaError_t le = ionic_enqueue(md->ion, L);
    e = cudaStreamEndCapture(s, out);
    return le ? le : e;
}

}  // namespace

#define CFG_G(x)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (x);                                                                 \
        if (e_ != cudaSuccess) {                                                              \
            if (g) cudaGraphDestroy(g);                                                       \
            return fail(CFG_ERR_CUDA, "step graph: %s failed: %s", #x, cudaGetErrorString(e_)); \
        }                                                                                     \
    } while (0)

// Step graph of the persistent form, captured from the stream:
//   k_step_begin -> ionic step -> persistent implicit diffusion
// (the corrector and PCG loops run inside the last kernel).  The timing
// events are recorded as external event nodes, so the host can read them.
static int build_persistent_graph(cfg_monodomain* md, double dt)
{
    fill_args_public(md, dt);
    DiffusionArgs a = md->args;
    cudaStream_t s = md->stream;
    cudaGraph_t g = nullptr;
    CFG_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    k_step_begin<<<unsigned(a.nblocks), kDiffBlock, 0, s>>>(a);
    le = cudaGetLastError();
    if (!le && md->timing) le = cudaEventRecordWithFlags(md->ev[0], s, cudaEventRecordExternal);
    if (!le) {
        IonicLaunch L = ionic_launch_args(md->ion, 0.0, dt, &md->d_st->t0, md->d_vm, md->d_iion);
        le = ionic_enqueue(md->ion, L);
    }
    if (!le && md->timing) le = cudaEventRecordWithFlags(md->ev[1], s, cudaEventRecordExternal);
    if (!le) le = launch_implicit_coop(a, md->coop_blocks, s);
    if (!le && md->timing) le = cudaEventRecordWithFlags(md->ev[2], s, cudaEventRecordExternal);
    const cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (le || ce) {
        if (g) cudaGraphDestroy(g);
        return fail(CFG_ERR_CUDA, "step graph capture failed: %s",
                    cudaGetErrorString(le ? le : ce));
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ie) return fail(CFG_ERR_CUDA, "step graph instantiation failed: %s", cudaGetErrorString(ie));
    md->graph_exec = exec;
    md->graph_dt = dt;
    md->graph_timing = md->timing;
    md->graph_persistent = true;
    return CFG_OK;
}

int build_step_graph(cfg_monodomain* md, double dt)
{
    if (md->graph_exec) {
        cudaGraphExecDestroy(md->graph_exec);
        md->graph_exec = nullptr;
    }
    if (md->implicit && md->persistent) return build_persistent_graph(md, dt);
    fill_args_public(md, dt);
    DiffusionArgs a = md->args;
    a.use_graph = 1;
    cudaGraph_t g = nullptr;
    CFG_G(cudaGraphCreate(&g, 0));
    Builder b{g, &a, unsigned(a.nblocks)};
    const bool timing = md->timing;
    cudaGraphNode_t n_begin, n_ev0, n_ionic, n_ev1, n_last;
    CFG_G(b.kernel(k_step_begin, &n_begin, nullptr, 0));
    cudaGraphNode_t prev = n_begin;
    if (timing) {
        CFG_G(b.event(md->ev[0], &n_ev0, &prev, 1));
        prev = n_ev0;
    }
    cudaGraph_t ionic = nullptr;
    CFG_G(capture_ionic(md, dt, &ionic));
    {
        cudaError_t e = cudaGraphAddChildGraphNode(&n_ionic, g, &prev, 1, ionic);
        cudaGraphDestroy(ionic);
        CFG_G(e);
    }
    prev = n_ionic;
    if (timing) {
        CFG_G(b.event(md->ev[1], &n_ev1, &prev, 1));
        prev = n_ev1;
    }
    if (!md->implicit) {
        cudaGraphNode_t n_ex, n_fin;
        if (md->corrected) {
            cudaGraphNode_t n_g;
            CFG_G(b.kernel(k_grad_start, &n_g, &prev, 1));
            prev = n_g;
        }
        CFG_G(b.kernel(k_explicit, &n_ex, &prev, 1));
        cudaKernelNodeParams p{};
        PcgState* st = md->d_st;
        int bw = md->ddt_backward ? 1 : 0;
        void* kargs[] = {&st, &bw};
        p.func = reinterpret_cast<void*>(k_explicit_finish);
        p.gridDim = dim3(1);
        p.blockDim = dim3(1);
        p.kernelParams = kargs;
        CFG_G(cudaGraphAddKernelNode(&n_fin, g, &n_ex, 1, &p));
        n_last = n_fin;
    } else {
        // PIMPLE corrector loop: the first corrector always runs
        CFG_G(cudaGraphConditionalHandleCreate(&a.h_outer, g, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = a.h_outer;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t n_outer;
        CFG_G(cudaGraphAddNode(&n_outer, g, &prev, nullptr, 1, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        // PCG iteration loop inside the corrector; k_solve_norm sets it
        CFG_G(cudaGraphConditionalHandleCreate(&a.h_inner, body, 0, 0));
        Builder bb{body, &a, unsigned(a.nblocks)};
        cudaGraphNode_t n_sb, n_sn, n_inner, n_oc;
        if (md->corrected) {
            cudaGraphNode_t n_g;
            CFG_G(bb.kernel(k_grad_iterate, &n_g, nullptr, 0));
            CFG_G(bb.kernel(k_solve_begin, &n_sb, &n_g, 1));
        } else {
            CFG_G(bb.kernel(k_solve_begin, &n_sb, nullptr, 0));
        }
        CFG_G(bb.kernel(k_solve_norm, &n_sn, &n_sb, 1));
        cudaGraphNodeParams ip{};
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = a.h_inner;
        ip.conditional.type = cudaGraphCondTypeWhile;
        ip.conditional.size = 1;
        CFG_G(cudaGraphAddNode(&n_inner, body, &n_sn, nullptr, 1, &ip));
        cudaGraph_t ibody = ip.conditional.phGraph_out[0];
        Builder ib{ibody, &a, unsigned(a.nblocks)};
        cudaGraphNode_t n_p, n_u;
        CFG_G(ib.kernel(k_pcg_p, &n_p, nullptr, 0));
        CFG_G(ib.kernel(k_pcg_update, &n_u, &n_p, 1));
        CFG_G(bb.kernel(k_outer_cond, &n_oc, &n_inner, 1, 1, 1));
        cudaGraphNode_t n_act;
        CFG_G(b.kernel(k_activation, &n_act, &n_outer, 1));
        n_last = n_act;
    }
    if (timing) {
        cudaGraphNode_t n_ev2;
        CFG_G(b.event(md->ev[2], &n_ev2, &n_last, 1));
    }
    cudaGraphExec_t exec = nullptr;
    CFG_G(cudaGraphInstantiate(&exec, g, 0));
    cudaGraphDestroy(g);
    md->graph_exec = exec;
    md->graph_dt = dt;
    md->graph_timing = timing;
    md->graph_persistent = md->persistent;
    return CFG_OK;
}

}  // namespace cfg
