// Host representation of a GPU monodomain context.
#pragma once

#include <vector>

#include "apd.cuh"
#include "diffusion_kernels.cuh"
#include "grid_sync.cuh"
#include "host_common.h"

struct cfg_purkinje;

struct cfg_monodomain {
    cfg_ionic* ion = nullptr;
    long long n = 0;
    int width = 0;
    size_t ell_bytes = 0;
    long long nnz_offdiag = 0;
    // structured stencil form
    int sx = 0, sy = 0, sz = 0;
    double cx = 0, cy = 0, cz = 0;
    bool use_stencil = false;
    // settings
    bool implicit = true, ddt_backward = true;
    double chicm = 0;
    int n_boxes = 0;
    double box_min[8][3], box_max[8][3], box_start[8], box_duration[8], box_intensity[8];
    std::vector<unsigned char> h_box;
    // device operator and fields
    int* d_col = nullptr;
    double* d_coef = nullptr;
    unsigned char* d_cnt = nullptr;
    double* d_lapdiag = nullptr;
    double* d_vol = nullptr;
    // explicit correction of the Laplacian on a general mesh
    bool corrected = false;
    bool nc_fp32 = false;         // correction arrays in float (mixed form)
    void *d_nc_gw = nullptr, *d_nc_k = nullptr, *d_nc_om = nullptr, *d_nc_bk = nullptr;
    void* d_grad = nullptr;
    double* d_bsrc = nullptr;     // corrector-independent source of the persistent kernel
    double *d_vm = nullptr, *d_vm_old = nullptr, *d_vm_oldold = nullptr, *d_iion = nullptr;
    double* d_act = nullptr;
    unsigned char* d_act_flag = nullptr;
    unsigned char* d_box = nullptr;
    // operator per ddt coefficient set, and PCG work
    double *d_diag2 = nullptr, *d_rdiag2 = nullptr, *d_sumA2 = nullptr;
    double prepared_dt = 0.0;
    double *d_b = nullptr, *d_r = nullptr, *d_z = nullptr, *d_ax = nullptr, *d_pA = nullptr,
           *d_pB = nullptr, *d_ap = nullptr;
    double* d_partial = nullptr;
    // float-pair PCG of the persistent solve (CFG_PCG_FLOAT_PAIRS, the mixed
    // form's default): the scaled operator as pairs and the published
    // iterate; the scale follows from the largest diagonal, bounded by
    // chi Cm 2 V_max / dt + max(-lapdiag)
    bool pair = false;
    float2 *d_pdiag2 = nullptr, *d_prdiag2 = nullptr, *d_psumA2 = nullptr, *d_pcoef = nullptr,
           *d_px = nullptr;
    double max_vol = 0.0, max_neglap = 0.0;
    cfg::PcgState* d_st = nullptr;
    cfg::PcgState* h_st = nullptr;   // pinned mirror
    cfg::DiffusionArgs args{};
    // control
    cudaStream_t stream = nullptr;
    int iter_chunk = 2;
    int graph_max_corr = 4, graph_max_iter = 4;
    // step graph (device-driven PIMPLE/PCG loops), rebuilt when dt or the
    // timing switch change
    cudaGraphExec_t graph_exec = nullptr;
    double graph_dt = 0.0;
    bool graph_timing = false;
    bool use_graph = true;
    // implicit diffusion as one persistent cooperative kernel per step
    // (cooperative launch needed; otherwise the per-kernel sequence)
    bool persistent = true;
    int coop_blocks = 0;
    bool graph_persistent = false;
    long long iter_cap = 100000;   // PCG iterations per step before the step aborts
    long long spin_limit = cfg::gsync::kSpinLimit;   // grid-barrier spins before the step aborts
    double t_host = 0.0;
    long long steps = 0;
    // per-cell beat detector on Vm (cfg_monodomain_track_apd): sampled after
    // every apd_every-th step
    cfg::ApdTracker* d_apd = nullptr;
    double *d_apd_ring_t = nullptr, *d_apd_ring_v = nullptr;
    cfg::ApdParams apdp{};
    int apd_every = 0;
    long long apd_steps = 0;
    // time step a caller may leave to the context (cfg_monodomain_step with
    // dt = 0), and the explicit algorithm's Courant limit at maxCo = 1
    double delta_t = 0.0;
    double explicit_dt_unit = -1.0;
    // a coupled conduction network (cfg_purkinje_couple): its step runs
    // before the myocardium's, and the tissue's source of the step is
    // d_src_total (the network's buffer)
    cfg_purkinje* pk = nullptr;
    double* d_src_total = nullptr;
    // phase timing
    bool timing = false;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    double ionic_ms = 0.0, diffusion_ms = 0.0;
    long long timed_steps = 0;
    long long timed_launches = 0;
};

namespace cfg {
int monodomain_create(const cfg_monodomain_desc* d, const cfg_mesh_desc* m, cfg_monodomain** out);
int enqueue_step(cfg_monodomain* md, double dt, bool host_control);
int check_step(cfg_monodomain* md);
int build_step_graph(cfg_monodomain* md, double dt);
void fill_args_public(cfg_monodomain* md, double dt);
int coop_grid_blocks(long long n);
cudaError_t launch_implicit_coop(const DiffusionArgs& a, int blocks, cudaStream_t s);
// coupling of a conduction network (csrc/purkinje.cu)
int monodomain_attach_network(cfg_monodomain* md, cfg_purkinje* pk, double* src_total);
int monodomain_source_total(cfg_monodomain* md, double t0, const int* dep_off,
                            const int* dep_term, const double* dep_value, double* src_total);
int purkinje_prepare_coupled_step(cfg_purkinje* pk, cfg_monodomain* md, double t0, double dt);
int purkinje_check(cfg_purkinje* pk);
void purkinje_detach(cfg_purkinje* pk);
}  // namespace cfg
