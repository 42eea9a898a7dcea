// Host representation of a GPU ionic model (one ionicModel instance).
#pragma once

#include <vector>

#include "host_common.h"
#include "ionic_registry.h"

struct cfg_ionic {
    const cfg::IonicModelOps* ops = nullptr;
    long long n = 0;
    int precision = CFG_PRECISION_FP64;
    bool solve_vm = false;
    int tissue = 0;
    cfg::OdeSettings ode{};
    cfg::CfgStimulus stim{};
    double* d_yw = nullptr;        // wide states, SoA: FP64, or FP32 (hi, lo) pairs (mixed)
    float* d_yn = nullptr;         // narrow (float) states, SoA (mixed form)
    double* d_step = nullptr;      // per-cell persistent ODE step
    double* d_vm = nullptr;        // staging for host-field solves
    double* d_im = nullptr;
    int* d_status = nullptr;
    unsigned long long* d_evals = nullptr;
    double* d_fail = nullptr;      // IonicFailure record of the first failing cell
    unsigned char* d_tissue = nullptr;   // per state slot
    double* d_scales = nullptr;
    // Per-cell tissue flags without conductance scales: the states are kept
    // grouped by tissue (slot k holds cell perm[k]) and each group runs the
    // kernel specialised for its tissue.
    struct Group {
        long long first, count;
        int tissue;
    };
    std::vector<Group> groups;
    std::vector<int> h_perm;
    int* d_perm = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // launch shape of the step kernel (cfg_ionic_autotune): threads per
    // block (0 = the kernel's largest) and cells per thread
    int block = 0;
    int cells_per_thread = 1;
};

namespace cfg {
OdeSettings make_ode(const cfg_ode_desc& d);
int ionic_validate(const cfg_ionic_desc* d, const IonicModelOps** model, int* tissue);
int ionic_create(const cfg_ionic_desc* d, cudaStream_t stream, cfg_ionic** out);
void ionic_free(cfg_ionic* ion);
IonicLaunch ionic_launch_args(const cfg_ionic* ion, double t0, double dt, const double* t_dev,
                              const double* vm_dev, double* im_dev);
cudaError_t ionic_enqueue(const cfg_ionic* ion, const IonicLaunch& L);
int ionic_check_status(cfg_ionic* ion);
int ionic_autotune(cfg_ionic* ion, double t0, double dt, const double* t_dev, const double* vm_dev,
                   int repeats, int* block, int* cells_per_thread, float* ms);
}  // namespace cfg
