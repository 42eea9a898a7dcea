// Host-side table of the ionic models compiled into the library: the
// GPU analogue of the ionicModel runtime-selection table
// (declareRunTimeSelectionTable in src/ionicModels/ionicModel/ionicModel.H:184-197).
#pragma once

#include <cuda_runtime.h>

#include "ionic_batch.cuh"
#include "ionic_kernels.cuh"

namespace cfg {

struct IonicModelOps {
    const char* name;            // ionicModel key
    int ns;                      // NUM_STATES
    int n_wide[2];               // states in the double array, per precision
    const int* wide_of;          // [2][ns] 1 if state i is double in that precision
    const int* slot_of;          // [2][ns] index in its array
    const char* const* state_names;
    const int* tissues;          // supported tissue flags, 0-terminated
    double iion_scale, time_scale;
    int vm_map;
    // launch one ionic step / the initialisation for a precision
    cudaError_t (*step[2][2])(const IonicLaunch&, cudaStream_t, int block);   // [prec][solve_vm]
    cudaError_t (*init[2])(long long n, int tissue, const unsigned char* tissue_cell,
                           const double* scales, long long stride, double init_step,
                           double* yw, float* yn, double* step, cudaStream_t);
    // host evaluation of initConsts (for checks and initial state export)
    void (*host_init)(double* C, double* y, int tissue, const double* scale);
    int nc;
    // batched single cells: initial states + trace sample 0, and one
    // work-stealing launch, per precision
    cudaError_t (*batch_init[2])(const BatchLaunch&, const double* scales, int tissue,
                                 double init_step, cudaStream_t);
    cudaError_t (*batch_step[2])(const BatchLaunch&, int tissue, cudaStream_t);
    int nsd;                     // scale-dependent constants per cell
    int ca_state;                // intracellular calcium state, or -1
    // sweepCurrent: the header's name tables, its dependency map (current ->
    // comma-separated variables, null-ended) and the FP64 sweep launch
    int na;                      // NUM_ALGEBRAIC
    const char* const* state_strings;
    const char* const* alg_strings;
    const char* const* sweep_currents;
    const char* const* sweep_deps;
    cudaError_t (*sweep)(const double* y0, const double* C, int tissue, int solve_vm,
                         const CfgStimulus& stim, double vmin, double vmax, int npts,
                         double t, int clamp, double* out, cudaStream_t);
    int (*max_block[2])();       // largest block the step kernel takes, per precision
};

const IonicModelOps* find_ionic_model(const char* name);
const char* ionic_model_names();   // "TNNP ORd ..." for error messages

}  // namespace cfg
