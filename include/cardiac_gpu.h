/*
 * cardiac_gpu.h - C ABI of the GB300 monodomain time step.
 *
 * A plain-C boundary (pointers, sizes, status codes; no C++ or torch types)
 * that cardiacFoam's own C++ can call from a thin adapter, so that the
 * electroProperties dictionary and the runtime selection tables stay as they
 * are.  Every function returns CFG_OK (0) or a CFG_ERR_* code; the message of
 * the last failure on the calling thread is available from cfg_last_error().
 * A context is not re-entrant: one host thread and one CUDA stream per
 * context (the reference is single-threaded per MPI rank).
 *
 * Units follow the reference: PDE fields in SI (Vm [V], Im [V/s], time [s],
 * sources [A/m^3]); ionic model state in the model's own units.
 */
#ifndef CARDIAC_GPU_H
#define CARDIAC_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define CFG_OK 0
#define CFG_ERR_INVALID 1       /* bad argument, unknown model/tissue/key */
#define CFG_ERR_CUDA 2          /* a CUDA call failed */
#define CFG_ERR_ODE_STEPS 4     /* RKF45 exceeded maxSteps (ODESolver FatalError) */
#define CFG_ERR_NONFINITE 8     /* a NaN/Inf ionic current was produced */
#define CFG_ERR_PCG 16          /* PCG reached maxIter without converging */
#define CFG_ERR_UNSUPPORTED 32  /* combination not built (e.g. solver other than RKF45) */

#define CFG_PRECISION_FP64 0    /* plain form: FP64 throughout */
#define CFG_PRECISION_MIXED 1   /* FP32 currents/gates, FP64 Vm/concentrations/PCG */

/* Message of the last failure on this thread ("" when none). */
const char* cfg_last_error(void);

/* ------------------------------------------------------------ ionic model */

/* ODESolver dictionary keys (solver, absTol, relTol, maxSteps) plus the
 * adaptiveSolver keys; a negative value selects OpenFOAM's default. */
typedef struct cfg_ode_desc {
    const char* solver;          /* "RKF45" (NULL = "RKF45") */
    double abs_tol;              /* default 1e-15 */
    double rel_tol;              /* default 1e-4 */
    long long max_steps;         /* default 10000 */
    double safe_scale, min_scale, max_scale, alpha_increase, alpha_decrease;
} cfg_ode_desc;

/* singleCellStimulus sub-dictionary (StimulusProtocol, stimulusIO.H:32-53) */
typedef struct cfg_stimulus_desc {
    double stim_start, stim_period_s1, stim_duration, stim_amplitude;
    int nstim1;
    double stim_period_s2;
    int nstim2;
} cfg_stimulus_desc;

typedef struct cfg_ionic_desc {
    const char* ionic_model;          /* ionicModel key: TNNP ORd ToRORd_dynCl
                                         AlievPanfilov BuenoOrovio */
    const char* tissue;               /* tissue key: epicardialCells mCells
                                         endocardialCells myocyte */
    long long n_cells;                /* nIntegrationPoints */
    double initial_delta_t;           /* initialDeltaT [s]; the reference uses it
                                         as the first ODE step in ms */
    int solve_vm_within_ode;          /* solveVmWithinODESolver */
    int precision;                    /* CFG_PRECISION_* */
    cfg_ode_desc ode;
    cfg_stimulus_desc stimulus;       /* used only when solve_vm_within_ode */
    const unsigned char* tissue_per_cell;  /* optional host [n] tissue flags */
    const double* scales;             /* optional host [6][n] per-cell factors on
                                         GNa GCaL GKr GKs GK1 Gto */
} cfg_ionic_desc;

typedef struct cfg_ionic cfg_ionic;

/* ionicModel::New(dict, nIntegrationPoints, initialDeltaT,
 * solveVmWithinODESolver) - src/ionicModels/ionicModel/ionicModel.C:76-94,
 * including the tissue check of ionicSelector::selectTissue
 * (ionicSelector.C:32-53). */
int cfg_ionic_create(const cfg_ionic_desc* desc, cfg_ionic** out);

/* ionicModel::solveODE(t0, dt, Vm, Im) - ionicModel.H:250-256 (e.g.
 * TNNP.C:114-179) on HOST fields: copies Vm in and Im out. */
int cfg_ionic_solve(cfg_ionic* ion, double t0, double dt, const double* vm, double* im);

/* The same on device pointers, enqueued on the context's stream. */
int cfg_ionic_solve_device(cfg_ionic* ion, double t0, double dt, const double* vm_dev,
                           double* im_dev);

/* Autotuner (no reference counterpart): times every launch shape of the
 * step kernel - threads per block (32 .. the kernel's largest) x cells per
 * thread (1, 2, 4) - on scratch copies of the states with the given Vm
 * (device pointer; NULL = resting Vm) and keeps the fastest for this
 * context.  The results of a step do not depend on the launch shape. */
int cfg_ionic_autotune(cfg_ionic* ion, double t0, double dt, const double* vm_dev,
                       int* block, int* cells_per_thread, float* ms_per_step);
/* The same launch shape set directly (block 0 = the kernel's largest). */
int cfg_ionic_set_launch(cfg_ionic* ion, int block, int cells_per_thread);

/* Number of states and their names (ioNumStates/ioStateNames,
 * ionicModel.H:115-168). */
int cfg_ionic_num_states(const cfg_ionic* ion, int* n_states);
int cfg_ionic_state_name(const cfg_ionic* ion, int index, char* buf, size_t len);

/* State export/import as [n_states][n_cells] doubles (exportStates /
 * importFields, ionicModel.H:584-638). */
int cfg_ionic_get_states(cfg_ionic* ion, double* host_states);
int cfg_ionic_set_states(cfg_ionic* ion, const double* host_states);
/* Per-cell persistent ODE step (ionicModel::step(), ionicModel.H:244-247). */
int cfg_ionic_get_steps(cfg_ionic* ion, double* host_steps);
/* RHS evaluations since creation (work counter for the roofline). */
int cfg_ionic_rhs_evaluations(const cfg_ionic* ion, unsigned long long* count);
int cfg_ionic_destroy(cfg_ionic* ion);

/* availableSweepCurrents (e.g. TNNP.C:274-277): the keys of the model's
 * dependency map, space-separated. */
int cfg_ionic_sweep_currents(const cfg_ionic* ion, char* buf, size_t len);
/* sweepCurrent(currentName, Vmin, Vmax, nPts, file) (ionicModel.H:742-759,
 * e.g. TNNP.C:208-272): the states of integration point 0 with state 0
 * clamped to Vmin + (Vmax - Vmin) i / (nPts - 1) (model units), the model's
 * variables at VOI = 0, and the current's dependency columns resolved as
 * ionicModelIO does (Vm, STATE names, ALGEBRAIC names, RATES_<state>).
 * out: host [n_points][n_columns], column 0 = V; header: "V,<deps...>" as the
 * reference writes it.  With out = NULL only n_columns and header are set.
 * Evaluated in FP64 on the device, one thread per voltage. */
int cfg_ionic_sweep_current(cfg_ionic* ion, const char* current, double v_min, double v_max,
                            int n_points, double* out, int* n_columns, char* header,
                            size_t header_len);

/* The single-cell trace (ionicModelIO::writeHeader / write,
 * genericWriter/ionicModelIO.C:28-86,169-232, as SingleCellSolver writes it,
 * singleCellSolver.C:100-118,226-229): "time" and the column names, then per
 * call one row for integration point `cell` at time t [s]: t and the values,
 * fixed with 7 decimals.  columns = NULL or "" writes every variable (Vm -
 * transformed for AlievPanfilov and BuenoOrovio -, the other states, the
 * algebraics, RATES_<state>); otherwise the variableExport names (separated
 * by spaces or commas) resolved as ionicModelIO does, unknown ones ignored.
 * The algebraics and rates are those of the model's variables at t. */
int cfg_ionic_trace_header(const cfg_ionic* ion, const char* columns, char* buf, size_t len);
int cfg_ionic_trace_row(cfg_ionic* ion, long long cell, double t, const char* columns, char* buf,
                        size_t len);

/* -------------------------------------------------------- monodomain step */

/* lduMesh view of the myocardium: OpenFOAM's lower/upper addressing of the
 * internal faces (upper-triangular order), cell volumes and centres, and
 * either per-face coefficients face_coeff = deltaCoeffs * (Sf.sigma_f.Sf)/|Sf|
 * (upper() of fvm::laplacian(conductivity, Vm), gaussLaplacianScheme), or the
 * face geometry (Sf and deltaCoeffs) from which the library forms them with
 * the descriptor's uniform conductivity.  zeroGradient walls contribute
 * nothing to the matrix (myocardiumDomain.C:207).
 *
 * General (non-orthogonal) meshes give the full geometry instead: with
 * face_centres and the boundary faces the library assembles OpenFOAM's
 * "Gauss linear corrected" Laplacian of a tensor conductivity
 * (gaussLaplacianScheme::fvmLaplacian, finiteVolume of OpenFOAM v2312, the
 * version line the reference builds against): linear interpolation weights,
 * non-orthogonal deltaCoeffs 1/max(n.d, 0.05|d|) in the matrix, and in the
 * source, re-evaluated every PIMPLE corrector, the explicit face fluxes
 * SfGammaCorr.grad_f (conductivity not aligned with the face normal) plus
 * SfGammaSn corrVec.grad_f (non-orthogonal correction), grad the cell
 * gradient of Vm (leastSquares or Gauss linear) linearly interpolated to the
 * face; on the walls SfGammaCorr.grad_b with grad_b the zeroGradient wall
 * value of the gradient.  Replaces fvm::laplacian(conductivity_, Vm) of
 * monodomainSolver.C:129-136 on such meshes. */
typedef struct cfg_mesh_desc {
    long long n_cells, n_faces;
    const int* owner;            /* [n_faces] lower addressing */
    const int* neighbour;        /* [n_faces] upper addressing */
    const double* volumes;       /* [n_cells] */
    const double* centres;       /* [n_cells][3] */
    const double* face_coeff;    /* [n_faces], or NULL to use the geometry below */
    const double* face_sf;       /* [n_faces][3] face area vectors, owner -> neighbour */
    const double* face_delta_coeffs;  /* [n_faces] 1/|d_PN| */
    int structured[3];           /* nx ny nz when the cells are a blockMesh block
                                    (x fastest) with uniform coefficients per
                                    direction; {0,0,0} for a general mesh */
    /* full geometry of a general mesh (all NULL/0 otherwise) */
    const double* face_centres;  /* [n_faces][3] */
    long long n_boundary_faces;
    const int* boundary_cell;    /* [n_boundary_faces] cell of each wall face */
    const double* boundary_sf;   /* [n_boundary_faces][3] outward area vectors */
    const double* boundary_centres;  /* [n_boundary_faces][3] */
} cfg_mesh_desc;

#define CFG_GRAD_LEAST_SQUARES 0    /* gradSchemes default leastSquares (tutorials) */
#define CFG_GRAD_GAUSS_LINEAR 1     /* gradSchemes default Gauss linear */

/* monodomainSolverCoeffs (tutorials/electroProperties.template) plus
 * fvSchemes/fvSolution settings used by the step. */
typedef struct cfg_monodomain_desc {
    cfg_ionic_desc ionic;        /* n_cells must equal the mesh's */
    double conductivity[6];      /* xx xy xz yy yz zz [S/m]; used when the mesh
                                    gives geometry instead of face_coeff */
    double chi;                  /* [1/m] */
    double cm;                   /* [F/m^2] */
    int implicit;                /* solutionAlgorithm implicit (1) / explicit (0) */
    int ddt_backward;            /* ddtSchemes default backward (1) / Euler (0) */
    double pcg_tol, pcg_rel_tol; /* solvers Vm tolerance / relTol */
    int pcg_max_iter;            /* maxIter (default 1000) */
    int n_outer;                 /* PIMPLE nOuterCorrectors */
    double outer_tol;            /* PIMPLE residualControl Vm tolerance */
    double vm0;                  /* initial Vm [V] (MyocardiumDomain default -0.084) */
    int n_boxes;                 /* externalStimulus boxes (<= 8) */
    double box_min[8][3], box_max[8][3];
    double box_start[8], box_duration[8], box_intensity[8];
    /* general meshes only (the mesh gives face_centres): */
    const double* conductivity_per_cell;  /* optional host [n_cells][6] xx xy xz yy
                                             yz zz, a 0/conductivity volTensorField
                                             (monodomainSolver.C:48-100); wall faces
                                             take their cell's value */
    int grad_scheme;             /* CFG_GRAD_* of the explicit correction */
    int laplacian_uncorrected;   /* laplacianSchemes Gauss linear uncorrected (1):
                                    drops the non-orthogonal part of the
                                    correction, keeps the tangential one */
} cfg_monodomain_desc;

typedef struct cfg_monodomain cfg_monodomain;

/* MyocardiumDomain + MonodomainSolver construction (myocardiumDomain.C:180-304,
 * monodomainSolver.C:39-100) on the given mesh. */
int cfg_monodomain_create(const cfg_monodomain_desc* desc, const cfg_mesh_desc* mesh,
                          cfg_monodomain** out);

/* The same from the text of a constant/electroProperties file: selects
 * myocardiumSolver, reads <type>Coeffs (conductivity, chi, cm, ionicModel,
 * tissue, solutionAlgorithm, solver, absTol, relTol, maxSteps,
 * externalStimulus) as electroModel::New / myocardiumDomainInterface::New do
 * (electroModel.C:142-200, myocardiumDomainInterface.C:54-96).  fv_settings
 * may override ddt scheme / PCG tolerances (NULL = the tutorials' values);
 * `precision` picks the GPU form. */
int cfg_monodomain_create_from_dict(const char* electro_properties, const cfg_mesh_desc* mesh,
                                    double delta_t, int precision, cfg_monodomain** out);

/* MyocardiumDomain::suggestExplicitDeltaT(maxCo) (myocardiumDomain.C:532-550):
 * maxCo * min over internal faces of dx^2/Df, dx = 1/deltaCoeffs = |C_N - C_P|,
 * Df = n.(n.sigma_f)/(chi Cm) with sigma_f the linear interpolate of the
 * conductivity (needs the mesh's face_sf and centres). */
int cfg_monodomain_suggest_explicit_delta_t(const cfg_monodomain* md, double max_co, double* dt);

/* The context's time step: delta_t of the description, or, for an explicit
 * electroProperties read by cfg_monodomain_create_from_dict, the value
 * electroModel::setDeltaT sets once (electroModel.C:238-257):
 * suggestExplicitDeltaT(maxCo) with maxCo from the Coeffs' gpu sub-dictionary
 * (the reference reads it from controlDict), default 0.1.  A caller passes
 * dt = 0 to cfg_monodomain_step / cfg_monodomain_run to step with it, as
 * runTime does after setDeltaT. */
int cfg_monodomain_delta_t(const cfg_monodomain* md, double* dt);
int cfg_monodomain_set_delta_t(cfg_monodomain* md, double dt);

/* One time step: runTime++ then electroModel::evolve with the staggered
 * scheme (electroModel.C:297-330, myocardiumDomain.C:487-529): box stimulus,
 * ionic solveODE, implicit (PIMPLE + PCG) or explicit diffusion, activation
 * time.  dt = 0 steps with the context's time step (cfg_monodomain_delta_t). */
int cfg_monodomain_step(cfg_monodomain* md, double dt);

/* The autotuner on the context's ionic model with its current Vm and
 * time (see cfg_ionic_autotune); the step graph is rebuilt at the next step.
 * The ELL width of the operator is the mesh's longest row (exact: tets 4,
 * hexahedra 6), so there is nothing to choose there. */
int cfg_monodomain_autotune(cfg_monodomain* md, int* block, int* cells_per_thread,
                            float* ionic_ms);

/* n_steps steps replayed from the step's CUDA graph, whose PIMPLE and PCG
 * loops are conditional nodes driven by device-side solver state: no host
 * work per step beyond the launch, one status check at the end. */
int cfg_monodomain_run(cfg_monodomain* md, double dt, long long n_steps);

/* Use the step graph (1, default) or drive the PIMPLE/PCG loops from the
 * host, reading the solver state after every solve start and iteration pair
 * (0; for debugging; same results). */
int cfg_monodomain_set_graph(cfg_monodomain* md, int enable);

#define CFG_FIELD_VM 0              /* Vm [V] */
#define CFG_FIELD_IION 1            /* ionicCurrent [V/s] */
#define CFG_FIELD_ACTIVATION 2      /* activationTime [s] */
#define CFG_FIELD_SOURCE 3          /* externalStimulusCurrent [A/m^3] */
#define CFG_FIELD_VM_OLD 4          /* Vm.oldTime() [V] */
#define CFG_FIELD_PHIE 5            /* bidomain: extracellular potential phiE [V] */
#define CFG_FIELD_PHII 6            /* bidomain: intracellular potential phiI = Vm + phiE [V] */

/* Host copies of the domain's fields (written at output times only). */
int cfg_monodomain_get_field(cfg_monodomain* md, int field, double* host);
int cfg_monodomain_set_field(cfg_monodomain* md, int field, const double* host);
double cfg_monodomain_time(const cfg_monodomain* md);
cfg_ionic* cfg_monodomain_ionic(cfg_monodomain* md);

typedef struct cfg_step_stats {
    int n_solves;                  /* PIMPLE correctors run in the last step */
    int iterations[16];            /* PCG iterations per solve */
    double initial_residual[16];
    double final_residual[16];
} cfg_step_stats;
int cfg_monodomain_last_stats(const cfg_monodomain* md, cfg_step_stats* stats);

/* Per-phase device time, the GPU counterpart of electroModel's
 * electrophysicsAdvanceTimings (electroModel.H:81, staggered...C:50-75):
 * when enabled, CUDA events on the context's stream bracket the ionic and
 * the diffusion phase of every step and the milliseconds accumulate. */
int cfg_monodomain_set_timing(cfg_monodomain* md, int enable);
int cfg_monodomain_timings(const cfg_monodomain* md, double* ionic_ms, double* diffusion_ms,
                           long long* steps, long long* kernel_launches);
/* Implicit diffusion as one persistent cooperative kernel per step (all
 * PIMPLE correctors and PCG iterations inside one launch; the default where
 * the device supports cooperative launches), or as a kernel sequence per
 * iteration (enable = 0).  Same numerics up to the order of the reduction
 * sums.  MonodomainSolver::solveDiffusionImplicit (monodomainSolver.C:112-150)
 * is what either form computes. */
int cfg_monodomain_set_persistent(cfg_monodomain* md, int enable);
#define CFG_PCG_FP64 0          /* operator, vectors and sums in FP64 */
#define CFG_PCG_FLOAT_PAIRS 1   /* (hi, lo) float pairs, about 48 significant bits,
                                   on the FP32 pipe; the system scaled by a power
                                   of two */
/* Arithmetic of the persistent implicit solve: the PCG of
 * MonodomainSolver::solveDiffusionImplicit (monodomainSolver.C:112-150,
 * lduMatrix PCG with its normFactor and convergence test) in FP64, or in
 * float pairs, the default of CFG_PRECISION_MIXED contexts on meshes whose
 * Laplacian needs no explicit correction (GB300 issues FP64 at 1/64 of the
 * FP32 rate; on corrected meshes the solve streams from HBM and keeps
 * FP64).  The source of each corrector is formed in FP64 either way.  The
 * kernel sequence (cfg_monodomain_set_persistent(md, 0)) always runs FP64;
 * the explicit algorithm has no solve. */
int cfg_monodomain_set_pcg_arithmetic(cfg_monodomain* md, int arithmetic);
/* Per-cell beat detection on the tissue's Vm: after every `every_steps`-th
 * step (and once at the call, the field as it is) each cell's Vm [mV] and
 * the time go through the reference's restitution post-processing as a
 * streaming detector (postProcessing_restCurves.py:121-205: central dV/dt,
 * upstroke at 5000 mV/s, baseline the minimum over the 2 ms before it, v90
 * crossing after the peak).  No counterpart in the reference's tissue solver,
 * whose traces are post-processed offline; it states the APD90 of a tissue
 * run without copying its trace to the host.  every_steps <= 0 stops it.
 * The sampling interval is every_steps times the context's time step, and
 * the 2 ms baseline window may hold at most 4096 samples. */
int cfg_monodomain_track_apd(cfg_monodomain* md, int every_steps);
/* The tracked trace as it ends at the last sample: beats detected, the last
 * beat's APD90 [ms] (NaN if it has not repolarised) and its upstroke time
 * [s], per cell (host arrays of n_cells). */
int cfg_monodomain_apd_results(cfg_monodomain* md, int* n_beats, double* apd90_ms, double* t_up);
/* Bound on each grid-barrier wait of the persistent diffusion kernel, in
 * spins of at least 32 ns (default 2^25, about a second; a negative value
 * restores it).  A block that waits longer makes every block leave at its
 * next barrier and the step returns CFG_ERR_PCG ("a grid barrier timed out");
 * the context's fields are then those of a partial step.  No counterpart in
 * the reference (its solver runs on the host); an application sets it to
 * shorten the watchdog of a step. */
int cfg_monodomain_set_wait_limit(cfg_monodomain* md, long long spins);
/* The CUDA stream (cudaStream_t) all work of the context is enqueued on. */
void* cfg_monodomain_stream(cfg_monodomain* md);
int cfg_monodomain_destroy(cfg_monodomain* md);

/* ------------------------------------------------ batched single cells
 * SingleCellSolver (singleCellSolver.C:45-230: runTime++; solveODE(t - dt,
 * dt) with Vm inside the ODE) for many independent cells in one persistent,
 * work-stealing launch: each cell has its own conductance scales, S1/S2
 * protocol (singleCellStimulus, stimulusIO.H:32-53) and end time.  The
 * restitution post-processing of the traces (postProcessing_restCurves.py:
 * upstroke where dV/dt crosses 5000 mV/s, baseline = minimum over the 2 ms
 * before it, APD90 at 90 % repolarisation, windows up to 2 s or the next
 * upstroke) runs on the device while the cells are stepped, together with
 * the peak intracellular Ca of each beat. */
typedef struct cfg_batch_desc {
    const char* ionic_model;           /* ionicModel key */
    const char* tissue;                /* tissue key (one for all cells) */
    long long n_cells;
    double delta_t;                    /* deltaT [s]: solver step, and first ODE step */
    int precision;                     /* CFG_PRECISION_* */
    cfg_ode_desc ode;
    const cfg_stimulus_desc* stimulus; /* host [n_cells] protocols, model time units */
    const double* end_time;            /* host [n_cells] endTime [s] */
    const double* scales;              /* optional host [6][n_cells] factors on
                                          GNa GCaL GKr GKs GK1 Gto */
    long long trace_cells;             /* keep the Vm and Ca traces of cells
                                          [0, trace_cells) */
    long long trace_samples;           /* samples kept per traced cell, from t = 0 */
    long long chunk;                   /* solver steps per claim (0: 2000) */
} cfg_batch_desc;

typedef struct cfg_batch cfg_batch;

int cfg_batch_create(const cfg_batch_desc* desc, cfg_batch** out);
/* Advance every cell to its end time; returns after the last launch. */
int cfg_batch_run(cfg_batch* b);
/* Per cell: beats detected, last beat's APD90 [ms] (NaN when it did not
 * repolarise inside its window), upstroke time [s] and peak Ca. */
int cfg_batch_results(cfg_batch* b, int* n_beats, double* apd90_ms, double* t_up,
                      double* peak_ca);
/* Traces as [trace_cells][2][trace_samples]: Vm [mV] then Ca. */
int cfg_batch_trace(cfg_batch* b, double* host);
/* Final states as [n_states][n_cells]. */
int cfg_batch_get_states(cfg_batch* b, double* host_states);
/* RHS evaluations, solver steps taken and kernel launches since creation. */
int cfg_batch_stats(const cfg_batch* b, unsigned long long* rhs_evaluations,
                    long long* solver_steps, long long* launches);
/* The CUDA stream (cudaStream_t) the batch runs on. */
void* cfg_batch_stream(cfg_batch* b);
int cfg_batch_destroy(cfg_batch* b);

/* ------------------------------------------------------ adjoint step
 *
 * No reference counterpart: the differentiable form of the monodomain step
 * and its adjoint, for gradients of a probe-voltage misfit
 *   J = sum over sampled steps and probe cells of (Vm - target)^2
 * with respect to per-cell log-scale fields of two conductances (TNNP g_Na
 * and g_K1: g = g0 exp(theta)) and the conductivities sigma_l, sigma_t of
 * sigma = sigma_t I + (sigma_l - sigma_t) f f (f the fibre direction).
 * The forward runs the ionic update with a fixed number of RKF45 substeps
 * per PDE step (no step-size control, so J is a smooth function of the
 * parameters), implicit Euler diffusion with one PCG solve per step on an
 * orthogonal mesh (no explicit correction), and keeps a checkpoint every
 * checkpoint_every steps; the backward recomputes each window from its
 * checkpoint and runs the adjoint kernels back through it. */
typedef struct cfg_adjoint_desc {
    const char* ionic_model;     /* "TNNP" */
    const char* tissue;          /* tissue key */
    double delta_t;              /* PDE step [s] */
    long long n_steps;
    int substeps;                /* RKF45 substeps per PDE step (1..16) */
    int checkpoint_every;        /* steps between checkpoints */
    int sample_every;            /* steps between probe samples */
    int n_probes;
    const int* probes;           /* [n_probes] probe cells */
    double chi, cm, vm0;
    double fibre[3];             /* fibre direction of sigma_l */
    int n_boxes;
    double box_min[8][3], box_max[8][3];
    double box_start[8], box_duration[8], box_intensity[8];
    double pcg_tol;              /* ||r||_2 <= pcg_tol ||b||_2 for both solves */
    int pcg_max_iter;
    int precision;               /* CFG_PRECISION_FP64, or _MIXED: the ionic right-hand
                                    side and its derivative in FP32, states and
                                    adjoint accumulations in FP64 */
} cfg_adjoint_desc;

typedef struct cfg_adjoint cfg_adjoint;

int cfg_adjoint_create(const cfg_adjoint_desc* desc, const cfg_mesh_desc* mesh,
                       cfg_adjoint** out);
/* target[n_steps / sample_every][n_probes] of the misfit */
int cfg_adjoint_set_target(cfg_adjoint* adj, const double* target);
/* Forward run from the model's initial states and Vm0: J and (optional)
 * the probe trace [n_samples][n_probes]. */
int cfg_adjoint_forward(cfg_adjoint* adj, const double* log_gna, const double* log_gk1,
                        double sigma_l, double sigma_t, double* loss, double* probe_trace);
/* dJ/dlog_gna [n], dJ/dlog_gk1 [n], dJ/d(sigma_l, sigma_t) [2] at the
 * parameters of the last forward run. */
int cfg_adjoint_backward(cfg_adjoint* adj, double* grad_log_gna, double* grad_log_gk1,
                         double* grad_sigma);
int cfg_adjoint_destroy(cfg_adjoint* adj);

/* ------------------------------------------------------------- bidomain
 * MyocardiumDomain with myocardiumSolver bidomainSolver (bidomainSolver.C:
 * 36-263): per PIMPLE corrector
 *   fvm::laplacian(Gi + Ge, phiE) == -fvc::div(Gi & fvc::grad(Vm)),
 *     setReference(the cell at phiERefPoint, phiEReferenceValue, true);
 *   chi Cm fvm::ddt(Vm) == fvm::laplacian(Gi, Vm) + fvc::div(Gi & fvc::grad(phiE))
 *     - chi Cm Iion + src;
 *   phiI = Vm + phiE,
 * after the box stimulus and the ionic update of the step, then the
 * activation time.  Diffusion in FP64 with diagonal-preconditioned PCG (the
 * reference's lduMatrix convergence test); gradients by gradSchemes default,
 * divergence Gauss linear.  Uniform conductivity tensors; the mesh needs its
 * full geometry, and meshes whose Laplacians need explicit non-orthogonal or
 * tangential corrections are CFG_ERR_UNSUPPORTED.  The reference cell is the
 * cell whose centre is nearest to ref_point (the first on ties). */
typedef struct cfg_bidomain_desc {
    cfg_ionic_desc ionic;            /* n_cells must equal the mesh's */
    double conductivity_i[6];        /* conductivityIntracellular xx xy xz yy yz zz */
    double conductivity_e[6];        /* conductivityExtracellular */
    double chi, cm;
    int ddt_backward;                /* ddt(Vm) backward (1) / Euler (0) */
    double pcg_tol, pcg_rel_tol;     /* Vm solver */
    int pcg_max_iter;
    double phie_tol, phie_rel_tol;   /* phiE solver */
    int phie_max_iter;
    int n_outer;                     /* PIMPLE nOuterCorrectors */
    double outer_tol;                /* residualControl on Vm (0: none) */
    double vm0;                      /* initial Vm [V] */
    double ref_point[3];             /* phiERefPoint */
    double ref_value;                /* phiEReferenceValue */
    int n_boxes;
    double box_min[8][3], box_max[8][3];
    double box_start[8], box_duration[8], box_intensity[8];
    int grad_scheme;                 /* CFG_GRAD_* */
    int explicit_algorithm;          /* solutionAlgorithm explicit (1): phiE solved as in
                                        the implicit form, then Vm from
                                        chi Cm ddt(Vm) == div(Gi grad(Vm + phiE))
                                        - chi Cm Iion + src with the diagonal ddt matrix
                                        (bidomainSolver.C:183-213), no PIMPLE loop */
} cfg_bidomain_desc;

typedef struct cfg_bidomain cfg_bidomain;

int cfg_bidomain_create(const cfg_bidomain_desc* desc, const cfg_mesh_desc* mesh,
                        cfg_bidomain** out);
/* The same from the text of a constant/electroProperties file with
 * myocardiumSolver bidomainSolver: bidomainSolverCoeffs' conductivityIntracellular,
 * conductivityExtracellular, phiERefPoint, phiEReferenceValue, chi, cm, the ionic
 * model keys and externalStimulus (bidomainSolver.C:36-127, as
 * cfg_monodomain_create_from_dict for the rest).  Solver settings are the
 * bidomain tutorial's (relTol 0 / maxIter 1000 for Vm and phiE,
 * nOuterCorrectors 2, backward ddt, Gauss linear gradients) with PCG
 * tolerance 1e-12 instead of its 1e-15 (rarely reached in double precision
 * within maxIter, which is an error here); a "gpu"
 * sub-dictionary may override them (tolerance, relTol, maxIter, phiETolerance,
 * phiERelTol, phiEMaxIter, nOuterCorrectors, residualControl, ddtScheme,
 * gradScheme). */
int cfg_bidomain_create_from_dict(const char* electro_properties, const cfg_mesh_desc* mesh,
                                  double delta_t, int precision, cfg_bidomain** out);
/* Arithmetic of the cooperative PCG solves of both bidomain systems (the
 * phiE and Vm solves of BidomainSolver, bidomainSolver.C:201-245, lduMatrix
 * PCG): CFG_PCG_FP64, or CFG_PCG_FLOAT_PAIRS, the default of
 * CFG_PRECISION_MIXED contexts.  The systems are assembled in FP64 either
 * way; float pairs need the cooperative solve (CFG_ERR_UNSUPPORTED where
 * the device has none). */
int cfg_bidomain_set_pcg_arithmetic(cfg_bidomain* bd, int arithmetic);
/* One time step (runTime++ then the staggered advance, as
 * cfg_monodomain_step). */
int cfg_bidomain_step(cfg_bidomain* bd, double dt);
int cfg_bidomain_run(cfg_bidomain* bd, double dt, long long n_steps);
/* CFG_FIELD_VM, _IION, _ACTIVATION, _SOURCE, _VM_OLD, _PHIE, _PHII */
int cfg_bidomain_get_field(cfg_bidomain* bd, int field, double* host);
int cfg_bidomain_set_field(cfg_bidomain* bd, int field, const double* host);
/* Device address of a field (CFG_FIELD_*; NULL for an unknown one), valid
 * until cfg_bidomain_destroy; work on it belongs on cfg_bidomain_stream. */
const double* cfg_bidomain_device_field(cfg_bidomain* bd, int field);
/* The last step's Vm and phiE solves (one of each per corrector). */
int cfg_bidomain_last_stats(const cfg_bidomain* bd, cfg_step_stats* vm, cfg_step_stats* phie);
double cfg_bidomain_time(const cfg_bidomain* bd);
long long cfg_bidomain_reference_cell(const cfg_bidomain* bd);
cfg_ionic* cfg_bidomain_ionic(cfg_bidomain* bd);
void* cfg_bidomain_stream(cfg_bidomain* bd);
int cfg_bidomain_destroy(cfg_bidomain* bd);

/* ----------------------------------------------------------- pseudo-ECG
 * ECGDomain with the pseudoECG solver (ecgDomain.C:119-159,
 * pseudoECGSolver.C:34-87): at each electrode P
 *   phi(P) = sum over cells c of ((sigma_c & grad(Vm)_c) V_c) & r / |r|^3,
 *   r = C_c - P, cells with |r| <= VSMALL skipped,
 * grad the mesh's gradSchemes default (leastSquares or Gauss linear) with
 * zeroGradient walls.  The mesh, the conductivity and the electrodes are
 * fixed for the object's life, so phi is a fixed linear functional of Vm:
 * creation folds the gradient weights and the dipole geometry into one row
 * of n_cells coefficients per electrode (8 bytes per cell and electrode in
 * device memory) and every evaluation is one pass over those rows and Vm.
 * The mesh needs its full geometry (face_centres, walls). */
#define CFG_ECG_FP64 0          /* FP64 multiply-add per cell and electrode */
#define CFG_ECG_FLOAT_PAIRS 1   /* float pairs: rows and Vm each carried to 48
                                   significant bits, error-free products and
                                   two-sum accumulation on the FP32 pipe; same
                                   bytes, a sixth of the FP64 operations' time */
typedef struct cfg_pseudo_ecg_desc {
    double conductivity[6];              /* xx xy xz yy yz zz, used when ... */
    const double* conductivity_per_cell; /* ... this is NULL; else host [n_cells][6] */
    int grad_scheme;                     /* CFG_GRAD_* */
    int n_electrodes;
    const double* electrodes;            /* host [n_electrodes][3] positions [m] */
    long long max_rows;                  /* rows of the device time series (0: none) */
    int arithmetic;                      /* CFG_ECG_* */
} cfg_pseudo_ecg_desc;

typedef struct cfg_pseudo_ecg cfg_pseudo_ecg;

int cfg_pseudo_ecg_create(const cfg_pseudo_ecg_desc* desc, const cfg_mesh_desc* mesh,
                          cfg_pseudo_ecg** out);
/* phi at every electrode of the device field vm [n_cells] into host
 * values [n_electrodes]; stream is a cudaStream_t (NULL: the legacy default
 * stream) and the call returns when the values are on the host. */
int cfg_pseudo_ecg_compute(cfg_pseudo_ecg* ecg, const double* vm, void* stream, double* values);
/* The same for a monodomain context's Vm on its stream. */
int cfg_pseudo_ecg_compute_monodomain(cfg_pseudo_ecg* ecg, cfg_monodomain* md, double* values);
/* ECGDomain::evolve (ecgDomain.C:167-190) after a monodomain step: phi of
 * the context's Vm appended to the device time series with the context's
 * time, enqueued on its stream without waiting (CFG_ERR_INVALID when the
 * series is full). */
int cfg_pseudo_ecg_record(cfg_pseudo_ecg* ecg, cfg_monodomain* md);
/* The same for a device field vm [n_cells] at time t, enqueued on stream. */
int cfg_pseudo_ecg_record_field(cfg_pseudo_ecg* ecg, const double* vm, void* stream, double t);
/* The recorded rows: times [rows], values [rows][n_electrodes] (host; up to
 * max_rows of them); *n_rows the number recorded.  reset empties the series. */
int cfg_pseudo_ecg_series(cfg_pseudo_ecg* ecg, double* times, double* values,
                          long long max_rows, long long* n_rows);
int cfg_pseudo_ecg_reset(cfg_pseudo_ecg* ecg);
/* Bound on each wait of the staged pseudo-ECG kernel for its tile copies, in
 * clock cycles (default 2^31, about a second; a negative value restores it).
 * A wait that runs out makes that evaluation's values NaN and the call that
 * reads them (compute, series) return CFG_ERR_CUDA, after which the flag is
 * cleared and the object is usable again.  No counterpart in the reference. */
int cfg_pseudo_ecg_set_wait_limit(cfg_pseudo_ecg* ecg, long long cycles);
int cfg_pseudo_ecg_destroy(cfg_pseudo_ecg* ecg);

/* Electrodes of an ecgDomains entry of constant/electroProperties
 * (<type>Coeffs.ecgDomains.<domain>: ecgSolver pseudoECG; electrodePositions
 * { name (x y z); ... }, ecgDomain.C:53-82): names space-separated into
 * names[len] in the dictionary's order, positions into [max][3].  domain
 * NULL or "" takes the first ecgDomains entry.  An ecgSolver other than
 * pseudoECG is CFG_ERR_UNSUPPORTED. */
int cfg_pseudo_ecg_electrodes_from_dict(const char* electro_properties, const char* domain,
                                        char* names, size_t len, double* positions, int max,
                                        int* n_electrodes);

/* ------------------------------------------------- Purkinje network
 * ConductionSystemDomain with the Monodomain1DSolver
 * (src/electroModels/conductionSystemModels/monodomain1DSolver/
 * monodomain1DSolver.C:36-190; conductionSystemDomain.C, conductionGraph.H):
 * a tree of nodes joined by edges of given length and conductance
 * (conductionEdges (nodeA nodeB length conductance) of the graph file), node 0
 * the root, Strang-split steps (ionic model over dt/2, the implicit cable step
 * solved exactly by Hines elimination, ionic model over dt/2), a root
 * stimulus (rootStimulus: node, startTime, duration, intensity; applied while
 * startTime <= t0 <= startTime + duration) and terminals (pvjNodes,
 * pvjLocations) where the network meets the tissue.  The ionic description's
 * n_cells is the node count (largest node index + 1) and its
 * solve_vm_within_ode 0; nodes start at the model's resting Vm
 * (ionicModel::vmRest). */
typedef struct cfg_purkinje_desc {
    cfg_ionic_desc ionic;
    long long n_edges;                 /* the nodes - 1 of a tree */
    const int* edge_a;                 /* [n_edges] */
    const int* edge_b;
    const double* edge_length;         /* [m] */
    const double* edge_conductance;    /* [S/m] */
    double chi, cm;
    int root_node;
    double root_start, root_duration, root_intensity;   /* start 1e300: no stimulus */
    int n_pvj;
    const int* pvj_nodes;              /* [n_pvj] */
    const double* pvj_locations;       /* [n_pvj][3] */
} cfg_purkinje_desc;

typedef struct cfg_purkinje cfg_purkinje;

int cfg_purkinje_create(const cfg_purkinje_desc* desc, cfg_purkinje** out);
/* One step of the network alone, Monodomain1DSolver::advance(t, dt), t then
 * advanced by dt (CFG_ERR_INVALID once the network is coupled). */
int cfg_purkinje_step(cfg_purkinje* pk, double dt);
/* ReactionDiffusionPvjCoupler between the network and a monodomain context
 * (reactionDiffusionPvjCoupler.C:36-164, pvjMapper.C): rPvj, pvjRadius and
 * couplingMode (bidirectional 1, unidirectional 0).  Each terminal maps to
 * the cell holding it (here the nearest cell centre, the first on ties) and
 * to the cells whose centres lie within pvjRadius (or that cell alone);
 * pvjRadius below the cube root of that cell's volume is rejected.  From
 * then on every cfg_monodomain_step / _run of the context runs the
 * staggered scheme's coupled step: the terminals' currents (Vnet -
 * Vtissue)/rPvj, the network's step with them as negative applied currents
 * (zero in unidirectional mode), the currents again from the new network
 * Vm, deposited as current/sphere volume into the tissue's source on top of
 * the box stimulus, then the myocardium's step.  `mesh` is the context's
 * mesh (centres and volumes are read). */
int cfg_purkinje_couple(cfg_purkinje* pk, cfg_monodomain* md, const cfg_mesh_desc* mesh,
                        double r_pvj, double pvj_radius, int bidirectional);
/* CFG_FIELD_VM [V] or CFG_FIELD_IION of the nodes (host, n nodes). */
int cfg_purkinje_get_field(cfg_purkinje* pk, int field, double* host);
/* The terminals' coupling currents of the last evaluation (host, n_pvj). */
int cfg_purkinje_terminal_current(cfg_purkinje* pk, double* host);
long long cfg_purkinje_nodes(const cfg_purkinje* pk);
double cfg_purkinje_time(const cfg_purkinje* pk);
/* Detaches from the coupled context, then frees the network. */
int cfg_purkinje_destroy(cfg_purkinje* pk);

/* ------------------------------------ diffusion solve without allocation
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * when they need a solve (a host application that owns all device memory
 * through its own pool, or one that cannot take the device-wide
 * synchronisation of cudaFree/cudaMalloc in the middle of a step): one
 * implicit diffusion corrector of the monodomain equation
 *   chi*Cm*ddt(Vm) - laplacian(sigma, Vm) = -chi*Cm*Iion
 * on a structured box (x fastest, uniform cells, one face coefficient per
 * direction), solved with the monodomain step's own PCG kernels, and no
 * device memory allocated: the temporaries live in one static device array
 * of CFG_NOALLOC_SCRATCH_BYTES, held on every GPU that loads the library
 * until the process exits.  Boxes above CFG_NOALLOC_MAX_CELLS cells are
 * rejected with CFG_ERR_INVALID.
 *
 * vm_old, vm_oldold (backward ddt only; may be NULL for Euler), iion are
 * read; vm holds the initial guess on entry and the solution on return;
 * all are device pointers of nx*ny*nz doubles.  stream is a cudaStream_t
 * (NULL: the legacy default stream); the call returns after the solve
 * finished.  The first call on a device looks up the array's address with
 * that device current and keeps it for the process: make it before any
 * stream capture on the device.  The address belongs to the device's
 * primary context as it was at that call; after cudaDeviceReset (or any
 * reset of the primary context) the entry point must not be called again in
 * the same process.  Every call shares the array: calls that overlap on the
 * GPU race. */
#define CFG_NOALLOC_MAX_CELLS 65536
#define CFG_NOALLOC_SCRATCH_BYTES 7880704   /* 15 vectors of 64 Ki doubles + state */

typedef struct cfg_box_diffusion_desc {
    int nx, ny, nz;                /* cells per direction */
    double cell_volume;            /* [m^3] */
    double face_coeff[3];          /* deltaCoeffs*(Sf.sigma.Sf)/|Sf| of x, y, z faces */
    double chi, cm;                /* surface-to-volume ratio, membrane capacitance */
    int ddt_backward;              /* 0: Euler, 1: backward with both old levels */
    double pcg_tol, pcg_rel_tol;
    int pcg_max_iter;
} cfg_box_diffusion_desc;

typedef struct cfg_solve_result {
    int iterations;
    int converged;                 /* 0 when maxIter ended the solve */
    double initial_residual, final_residual;
} cfg_solve_result;

int cfg_box_diffusion_solve_noalloc(const cfg_box_diffusion_desc* desc, double delta_t,
                                    const double* vm_old, const double* vm_oldold,
                                    const double* iion, double* vm, void* stream,
                                    cfg_solve_result* result);

#ifdef __cplusplus
}
#endif
#endif
