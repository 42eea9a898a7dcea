/* CPU oracle for the monodomain time step - TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithm for cardiacFoam's
 * MonodomainSolver step, used by tests/, the smoke check and bench.py's CPU
 * baseline leg as the checker; the product never links it.
 *
 *  - ionic update: <Model>::solveODE (e.g. src/ionicModels/TNNP/TNNP.C:114-179)
 *    driving OpenFOAM's RKF45 ODESolver (restated from the published
 *    Fehlberg 4(5) method and OpenFOAM's adaptiveSolver/ODESolver step control,
 *    which live outside the reference tree);
 *  - box stimulus and activation time: MyocardiumDomain
 *    (src/electroModels/electroDomains/myocardiumDomain/myocardiumDomain.C:307-374);
 *  - diffusion: MonodomainSolver::solveDiffusionImplicit/Explicit
 *    (src/electroModels/myocardiumModels/monodomainSolver/monodomainSolver.C:103-150)
 *    with OpenFOAM's Gauss-linear-corrected Laplacian, Euler/backward ddt,
 *    lduMatrix PCG with DIC or diagonal preconditioning, and the PIMPLE
 *    residual control of the tutorials' fvSolution - restated.
 *
 * Parity status: the ionic right-hand sides are pinned bit-for-bit against
 * the reference's own generated headers (golden vectors under tests/golden);
 * RKF45 is pinned by the reference's single-cell regression values; the
 * explicit tissue step by the NiedererEtAl2012 regression probes (all six
 * within the reference's tolerances on OpenFOAM's rounding of the case's
 * cell centres, oracle_blockmesh_centres); the implicit PCG path has no
 * reference test and is "parity unpinned"; so is
 * the corrected Laplacian on general meshes, restated from OpenFOAM v2312's
 * finiteVolume library (absent from the reference tree).
 */
#ifndef ORACLE_H
#define ORACLE_H

#include "oracle_common.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_TNNP = 0, ORACLE_ORD = 1, ORACLE_TORORD = 2, ORACLE_ALIEV = 3,
       ORACLE_BUENO = 4, ORACLE_MMS = 5, ORACLE_BIDOMAIN_MMS = 6, ORACLE_NMODELS = 7 };

/* --- model-level entry points (golden-vector pins) --------------------- */
int oracle_model_sizes(int model, int* ns, int* na, int* nc);
void oracle_model_init(int model, int tissue, double* C, double* y, const double* scale);
/* constants the reference's initConsts leaves unset (ORd's Na/K pump and
 * upScale); the ionic and tissue paths apply it after oracle_model_init */
void oracle_model_supplement(int model, double* C);
void oracle_model_rates(int model, double t, const double* C, const double* y,
                        double* dydt, double* alg, int tissue, int solve_vm,
                        const oracle_stimulus* stim);
void oracle_model_variables(int model, double t, const double* C, const double* y,
                            double* rates, double* alg, int tissue, int solve_vm,
                            const oracle_stimulus* stim);
int oracle_model_iion_index(int model);

/* --- ODE solver settings (ODESolver/adaptiveSolver dictionary keys) ----- */
typedef struct oracle_ode_settings {
    double abs_tol, rel_tol;     /* absTol (default 1e-15), relTol (1e-4) */
    long max_steps;              /* maxSteps (10000) */
    double safe_scale, min_scale, max_scale, alpha_inc, alpha_dec;
} oracle_ode_settings;
void oracle_ode_default(oracle_ode_settings* s);

/* --- ionic model over N cells (one ionicModel instance) ----------------- */
typedef struct oracle_ionic oracle_ionic;
oracle_ionic* oracle_ionic_new(int model, long n, int tissue, double initial_dt,
                               int solve_vm, const oracle_ode_settings* ode,
                               const oracle_stimulus* stim, const double* scales);
/* per-cell tissue flags (NULL: `tissue` for every cell) */
oracle_ionic* oracle_ionic_new_cells(int model, long n, int tissue,
                                     const unsigned char* tissue_cell, double initial_dt,
                                     int solve_vm, const oracle_ode_settings* ode,
                                     const oracle_stimulus* stim, const double* scales);
void oracle_ionic_free(oracle_ionic*);
/* ionicModel::solveODE(t0 [s], dt [s], Vm [V], Im [V/s]); returns the total
 * number of accepted RKF45 substeps, or -1 on maxSteps overflow.  nthreads>1
 * splits the independent cells over OpenMP threads. */
long oracle_ionic_solve(oracle_ionic*, double t0, double dt, const double* vm,
                        double* im, int nthreads);
double* oracle_ionic_states(oracle_ionic*);   /* AoS: cell*ns + i */
double* oracle_ionic_steps(oracle_ionic*);
long oracle_ionic_rhs_evals(oracle_ionic*);

/* --- structured hex mesh (blockMesh single block, x fastest) ------------ */
typedef struct oracle_mesh oracle_mesh;
oracle_mesh* oracle_mesh_box(int nx, int ny, int nz, double lx, double ly, double lz);
void oracle_mesh_free(oracle_mesh*);
long oracle_mesh_ncells(const oracle_mesh*);
long oracle_mesh_nfaces(const oracle_mesh*);
void oracle_mesh_addressing(const oracle_mesh*, int* owner, int* neighbour);
void oracle_mesh_centres(const oracle_mesh*, double* c);
/* Cell centres of one uniformly graded blockMesh block as OpenFOAM's
 * geometry code rounds them (block point interpolation, face and cell
 * centres in polyMesh face order); contract: fma fusion bits (1 blockMesh
 * weights, 2 cross, 4 dot, 8 magSqr); extent: far block vertex before
 * `scale`; patch_order: block faces 0..5 (x-min x-max y-min y-max z-min
 * z-max) in the boundary patch's order.  0 on success. */
int oracle_blockmesh_centres(int ni, int nj, int nk, const double* extent, double scale,
                             const int* patch_order, int contract, double* centres);
/* --- general mesh: lduAddressing plus the geometry of fvMesh ----------- */
oracle_mesh* oracle_mesh_general(long n, long nf, const int* owner, const int* neigh,
                                 const double* centres, const double* vol,
                                 const double* face_centres, const double* face_sf, long nb,
                                 const int* bcell, const double* bsf, const double* bcf);

/* --- monodomain tissue model -------------------------------------------- */
typedef struct oracle_tissue_desc {
    int model, tissue;
    double sigma[6];                 /* xx xy xz yy yz zz [S/m] */
    double chi, cm;                  /* [1/m], [F/m^2] */
    int implicit;                    /* solutionAlgorithm implicit/explicit */
    int ddt_backward;                /* ddtSchemes backward (1) or Euler (0) */
    int precond_dic;                 /* 1 = DIC, 0 = diagonal */
    double pcg_tol, pcg_rel_tol;     /* fvSolution solver tolerance / relTol */
    int pcg_max_iter;                /* default 1000 */
    int n_outer;                     /* PIMPLE nOuterCorrectors */
    double outer_tol;                /* PIMPLE residualControl tolerance */
    double vm0;                      /* initial Vm [V] (-0.084) */
    int n_boxes;
    double box_min[8][3], box_max[8][3];
    double box_start[8], box_duration[8], box_intensity[8];   /* s, s, A/m^3 */
    oracle_ode_settings ode;
    /* general meshes (fvSchemes): gradSchemes default leastSquares (0) or
     * Gauss linear (1); laplacianSchemes Gauss linear corrected (0) or
     * uncorrected (1) */
    int grad_gauss;
    int uncorrected;
} oracle_tissue_desc;

typedef struct oracle_tissue oracle_tissue;
oracle_tissue* oracle_tissue_new(const oracle_tissue_desc*, const oracle_mesh*);
void oracle_tissue_free(oracle_tissue*);
/* One runTime++ / evolve(): returns PCG iterations of the step (all outer
 * correctors), or -1 on failure.  `nthreads` parallelises the ionic loop. */
int oracle_tissue_init_ionic(oracle_tissue* T, double dt);
int oracle_tissue_step(oracle_tissue*, double dt, int nthreads);
double oracle_tissue_time(const oracle_tissue*);
double* oracle_tissue_vm(oracle_tissue*);
double* oracle_tissue_iion(oracle_tissue*);
double* oracle_tissue_activation(oracle_tissue*);
double* oracle_tissue_source(oracle_tissue*);
oracle_ionic* oracle_tissue_ionic(oracle_tissue*);
int oracle_tissue_last_solves(const oracle_tissue*, double* init_res, double* final_res,
                              int* iters, int max_solves);
/* per-cell conductivity [n][6] (xx xy xz yy yz zz); re-assembles */
void oracle_tissue_set_conductivity(oracle_tissue*, const double* sigma6);
/* per-cell tissue flags for the ionic model, before the first step */
int oracle_tissue_set_cell_tissue(oracle_tissue*, const unsigned char* flags);
/* fvc::laplacian(sigma, phi) [per volume] and the cell gradient of phi */
void oracle_tissue_laplacian(oracle_tissue*, const double* phi, double* out);
int oracle_tissue_gradient(oracle_tissue*, const double* phi, double* g);
/* bidomain (BidomainSolver) on a general mesh: d carries Gi, the Vm solver
 * settings, the ionic model and the stimulus; sigma_e is Ge */
typedef struct oracle_bidomain oracle_bidomain;
oracle_bidomain* oracle_bidomain_new(const oracle_tissue_desc* d, const double* sigma_e,
                                     const oracle_mesh* mesh, const double* ref_point,
                                     double ref_value, double phie_tol, double phie_rel_tol,
                                     int phie_max_iter);
void oracle_bidomain_free(oracle_bidomain*);
int oracle_bidomain_step(oracle_bidomain*, double dt, int nthreads);
oracle_tissue* oracle_bidomain_tissue(oracle_bidomain*);
double* oracle_bidomain_phie(oracle_bidomain*);
double* oracle_bidomain_phii(oracle_bidomain*);
long oracle_bidomain_ref_cell(const oracle_bidomain*);
int oracle_bidomain_last_solves(const oracle_bidomain*, double* init_res, double* final_res,
                                int* iters, int max_solves);
/* the pseudo-ECG of a Vm field at n_el electrodes [n_el][3] (general mesh) */
int oracle_tissue_pseudo_ecg(oracle_tissue*, const double* vm, int n_el, const double* el,
                             double* out);

/* --- single cell (SingleCellSolver::evolve) ------------------------------ */
/* Runs n_steps of dt [s] from t=0 with Vm inside the ODE; writes the
 * membrane potential in mV after each step into vm_trace (n_steps values). */
long oracle_single_cell(int model, int tissue, double dt, long n_steps,
                        const oracle_ode_settings* ode, const oracle_stimulus* stim,
                        const double* scales, double* vm_trace, double* final_states);
long oracle_single_cell_traces(int model, int tissue, double dt, long n_steps,
                               const oracle_ode_settings* ode, const oracle_stimulus* stim,
                               const double* scales, double* vm_trace, int state_b,
                               double* b_trace, double* final_states);

/* --- Purkinje network (ConductionSystemDomain + Monodomain1DSolver) and
 * the reaction-diffusion PVJ coupling ------------------------------------ */
typedef struct oracle_purkinje oracle_purkinje;
oracle_purkinje* oracle_purkinje_new(long n_edges, const int* ea, const int* eb, const double* len,
                                     const double* cond, int model, int tissue,
                                     const oracle_ode_settings* ode, double initial_dt,
                                     double chi, double cm, int root, double root_start,
                                     double root_dur, double root_int, long n_term,
                                     const int* term_node, const double* term_loc);
void oracle_purkinje_free(oracle_purkinje*);
int oracle_purkinje_advance(oracle_purkinje*, double t0, double dt, int nthreads);
int oracle_purkinje_couple(oracle_purkinje*, const oracle_mesh* M, double r_pvj, double radius,
                           int mode);
int oracle_purkinje_coupled_step(oracle_purkinje*, oracle_tissue* T, double dt, int nthreads);
double* oracle_purkinje_vm(oracle_purkinje*);
double* oracle_purkinje_iion(oracle_purkinje*);
double* oracle_purkinje_terminal_current(oracle_purkinje*);
long oracle_purkinje_nodes(oracle_purkinje*);
const int* oracle_purkinje_order(oracle_purkinje*);
const int* oracle_purkinje_parent(oracle_purkinje*);

#ifdef __cplusplus
}
#endif
#endif
