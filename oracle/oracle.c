/* CPU oracle for the monodomain time step - TEST INFRASTRUCTURE ONLY.
 * See oracle.h for what each part restates and its parity status.
 *
 * Build with -ffp-contract=off: the reference is compiled without fused
 * multiply-add contraction on x86-64, and the oracle must round the same way
 * on the aarch64 host, where GCC would otherwise contract a*b+c.
 */
#include "oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "models/tnnp.h"
#include "models/ord.h"
#include "models/torord_dyncl.h"
#include "models/alievpanfilov.h"
#include "models/buenoorovio.h"
#include "models/monodomainfdamanufactured.h"
#include "models/bidomainfdamanufactured.h"

void oracle_fatal(const char* what)
{
    fprintf(stderr, "oracle: fatal: %s\n", what);
    abort();
}

/* ------------------------------------------------------------------------ */
/* model table                                                              */

typedef void (*init_fn)(double*, double*, int, const double*);
typedef void (*supp_fn)(double*);
typedef void (*rhs_fn)(double, const double*, double*, const double*, double*, int, int,
                       const oracle_stimulus*);

typedef struct {
    const char* name;
    int ns, na, nc;
    init_fn init;
    supp_fn supplement; /* constants initConsts leaves unset (ORd) */
    rhs_fn rates;       /* body used by <Model>::derivatives */
    rhs_fn variables;   /* body(ies) called after the ODE solve */
    int iion;
    double iion_scale;
    double time_scale;  /* model time = 1000 t / time_scale */
    int vm_map;         /* 0: mV, 1: Aliev-Panfilov u, 2: Bueno-Orovio u, 3: Vm */
} model_info;

static const model_info MODELS[ORACLE_NMODELS] = {
    {"TNNP", TNNP_NS, TNNP_NA, TNNP_NC, tnnp_init, tnnp_supplement, tnnp_rates, tnnp_variables,
     TNNP_IION_INDEX, TNNP_IION_SCALE, TNNP_TIME_SCALE, 0},
    {"ORd", ORD_NS, ORD_NA, ORD_NC, ord_init, ord_supplement, ord_rates, ord_variables,
     ORD_IION_INDEX, ORD_IION_SCALE, ORD_TIME_SCALE, 0},
    {"ToRORd_dynCl", TORORD_DYNCL_NS, TORORD_DYNCL_NA, TORORD_DYNCL_NC, torord_dyncl_init, torord_dyncl_supplement,
     torord_dyncl_rates, torord_dyncl_variables, TORORD_DYNCL_IION_INDEX,
     TORORD_DYNCL_IION_SCALE, TORORD_DYNCL_TIME_SCALE, 0},
    {"AlievPanfilov", ALIEVPANFILOV_NS, ALIEVPANFILOV_NA, ALIEVPANFILOV_NC,
     alievpanfilov_init, alievpanfilov_supplement, alievpanfilov_rates, alievpanfilov_variables,
     ALIEVPANFILOV_IION_INDEX, ALIEVPANFILOV_IION_SCALE, ALIEVPANFILOV_TIME_SCALE, 1},
    {"BuenoOrovio", BUENOOROVIO_NS, BUENOOROVIO_NA, BUENOOROVIO_NC, buenoorovio_init, buenoorovio_supplement,
     buenoorovio_rates, buenoorovio_variables, BUENOOROVIO_IION_INDEX,
     BUENOOROVIO_IION_SCALE, BUENOOROVIO_TIME_SCALE, 2},
    {"monodomainFDAManufactured", MONODOMAINFDAMANUFACTURED_NS, MONODOMAINFDAMANUFACTURED_NA,
     MONODOMAINFDAMANUFACTURED_NC, monodomainfdamanufactured_init,
     monodomainfdamanufactured_supplement, monodomainfdamanufactured_rates,
     monodomainfdamanufactured_variables, MONODOMAINFDAMANUFACTURED_IION_INDEX,
     MONODOMAINFDAMANUFACTURED_IION_SCALE, MONODOMAINFDAMANUFACTURED_TIME_SCALE, 3},
    {"bidomainFDAManufactured", BIDOMAINFDAMANUFACTURED_NS, BIDOMAINFDAMANUFACTURED_NA,
     BIDOMAINFDAMANUFACTURED_NC, bidomainfdamanufactured_init,
     bidomainfdamanufactured_supplement, bidomainfdamanufactured_rates,
     bidomainfdamanufactured_variables, BIDOMAINFDAMANUFACTURED_IION_INDEX,
     BIDOMAINFDAMANUFACTURED_IION_SCALE, BIDOMAINFDAMANUFACTURED_TIME_SCALE, 3},
};

int oracle_model_sizes(int model, int* ns, int* na, int* nc)
{
    if (model < 0 || model >= ORACLE_NMODELS) return -1;
    *ns = MODELS[model].ns;
    *na = MODELS[model].na;
    *nc = MODELS[model].nc;
    return 0;
}

void oracle_model_init(int model, int tissue, double* C, double* y, const double* scale)
{
    MODELS[model].init(C, y, tissue, scale);
}

void oracle_model_supplement(int model, double* C) { MODELS[model].supplement(C); }

void oracle_model_rates(int model, double t, const double* C, const double* y, double* dydt,
                        double* alg, int tissue, int solve_vm, const oracle_stimulus* stim)
{
    MODELS[model].rates(t, C, dydt, y, alg, tissue, solve_vm, stim);
}

void oracle_model_variables(int model, double t, const double* C, const double* y,
                            double* rates, double* alg, int tissue, int solve_vm,
                            const oracle_stimulus* stim)
{
    MODELS[model].variables(t, C, rates, y, alg, tissue, solve_vm, stim);
}

int oracle_model_iion_index(int model) { return MODELS[model].iion; }

/* ------------------------------------------------------------------------ */
/* OpenFOAM RKF45 (ODESolver + adaptiveSolver + RKF45), restated            */

void oracle_ode_default(oracle_ode_settings* s)
{
    s->abs_tol = 1e-15;   /* SMALL */
    s->rel_tol = 1e-4;
    s->max_steps = 10000;
    s->safe_scale = 0.9;
    s->min_scale = 0.2;
    s->max_scale = 10.0;
    s->alpha_inc = 0.2;
    s->alpha_dec = 0.25;
}

/* Fehlberg 4(5) tableau; the 5th-order solution is propagated and the
 * difference to the embedded 4th-order one is the error estimate. */
static const double c2 = 1.0 / 4.0, c3 = 3.0 / 8.0, c4 = 12.0 / 13.0, c5 = 1.0, c6 = 1.0 / 2.0;
static const double a21 = 1.0 / 4.0;
static const double a31 = 3.0 / 32.0, a32 = 9.0 / 32.0;
static const double a41 = 1932.0 / 2197.0, a42 = -7200.0 / 2197.0, a43 = 7296.0 / 2197.0;
static const double a51 = 439.0 / 216.0, a52 = -8.0, a53 = 3680.0 / 513.0,
                    a54 = -845.0 / 4104.0;
static const double a61 = -8.0 / 27.0, a62 = 2.0, a63 = -3544.0 / 2565.0,
                    a64 = 1859.0 / 4104.0, a65 = -11.0 / 40.0;
static const double b1 = 16.0 / 135.0, b3 = 6656.0 / 12825.0, b4 = 28561.0 / 56430.0,
                    b5 = -9.0 / 50.0, b6 = 2.0 / 55.0;
#define E1 (25.0 / 216.0 - b1)
#define E3 (1408.0 / 2565.0 - b3)
#define E4 (2197.0 / 4104.0 - b4)
#define E5 (-1.0 / 5.0 - b5)
#define E6 (-b6)

struct oracle_ionic {
    const model_info* m;
    int model;
    long n;
    int tissue;
    unsigned char* tissue_cell;   /* per-cell tissue flags, or NULL */
    int solve_vm;
    oracle_ode_settings ode;
    oracle_stimulus stim;
    int has_stim;
    double* C;          /* constants: one row, or one row per cell when scaled */
    int per_cell_consts;
    double* y;          /* STATES, AoS */
    double* alg;        /* ALGEBRAIC, AoS (persistent, as ALGEBRAIC_) */
    double* rates;      /* RATES, AoS */
    double* step;       /* per-cell persistent ODE step (ms), ionicModel::step_ */
    long rhs_evals;
};

typedef struct {
    /* one RKF45 solver object's work arrays (OpenFOAM allocates these once per
     * solver; the k arrays keep entries a model never writes, i.e. RATES[V]
     * in tissue mode, at their initial zero) */
    double *dydx0, *k2, *k3, *k4, *k5, *k6, *ytmp, *yout, *err, *algtmp;
    long evals;
    int tissue;         /* tissue flag of the cell being integrated */
} rk_ws;

static void ws_alloc(rk_ws* w, int ns, int na)
{
    double* p = (double*)calloc((size_t)(9 * ns + na), sizeof(double));
    w->dydx0 = p;
    w->k2 = p + ns;
    w->k3 = p + 2 * ns;
    w->k4 = p + 3 * ns;
    w->k5 = p + 4 * ns;
    w->k6 = p + 5 * ns;
    w->ytmp = p + 6 * ns;
    w->yout = p + 7 * ns;
    w->err = p + 8 * ns;
    w->algtmp = p + 9 * ns;
    w->evals = 0;
    w->tissue = 0;
}

static void ws_free(rk_ws* w) { free(w->dydx0); }

/* <Model>::derivatives: fresh zeroed ALGEBRAIC scratch, RATES = dydt */
static void derivs(const oracle_ionic* io, const double* C, rk_ws* w, double t, const double* y,
                   double* dydt)
{
    memset(w->algtmp, 0, sizeof(double) * (size_t)io->m->na);
    io->m->rates(t, C, dydt, y, w->algtmp, w->tissue, io->solve_vm,
                 io->has_stim ? &io->stim : NULL);
    w->evals++;
}

/* RKF45::solve(x0, y0, dydx0, dx, y): one trial step, returns the error norm */
static double rkf45_trial(const oracle_ionic* io, const double* C, rk_ws* w, double x0,
                          const double* y0, double dx, double* y)
{
    const int ns = io->m->ns;
    int i;
    for (i = 0; i < ns; i++) w->ytmp[i] = y0[i] + a21 * dx * w->dydx0[i];
    derivs(io, C, w, x0 + c2 * dx, w->ytmp, w->k2);
    for (i = 0; i < ns; i++) w->ytmp[i] = y0[i] + dx * (a31 * w->dydx0[i] + a32 * w->k2[i]);
    derivs(io, C, w, x0 + c3 * dx, w->ytmp, w->k3);
    for (i = 0; i < ns; i++)
        w->ytmp[i] = y0[i] + dx * (a41 * w->dydx0[i] + a42 * w->k2[i] + a43 * w->k3[i]);
    derivs(io, C, w, x0 + c4 * dx, w->ytmp, w->k4);
    for (i = 0; i < ns; i++)
        w->ytmp[i] = y0[i] + dx * (a51 * w->dydx0[i] + a52 * w->k2[i] + a53 * w->k3[i]
                                   + a54 * w->k4[i]);
    derivs(io, C, w, x0 + c5 * dx, w->ytmp, w->k5);
    for (i = 0; i < ns; i++)
        w->ytmp[i] = y0[i] + dx * (a61 * w->dydx0[i] + a62 * w->k2[i] + a63 * w->k3[i]
                                   + a64 * w->k4[i] + a65 * w->k5[i]);
    derivs(io, C, w, x0 + c6 * dx, w->ytmp, w->k6);
    for (i = 0; i < ns; i++)
        y[i] = y0[i] + dx * (b1 * w->dydx0[i] + b3 * w->k3[i] + b4 * w->k4[i] + b5 * w->k5[i]
                             + b6 * w->k6[i]);
    for (i = 0; i < ns; i++)
        w->err[i] = dx * (E1 * w->dydx0[i] + E3 * w->k3[i] + E4 * w->k4[i] + E5 * w->k5[i]
                          + E6 * w->k6[i]);
    /* ODESolver::normalizeError */
    double maxerr = 0.0;
    for (i = 0; i < ns; i++) {
        double a = fabs(y0[i]), b = fabs(y[i]);
        double tol = io->ode.abs_tol + io->ode.rel_tol * (a > b ? a : b);
        double e = fabs(w->err[i]) / tol;
        if (e > maxerr) maxerr = e;
    }
    return maxerr;
}

/* adaptiveSolver::solve(odes, x, y, dxTry) */
static int adaptive_step(const oracle_ionic* io, const double* C, rk_ws* w, double* x, double* y,
                         double* dx_try)
{
    const oracle_ode_settings* s = &io->ode;
    double dx = *dx_try, err = 0.0;
    derivs(io, C, w, *x, y, w->dydx0);
    do {
        err = rkf45_trial(io, C, w, *x, y, dx, w->yout);
        if (err > 1) {
            double scale = s->safe_scale * pow(err, -s->alpha_dec);
            if (scale < s->min_scale) scale = s->min_scale;
            dx *= scale;
            if (dx < 1e-300) return -1;   /* stepsize underflow */
        }
    } while (err > 1);
    *x += dx;
    memcpy(y, w->yout, sizeof(double) * (size_t)io->m->ns);
    if (err > pow(s->max_scale / s->safe_scale, -1.0 / s->alpha_inc)) {
        double scale = s->safe_scale * pow(err, -s->alpha_inc);
        if (scale > s->max_scale) scale = s->max_scale;
        *dx_try = scale * dx;
    } else {
        *dx_try = s->safe_scale * s->max_scale * dx;
    }
    return 0;
}

/* ODESolver::solve(xStart, xEnd, y, dxTry): returns accepted steps or -1 */
static long ode_solve(const oracle_ionic* io, const double* C, rk_ws* w, double xs, double xe,
                      double* y, double* dx_try)
{
    double step_dx = *dx_try;
    int last = 0;
    double x = xs;
    long n;
    for (n = 0; n < io->ode.max_steps; n++) {
        double dx_try0 = step_dx;
        if ((x + step_dx - xe) * (x + step_dx - xs) > 0) {
            last = 1;
            step_dx = xe - x;
        }
        if (adaptive_step(io, C, w, &x, y, &step_dx) != 0) return -1;
        if ((x - xe) * (xe - xs) >= 0) {
            if (n > 0 && last) step_dx = dx_try0;
            *dx_try = step_dx;
            return n + 1;
        }
    }
    return -1;
}

oracle_ionic* oracle_ionic_new(int model, long n, int tissue, double initial_dt, int solve_vm,
                               const oracle_ode_settings* ode, const oracle_stimulus* stim,
                               const double* scales)
{
    return oracle_ionic_new_cells(model, n, tissue, NULL, initial_dt, solve_vm, ode, stim, scales);
}

/* The same with a tissue flag per cell (tissue_cell, or NULL for `tissue`
 * everywhere); per-cell flags give each cell its own constants. */
oracle_ionic* oracle_ionic_new_cells(int model, long n, int tissue,
                                     const unsigned char* tissue_cell, double initial_dt,
                                     int solve_vm, const oracle_ode_settings* ode,
                                     const oracle_stimulus* stim, const double* scales)
{
    if (model < 0 || model >= ORACLE_NMODELS || n < 0) return NULL;
    oracle_ionic* io = (oracle_ionic*)calloc(1, sizeof(oracle_ionic));
    const model_info* m = &MODELS[model];
    io->m = m;
    io->model = model;
    io->n = n;
    io->tissue = tissue;
    io->solve_vm = solve_vm;
    if (ode) io->ode = *ode; else oracle_ode_default(&io->ode);
    if (stim) { io->stim = *stim; io->has_stim = 1; }
    io->per_cell_consts = scales != NULL || tissue_cell != NULL;
    if (tissue_cell) {
        io->tissue_cell = (unsigned char*)malloc((size_t)(n > 0 ? n : 1));
        memcpy(io->tissue_cell, tissue_cell, (size_t)n);
    }
    io->C = (double*)calloc((size_t)m->nc * (size_t)(io->per_cell_consts ? (n > 0 ? n : 1) : 1),
                            sizeof(double));
    io->y = (double*)calloc((size_t)(n * m->ns + 1), sizeof(double));
    io->alg = (double*)calloc((size_t)(n * m->na + 1), sizeof(double));
    io->rates = (double*)calloc((size_t)(n * m->ns + 1), sizeof(double));
    io->step = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    for (long c = 0; c < n; c++) {
        /* the reference re-runs initConsts into the shared CONSTANTS for
         * every cell (TNNP.C:64-76); per-cell scales need a row per cell */
        double* Crow = io->C + (io->per_cell_consts ? (size_t)c * (size_t)m->nc : 0);
        const int tc = tissue_cell ? (int)tissue_cell[c] : tissue;
        m->init(Crow, io->y + (size_t)c * (size_t)m->ns, tc, scales ? scales + 6 * c : NULL);
        m->supplement(Crow);
        io->step[c] = initial_dt;
    }
    if (n == 0) { m->init(io->C, io->y, tissue, NULL); m->supplement(io->C); }
    return io;
}

void oracle_ionic_free(oracle_ionic* io)
{
    if (!io) return;
    free(io->C);
    free(io->y);
    free(io->alg);
    free(io->rates);
    free(io->step);
    free(io->tissue_cell);
    free(io);
}

double* oracle_ionic_states(oracle_ionic* io) { return io->y; }
double* oracle_ionic_steps(oracle_ionic* io) { return io->step; }
long oracle_ionic_rhs_evals(oracle_ionic* io) { return io->rhs_evals; }

static double vm_to_state0(int map, double vm)
{
    if (map == 1) return (vm * 1000.0 + 80) / 100;       /* AlievPanfilov.C:121 */
    if (map == 2) return (vm * 1000.0 + 84) / 85.7;      /* BuenoOrovio.C:120 */
    if (map == 3) return vm;                             /* monodomainFDAManufactured.C:108 */
    return vm * 1000.0;                                  /* TNNP.C:137 */
}

/* <Model>::solveODE for cells [c0, c1) with one solver work set */
static long solve_range(oracle_ionic* io, rk_ws* w, long c0, long c1, double t0, double dt,
                        const double* vm, double* im)
{
    const model_info* m = io->m;
    const double ts = m->time_scale;
    /* tStart/tEnd in model time: TNNP.C:122-123, AlievPanfilov.C:107-108 */
    /* model time in seconds: monodomainFDAManufactured.C:96-97, 109 */
    const double t_start = (ts == 1000.0) ? t0 : (ts == 1.0) ? t0 * 1000 : t0 * 1000.0 / ts;
    const double t_end = (ts == 1000.0) ? t0 + dt
                       : (ts == 1.0) ? (t0 + dt) * 1000 : (t0 + dt) * 1000.0 / ts;
    const double dt_model = (ts == 1000.0) ? dt : (ts == 1.0) ? dt * 1000.0 : dt * 1000.0 / ts;
    long total = 0;
    for (long c = c0; c < c1; c++) {
        double* y = io->y + (size_t)c * (size_t)m->ns;
        double* alg = io->alg + (size_t)c * (size_t)m->na;
        double* rates = io->rates + (size_t)c * (size_t)m->ns;
        const double* C = io->C + (io->per_cell_consts ? (size_t)c * (size_t)m->nc : 0);
        w->tissue = io->tissue_cell ? (int)io->tissue_cell[c] : io->tissue;
        if (!io->solve_vm) y[0] = vm_to_state0(m->vm_map, vm[c]);
        double* step = &io->step[c];
        if (dt_model < *step) *step = dt_model;
        long k = ode_solve(io, C, w, t_start, t_end, y, step);
        if (k < 0) return -1;
        total += k;
        m->variables(t_end, C, rates, y, alg, w->tissue, io->solve_vm,
                     io->has_stim ? &io->stim : NULL);
        if (im) im[c] = alg[m->iion] * m->iion_scale;
    }
    return total;
}

long oracle_ionic_solve(oracle_ionic* io, double t0, double dt, const double* vm, double* im,
                        int nthreads)
{
    long total = 0;
    int failed = 0;
    long evals = 0;
#ifdef _OPENMP
    if (nthreads > 1) {
#pragma omp parallel num_threads(nthreads) reduction(+ : total, evals) reduction(| : failed)
        {
            rk_ws w;
            ws_alloc(&w, io->m->ns, io->m->na);
            int tid = omp_get_thread_num(), nt = omp_get_num_threads();
            long chunk = (io->n + nt - 1) / nt;
            long c0 = tid * chunk, c1 = c0 + chunk < io->n ? c0 + chunk : io->n;
            if (c0 < c1) {
                long k = solve_range(io, &w, c0, c1, t0, dt, vm, im);
                if (k < 0) failed = 1; else total += k;
            }
            evals += w.evals;
            ws_free(&w);
        }
        io->rhs_evals += evals;
        return failed ? -1 : total;
    }
#else
    (void)nthreads;
#endif
    rk_ws w;
    ws_alloc(&w, io->m->ns, io->m->na);
    total = solve_range(io, &w, 0, io->n, t0, dt, vm, im);
    io->rhs_evals += w.evals;
    ws_free(&w);
    (void)failed;
    return total;
}

/* ------------------------------------------------------------------------ */
/* structured hex mesh as blockMesh builds one block: cells x-fastest;       */
/* internal faces in upper-triangular order (per owner: +x, +y, +z)         */

struct oracle_mesh {
    int nx, ny, nz;
    long n, nf;
    double dx, dy, dz;
    int* owner;
    int* neigh;
    double* centres;  /* 3n */
    double* vol;      /* n */
    double* sf;       /* 3nf face area vectors, owner -> neighbour */
    double* delta;    /* nf: |d_PN| */
    /* full geometry of a general mesh (NULL/0 for the structured box) */
    double* cf;       /* 3nf face centres */
    long nb;          /* boundary faces (all zeroGradient for Vm) */
    int* bcell;       /* nb owner cells */
    double* bsf;      /* 3nb outward area vectors */
    double* bcf;      /* 3nb face centres */
};

oracle_mesh* oracle_mesh_box(int nx, int ny, int nz, double lx, double ly, double lz)
{
    oracle_mesh* m = (oracle_mesh*)calloc(1, sizeof(oracle_mesh));
    m->nx = nx; m->ny = ny; m->nz = nz;
    m->n = (long)nx * ny * nz;
    m->dx = lx / nx; m->dy = ly / ny; m->dz = lz / nz;
    long nf = (long)(nx - 1) * ny * nz + (long)nx * (ny - 1) * nz + (long)nx * ny * (nz - 1);
    m->nf = nf;
    m->owner = (int*)malloc(sizeof(int) * (size_t)(nf + 1));
    m->neigh = (int*)malloc(sizeof(int) * (size_t)(nf + 1));
    m->sf = (double*)malloc(sizeof(double) * 3 * (size_t)(nf + 1));
    m->delta = (double*)malloc(sizeof(double) * (size_t)(nf + 1));
    m->centres = (double*)malloc(sizeof(double) * 3 * (size_t)m->n);
    m->vol = (double*)malloc(sizeof(double) * (size_t)m->n);
    /* points of a uniform block: x_i = i*lx/nx */
    long f = 0;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                long c = ((long)k * ny + j) * nx + i;
                double x0 = lx * i / nx, x1 = lx * (i + 1) / nx;
                double y0 = ly * j / ny, y1 = ly * (j + 1) / ny;
                double z0 = lz * k / nz, z1 = lz * (k + 1) / nz;
                m->centres[3 * c + 0] = 0.5 * (x0 + x1);
                m->centres[3 * c + 1] = 0.5 * (y0 + y1);
                m->centres[3 * c + 2] = 0.5 * (z0 + z1);
                m->vol[c] = (x1 - x0) * (y1 - y0) * (z1 - z0);
            }
    for (long c = 0; c < m->n; c++) {
        int i = (int)(c % nx), j = (int)((c / nx) % ny), k = (int)(c / ((long)nx * ny));
        long nb[3] = {i + 1 < nx ? c + 1 : -1, j + 1 < ny ? c + nx : -1,
                      k + 1 < nz ? c + (long)nx * ny : -1};
        for (int d = 0; d < 3; d++) {
            if (nb[d] < 0) continue;
            m->owner[f] = (int)c;
            m->neigh[f] = (int)nb[d];
            double area = d == 0 ? (ly / ny) * (lz / nz) : d == 1 ? (lx / nx) * (lz / nz)
                                                                 : (lx / nx) * (ly / ny);
            m->sf[3 * f + 0] = d == 0 ? area : 0.0;
            m->sf[3 * f + 1] = d == 1 ? area : 0.0;
            m->sf[3 * f + 2] = d == 2 ? area : 0.0;
            double dd = m->centres[3 * nb[d] + d] - m->centres[3 * c + d];
            m->delta[f] = dd;
            f++;
        }
    }
    return m;
}

static void* dup_array(const void* src, size_t bytes)
{
    void* p = malloc(bytes ? bytes : 1);
    if (bytes) memcpy(p, src, bytes);
    return p;
}

/* A general (unstructured) mesh from its lduAddressing and geometry as
 * fvMesh holds them: cell centres and volumes, internal faces (owner <
 * neighbour, upper-triangular order) with area vectors owner -> neighbour
 * and centres, and the boundary faces with their cells, outward area
 * vectors and centres. */
oracle_mesh* oracle_mesh_general(long n, long nf, const int* owner, const int* neigh,
                                 const double* centres, const double* vol,
                                 const double* face_centres, const double* face_sf, long nb,
                                 const int* bcell, const double* bsf, const double* bcf)
{
    oracle_mesh* m = (oracle_mesh*)calloc(1, sizeof(oracle_mesh));
    m->n = n;
    m->nf = nf;
    m->nb = nb;
    m->owner = (int*)dup_array(owner, sizeof(int) * (size_t)nf);
    m->neigh = (int*)dup_array(neigh, sizeof(int) * (size_t)nf);
    m->centres = (double*)dup_array(centres, sizeof(double) * 3 * (size_t)n);
    m->vol = (double*)dup_array(vol, sizeof(double) * (size_t)n);
    m->cf = (double*)dup_array(face_centres, sizeof(double) * 3 * (size_t)nf);
    m->sf = (double*)dup_array(face_sf, sizeof(double) * 3 * (size_t)nf);
    m->bcell = (int*)dup_array(bcell, sizeof(int) * (size_t)nb);
    m->bsf = (double*)dup_array(bsf, sizeof(double) * 3 * (size_t)nb);
    m->bcf = (double*)dup_array(bcf, sizeof(double) * 3 * (size_t)nb);
    m->delta = (double*)malloc(sizeof(double) * (size_t)(nf + 1));
    for (long f = 0; f < nf; f++) {
        const double* P = m->centres + 3 * (size_t)owner[f];
        const double* N = m->centres + 3 * (size_t)neigh[f];
        double d0 = N[0] - P[0], d1 = N[1] - P[1], d2 = N[2] - P[2];
        m->delta[f] = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    }
    return m;
}

void oracle_mesh_free(oracle_mesh* m)
{
    if (!m) return;
    free(m->owner); free(m->neigh); free(m->sf); free(m->delta);
    free(m->centres); free(m->vol);
    free(m->cf); free(m->bcell); free(m->bsf); free(m->bcf);
    free(m);
}

long oracle_mesh_ncells(const oracle_mesh* m) { return m->n; }
long oracle_mesh_nfaces(const oracle_mesh* m) { return m->nf; }

void oracle_mesh_addressing(const oracle_mesh* m, int* owner, int* neighbour)
{
    memcpy(owner, m->owner, sizeof(int) * (size_t)m->nf);
    memcpy(neighbour, m->neigh, sizeof(int) * (size_t)m->nf);
}

void oracle_mesh_centres(const oracle_mesh* m, double* c)
{
    memcpy(c, m->centres, sizeof(double) * 3 * (size_t)m->n);
}

/* ------------------------------------------------------------------------ */
/* Cell centres of one uniformly graded blockMesh block with every rounding  */
/* of OpenFOAM's own geometry (v2312 published algorithms, restated):        */
/*  - blockMesh's block point interpolation (block::createPoints): each      */
/*    point is a third of the sum over the 12 straight edges of edge point x  */
/*    edge weight, the 4 weights per direction normalised by their sum;      */
/*    lineDivide's uniform lambdas i/n; the scale applied at the end;        */
/*  - primitiveMeshTools::makeFaceCentresAndAreas: the triangle fan about    */
/*    the face's point average;                                             */
/*  - primitiveMeshTools::makeCellCentresAndVols: face-pyramid centroids     */
/*    weighted by 3 x pyramid volume, about the average of the face centres; */
/*  - polyMesh from cell shapes: internal faces upper-triangular (per owner  */
/*    +x, +y, +z, as the owner's hex faces (1 2 6 5), (3 7 6 2), (4 5 6 7)),  */
/*    then the boundary faces in the patch's block-face order.              */
/* The sums over a cell's faces run in face order: its owned faces, then the */
/* faces it neighbours.  A cell centre that lies exactly on a plane of the   */
/* grid comes out a few units in the last place either side of it, and an    */
/* inclusive box test (stimulus boxes) on such a plane takes part of the     */
/* layer.  `contract` selects which expressions a compiler fuses into fma    */
/* (clang's -ffp-contract=on on an FMA target): bit 1 the blockMesh weights, */
/* bit 2 cross products, bit 4 dot products, bit 8 squared magnitudes.       */
/* extent = the block's far vertex before scaling (the near one is 0);       */
/* patch_order = the 6 block faces (0 x-min, 1 x-max, 2 y-min, 3 y-max,      */
/* 4 z-min, 5 z-max) in the order the boundary patch lists them.  Centres    */
/* out: 3 per cell, x fastest. Test infrastructure.                          */

typedef struct { double x, y, z; } bm_v;

static bm_v bm_add(bm_v a, bm_v b) { bm_v r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static bm_v bm_sub(bm_v a, bm_v b) { bm_v r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static bm_v bm_scale(double s, bm_v a) { bm_v r = {s * a.x, s * a.y, s * a.z}; return r; }
static bm_v bm_div(bm_v a, double s) { bm_v r = {a.x / s, a.y / s, a.z / s}; return r; }

/* a*b - c*d as one expression */
static double bm_msub(double a, double b, double c, double d, int fuse)
{
    return fuse ? fma(a, b, -(c * d)) : a * b - c * d;
}

static double bm_dot(bm_v a, bm_v b, int fuse)
{
    return fuse ? fma(a.z, b.z, fma(a.x, b.x, a.y * b.y)) : a.x * b.x + a.y * b.y + a.z * b.z;
}

static bm_v bm_cross(bm_v a, bm_v b, int fuse)
{
    bm_v r = {bm_msub(a.y, b.z, a.z, b.y, fuse), bm_msub(a.z, b.x, a.x, b.z, fuse),
              bm_msub(a.x, b.y, a.y, b.x, fuse)};
    return r;
}

/* edge weight (1-a)(1-b)(1-c) + a(1-d)(1-e) style: p*q*r + s*t*u */
static double bm_w(double p, double q, double r, double s, double t, double u, int fuse)
{
    return fuse ? fma(p * q, r, s * t * u) : p * q * r + s * t * u;
}

static void bm_face(const bm_v* q, int contract, bm_v* centre, bm_v* area)
{
    bm_v avg = q[0];
    for (int t = 1; t < 4; t++) avg = bm_add(avg, q[t]);
    avg = bm_div(avg, 4.0);
    bm_v sum_n = {0, 0, 0}, sum_ac = {0, 0, 0};
    double sum_a = 0.0;
    for (int t = 0; t < 4; t++) {
        const bm_v a = q[t], b = q[(t + 1) % 4];
        const bm_v c = bm_add(bm_add(a, b), avg);
        const bm_v n = bm_cross(bm_sub(b, a), bm_sub(avg, a), contract & 2);
        const double mag = sqrt(bm_dot(n, n, contract & 8));
        sum_n = bm_add(sum_n, n);
        sum_a += mag;
        sum_ac = bm_add(sum_ac, bm_scale(mag, c));
    }
    *centre = bm_div(bm_scale(1.0 / 3.0, sum_ac), sum_a);
    *area = bm_scale(0.5, sum_n);
}

int oracle_blockmesh_centres(int ni, int nj, int nk, const double* extent, double scale,
                             const int* patch_order, int contract, double* centres)
{
    if (ni < 1 || nj < 1 || nk < 1) return -1;
    for (int r = 0; r < 6; r++)
        if (patch_order[r] < 0 || patch_order[r] > 5) return -1;
    const long pi_ = ni + 1, pj_ = nj + 1;
    const long np = pi_ * pj_ * (nk + 1);
    bm_v* pts = (bm_v*)malloc(sizeof(bm_v) * (size_t)np);
    if (!pts) return -1;
    const double X = extent[0], Y = extent[1], Z = extent[2];
    /* block vertices in hex order; edges x1..x4, y1..y4, z1..z4 */
    const bm_v v000 = {0, 0, 0}, v100 = {X, 0, 0}, v110 = {X, Y, 0}, v010 = {0, Y, 0};
    const bm_v v001 = {0, 0, Z}, v101 = {X, 0, Z}, v111 = {X, Y, Z}, v011 = {0, Y, Z};
    const int fw = contract & 1;
    for (int k = 0; k <= nk; k++)
        for (int j = 0; j <= nj; j++)
            for (int i = 0; i <= ni; i++) {
                bm_v p;
                if ((i == 0 || i == ni) && (j == 0 || j == nj) && (k == 0 || k == nk)) {
                    p.x = i ? X : 0.0; p.y = j ? Y : 0.0; p.z = k ? Z : 0.0;
                } else {
                    const double a = 0.0 + 1.0 * (double)i / ni;
                    const double b = 0.0 + 1.0 * (double)j / nj;
                    const double c = 0.0 + 1.0 * (double)k / nk;
                    double wx[4] = {bm_w(1 - a, 1 - b, 1 - c, a, 1 - b, 1 - c, fw),
                                    bm_w(1 - a, b, 1 - c, a, b, 1 - c, fw),
                                    bm_w(1 - a, b, c, a, b, c, fw),
                                    bm_w(1 - a, 1 - b, c, a, 1 - b, c, fw)};
                    double wy[4] = {bm_w(1 - b, 1 - a, 1 - c, b, 1 - a, 1 - c, fw),
                                    bm_w(1 - b, a, 1 - c, b, a, 1 - c, fw),
                                    bm_w(1 - b, a, c, b, a, c, fw),
                                    bm_w(1 - b, 1 - a, c, b, 1 - a, c, fw)};
                    double wz[4] = {bm_w(1 - c, 1 - a, 1 - b, c, 1 - a, 1 - b, fw),
                                    bm_w(1 - c, a, 1 - b, c, a, 1 - b, fw),
                                    bm_w(1 - c, a, b, c, a, b, fw),
                                    bm_w(1 - c, 1 - a, b, c, 1 - a, b, fw)};
                    double* ws[3] = {wx, wy, wz};
                    for (int d = 0; d < 3; d++) {
                        const double s = ws[d][0] + ws[d][1] + ws[d][2] + ws[d][3];
                        for (int e = 0; e < 4; e++) ws[d][e] /= s;
                    }
                    const bm_v e[12] = {
                        bm_add(v000, bm_scale(a, bm_sub(v100, v000))),
                        bm_add(v010, bm_scale(a, bm_sub(v110, v010))),
                        bm_add(v011, bm_scale(a, bm_sub(v111, v011))),
                        bm_add(v001, bm_scale(a, bm_sub(v101, v001))),
                        bm_add(v000, bm_scale(b, bm_sub(v010, v000))),
                        bm_add(v100, bm_scale(b, bm_sub(v110, v100))),
                        bm_add(v101, bm_scale(b, bm_sub(v111, v101))),
                        bm_add(v001, bm_scale(b, bm_sub(v011, v001))),
                        bm_add(v000, bm_scale(c, bm_sub(v001, v000))),
                        bm_add(v100, bm_scale(c, bm_sub(v101, v100))),
                        bm_add(v110, bm_scale(c, bm_sub(v111, v110))),
                        bm_add(v010, bm_scale(c, bm_sub(v011, v010)))};
                    bm_v s = bm_scale(wx[0], e[0]);
                    for (int m = 1; m < 12; m++) s = bm_add(s, bm_scale(ws[m / 4][m % 4], e[m]));
                    p = bm_div(s, 3.0);
                }
                pts[i + pi_ * (j + pj_ * (long)k)] = bm_scale(scale, p);
            }
#define BM_P(i, j, k) pts[(i) + pi_ * ((j) + pj_ * (long)(k))]
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                /* the cell's 6 faces in face order, with the side they are
                 * owned from: owned internal (+x +y +z), boundary (patch
                 * order), then neighboured internal (-z -y -x) */
                bm_v q[6][4];
                int owned[6], nfc = 0;
#define BM_FACE(own_, a0, a1, a2, a3)                                      \
    do {                                                                   \
        q[nfc][0] = a0; q[nfc][1] = a1; q[nfc][2] = a2; q[nfc][3] = a3;    \
        owned[nfc++] = own_;                                               \
    } while (0)
                if (i + 1 < ni)
                    BM_FACE(1, BM_P(i + 1, j, k), BM_P(i + 1, j + 1, k), BM_P(i + 1, j + 1, k + 1),
                            BM_P(i + 1, j, k + 1));
                if (j + 1 < nj)
                    BM_FACE(1, BM_P(i, j + 1, k), BM_P(i, j + 1, k + 1), BM_P(i + 1, j + 1, k + 1),
                            BM_P(i + 1, j + 1, k));
                if (k + 1 < nk)
                    BM_FACE(1, BM_P(i, j, k + 1), BM_P(i + 1, j, k + 1), BM_P(i + 1, j + 1, k + 1),
                            BM_P(i, j + 1, k + 1));
                for (int r = 0; r < 6; r++) {
                    const int bf = patch_order[r];
                    if (bf == 0 && i == 0)
                        BM_FACE(1, BM_P(0, j, k), BM_P(0, j, k + 1), BM_P(0, j + 1, k + 1),
                                BM_P(0, j + 1, k));
                    if (bf == 1 && i == ni - 1)
                        BM_FACE(1, BM_P(ni, j, k), BM_P(ni, j + 1, k), BM_P(ni, j + 1, k + 1),
                                BM_P(ni, j, k + 1));
                    if (bf == 2 && j == 0)
                        BM_FACE(1, BM_P(i, 0, k), BM_P(i + 1, 0, k), BM_P(i + 1, 0, k + 1),
                                BM_P(i, 0, k + 1));
                    if (bf == 3 && j == nj - 1)
                        BM_FACE(1, BM_P(i, nj, k), BM_P(i, nj, k + 1), BM_P(i + 1, nj, k + 1),
                                BM_P(i + 1, nj, k));
                    if (bf == 4 && k == 0)
                        BM_FACE(1, BM_P(i, j, 0), BM_P(i, j + 1, 0), BM_P(i + 1, j + 1, 0),
                                BM_P(i + 1, j, 0));
                    if (bf == 5 && k == nk - 1)
                        BM_FACE(1, BM_P(i, j, nk), BM_P(i + 1, j, nk), BM_P(i + 1, j + 1, nk),
                                BM_P(i, j + 1, nk));
                }
                /* internal faces the cell neighbours, as their owners hold them */
                if (k > 0)
                    BM_FACE(0, BM_P(i, j, k), BM_P(i + 1, j, k), BM_P(i + 1, j + 1, k),
                            BM_P(i, j + 1, k));
                if (j > 0)
                    BM_FACE(0, BM_P(i, j, k), BM_P(i, j, k + 1), BM_P(i + 1, j, k + 1),
                            BM_P(i + 1, j, k));
                if (i > 0)
                    BM_FACE(0, BM_P(i, j, k), BM_P(i, j + 1, k), BM_P(i, j + 1, k + 1),
                            BM_P(i, j, k + 1));
#undef BM_FACE
                bm_v fc[6], fa[6];
                bm_v est = {0, 0, 0};
                for (int f = 0; f < nfc; f++) {
                    bm_face(q[f], contract, &fc[f], &fa[f]);
                    est = bm_add(est, fc[f]);
                }
                est = bm_div(est, (double)nfc);
                bm_v sum_c = {0, 0, 0};
                double sum_v = 0.0;
                for (int f = 0; f < nfc; f++) {
                    const double pv = owned[f] ? bm_dot(fa[f], bm_sub(fc[f], est), contract & 4)
                                               : bm_dot(fa[f], bm_sub(est, fc[f]), contract & 4);
                    const bm_v pc = bm_add(bm_scale(3.0 / 4.0, fc[f]), bm_scale(1.0 / 4.0, est));
                    sum_c = bm_add(sum_c, bm_scale(pv, pc));
                    sum_v += pv;
                }
                const bm_v cc = bm_div(sum_c, sum_v);
                double* out = centres + 3 * ((size_t)i + (size_t)ni * ((size_t)j + (size_t)nj * k));
                out[0] = cc.x; out[1] = cc.y; out[2] = cc.z;
            }
#undef BM_P
    free(pts);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* monodomain tissue                                                        */

#define MAX_SOLVES 64

struct oracle_tissue {
    oracle_tissue_desc d;
    const oracle_mesh* mesh;
    oracle_ionic* ionic;
    long n, nf;
    double t;           /* runTime value */
    long time_index;
    double* vm;
    double* vm_old;
    double* vm_oldold;
    int n_old;          /* stored old-time levels of Vm (GeometricField::nOldTimes) */
    double* iion;
    double* src;
    double* act;
    unsigned char* calc_act;
    double* lap;        /* upper coefficient per face: deltaCoeff * (Sf.sigma.Sf)/|Sf| */
    double* sigma_cell; /* [n][6] conductivity per cell, or NULL (uniform) */
    unsigned char* tissue_cell;   /* [n] tissue flag per cell, or NULL */
    /* general mesh: gaussLaplacianScheme with corrected snGrad */
    int corrected_mesh; /* face centres given: explicit corrections are on */
    const double* extra_src;  /* bidomain: V fvc::div(Gi & grad(phiE)) added to the source */
    /* PVJ coupling (reactionDiffusionPvjCoupler): per step, source densities
     * deposited after the box stimulus, pair k adding dep_value[dep_term[k]]
     * to cell dep_cell[k], in pair order */
    long n_dep;
    const long* dep_cell;
    const long* dep_term;
    const double* dep_value;
    double *w, *dcoef, *corrv, *sfgsn, *sfgcorr, *bsfgcorr, *bn, *lsp, *lsn, *grad, *fflux;
    /* PCG work */
    double *diag, *upper, *b, *rA, *wA, *pA, *rD, *tmp;
    int n_solves;
    double init_res[MAX_SOLVES], final_res[MAX_SOLVES];
    int iters[MAX_SOLVES];
};

/* Conductivity of cell c as a full tensor, row-major (the symmTensor &
 * tensor(I) of monodomainSolver.C:86-95 for the uniform case). */
static void cell_sigma(const oracle_tissue* T, long c, double s[9])
{
    const double* v = T->sigma_cell ? T->sigma_cell + 6 * (size_t)c : T->d.sigma;
    s[0] = v[0]; s[1] = v[1]; s[2] = v[2];
    s[3] = v[1]; s[4] = v[3]; s[5] = v[4];
    s[6] = v[2]; s[7] = v[4]; s[8] = v[5];
}

/* vector & tensor: out_j = sum_i S_i G_ij */
static void vec_dot_tensor(const double* S, const double* G, double* out)
{
    out[0] = S[0] * G[0] + S[1] * G[3] + S[2] * G[6];
    out[1] = S[0] * G[1] + S[1] * G[4] + S[2] * G[7];
    out[2] = S[0] * G[2] + S[1] * G[5] + S[2] * G[8];
}

static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* SfGamma, SfGammaSn and SfGammaCorr of one face (gaussLaplacianScheme::
 * fvmLaplacian for a tensor Gamma, OpenFOAM v2312). */
static double face_gamma(const double* S, const double* G, double* corr)
{
    const double magSf = sqrt(dot3(S, S));
    const double Sn[3] = {S[0] / magSf, S[1] / magSf, S[2] / magSf};
    double SfG[3];
    vec_dot_tensor(S, G, SfG);
    const double sfgsn = dot3(SfG, Sn);
    for (int k = 0; k < 3; k++) corr[k] = SfG[k] - sfgsn * Sn[k];
    return sfgsn;
}

/* The uncorrected coefficients (orthogonal structured box, uniform sigma)
 * or, for a general mesh, every geometric quantity of OpenFOAM's
 * Gauss-linear-corrected Laplacian and of the cell gradient its explicit
 * part needs:
 *   weights      w = |Sf.(N - Cf)| / (|Sf.(Cf - P)| + |Sf.(N - Cf)|)
 *                (surfaceInterpolation::makeWeights)
 *   deltaCoeffs  1/max(Sn.d, 0.05|d|)  (makeNonOrthDeltaCoeffs)
 *   corrVecs     Sn - d*deltaCoeff     (makeNonOrthCorrectionVectors;
 *                zero on boundary faces)
 *   Gamma_f      w (Gamma_P - Gamma_N) + Gamma_N  (linear interpolation)
 *   leastSquares vectors (leastSquaresVectors::calcLeastSquaresVectors):
 *                dd = sum over faces of d d/|d|^2 with boundary d the
 *                patch-normal delta n (n.(Cf - C)); P: invDd_P.d/|d|^2,
 *                N: -invDd_N.d/|d|^2. */
static void assemble_laplacian(oracle_tissue* T)
{
    const oracle_mesh* M = T->mesh;
    const long nf = T->nf;
    if (!T->corrected_mesh) {
        /* uniform conductivity tensor (monodomainSolver.C:86-95); on a face,
         * SfGammaSn = Sf.(sigma.Sf)/|Sf| and the implicit coefficient is
         * deltaCoeffs * SfGammaSn (gaussLaplacianScheme, orthogonal mesh) */
        const double* s = T->d.sigma;
        for (long f = 0; f < nf; f++) {
            const double* S = M->sf + 3 * f;
            double magSf = sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
            double g0 = S[0] * s[0] + S[1] * s[1] + S[2] * s[2];
            double g1 = S[0] * s[1] + S[1] * s[3] + S[2] * s[4];
            double g2 = S[0] * s[2] + S[1] * s[4] + S[2] * s[5];
            double sfgsn = (g0 * S[0] + g1 * S[1] + g2 * S[2]) / magSf;
            double delta_coeff = 1.0 / M->delta[f];
            T->lap[f] = delta_coeff * sfgsn;
        }
        return;
    }
    double* dd = (double*)calloc(6 * (size_t)T->n, sizeof(double));
    for (long f = 0; f < nf; f++) {
        const long P = M->owner[f], N = M->neigh[f];
        const double* S = M->sf + 3 * f;
        const double* Cf = M->cf + 3 * f;
        const double* CP = M->centres + 3 * P;
        const double* CN = M->centres + 3 * N;
        const double magSf = sqrt(dot3(S, S));
        const double Sn[3] = {S[0] / magSf, S[1] / magSf, S[2] / magSf};
        const double fo[3] = {Cf[0] - CP[0], Cf[1] - CP[1], Cf[2] - CP[2]};
        const double nf3[3] = {CN[0] - Cf[0], CN[1] - Cf[1], CN[2] - Cf[2]};
        const double SfdOwn = fabs(dot3(S, fo)), SfdNei = fabs(dot3(S, nf3));
        const double w = SfdNei / (SfdOwn + SfdNei);
        T->w[f] = w;
        const double d[3] = {CN[0] - CP[0], CN[1] - CP[1], CN[2] - CP[2]};
        const double magd = sqrt(dot3(d, d));
        const double sd = dot3(Sn, d);
        const double dc = 1.0 / (sd > 0.05 * magd ? sd : 0.05 * magd);
        T->dcoef[f] = dc;
        for (int k = 0; k < 3; k++) T->corrv[3 * f + k] = Sn[k] - d[k] * dc;
        double GP[9], GN[9], G[9];
        cell_sigma(T, P, GP);
        cell_sigma(T, N, GN);
        for (int k = 0; k < 9; k++) G[k] = w * (GP[k] - GN[k]) + GN[k];
        T->sfgsn[f] = face_gamma(S, G, T->sfgcorr + 3 * f);
        T->lap[f] = dc * T->sfgsn[f];
        /* leastSquares dd */
        const double md2 = dot3(d, d);
        double* a = dd + 6 * P;
        double* b = dd + 6 * N;
        const double wdd[6] = {d[0] * d[0] / md2, d[0] * d[1] / md2, d[0] * d[2] / md2,
                               d[1] * d[1] / md2, d[1] * d[2] / md2, d[2] * d[2] / md2};
        for (int k = 0; k < 6; k++) { a[k] += wdd[k]; b[k] += wdd[k]; }
    }
    for (long bf = 0; bf < M->nb; bf++) {
        const long P = M->bcell[bf];
        const double* S = M->bsf + 3 * bf;
        const double magSf = sqrt(dot3(S, S));
        double* n = T->bn + 3 * bf;
        for (int k = 0; k < 3; k++) n[k] = S[k] / magSf;
        double G[9];
        cell_sigma(T, P, G);
        (void)face_gamma(S, G, T->bsfgcorr + 3 * bf);
        const double* Cf = M->bcf + 3 * bf;
        const double* CP = M->centres + 3 * P;
        const double r[3] = {Cf[0] - CP[0], Cf[1] - CP[1], Cf[2] - CP[2]};
        const double nr = dot3(n, r);
        const double d[3] = {n[0] * nr, n[1] * nr, n[2] * nr};
        const double md2 = dot3(d, d);
        double* a = dd + 6 * P;
        a[0] += d[0] * d[0] / md2; a[1] += d[0] * d[1] / md2; a[2] += d[0] * d[2] / md2;
        a[3] += d[1] * d[1] / md2; a[4] += d[1] * d[2] / md2; a[5] += d[2] * d[2] / md2;
    }
    /* invert dd (symmetric 3x3, cofactors over the determinant) */
    for (long c = 0; c < T->n; c++) {
        double* a = dd + 6 * c;
        const double xx = a[0], xy = a[1], xz = a[2], yy = a[3], yz = a[4], zz = a[5];
        const double det = xx * (yy * zz - yz * yz) - xy * (xy * zz - xz * yz) +
                           xz * (xy * yz - yy * xz);
        a[0] = (yy * zz - yz * yz) / det;
        a[1] = (xz * yz - xy * zz) / det;
        a[2] = (xy * yz - xz * yy) / det;
        a[3] = (xx * zz - xz * xz) / det;
        a[4] = (xy * xz - xx * yz) / det;
        a[5] = (xx * yy - xy * xy) / det;
    }
    for (long f = 0; f < nf; f++) {
        const long P = M->owner[f], N = M->neigh[f];
        const double* CP = M->centres + 3 * P;
        const double* CN = M->centres + 3 * N;
        const double d[3] = {CN[0] - CP[0], CN[1] - CP[1], CN[2] - CP[2]};
        const double k = 1.0 / dot3(d, d);
        const double* a = dd + 6 * P;
        const double* b = dd + 6 * N;
        T->lsp[3 * f + 0] = k * (a[0] * d[0] + a[1] * d[1] + a[2] * d[2]);
        T->lsp[3 * f + 1] = k * (a[1] * d[0] + a[3] * d[1] + a[4] * d[2]);
        T->lsp[3 * f + 2] = k * (a[2] * d[0] + a[4] * d[1] + a[5] * d[2]);
        T->lsn[3 * f + 0] = -k * (b[0] * d[0] + b[1] * d[1] + b[2] * d[2]);
        T->lsn[3 * f + 1] = -k * (b[1] * d[0] + b[3] * d[1] + b[4] * d[2]);
        T->lsn[3 * f + 2] = -k * (b[2] * d[0] + b[4] * d[1] + b[5] * d[2]);
    }
    free(dd);
}

/* Cell gradient of phi: leastSquaresGrad::calcGrad (the boundary terms
 * carry phi_b - phi_P = 0 on zeroGradient walls) or gaussGrad (face values
 * by linear interpolation, boundary value phi_P, divided by V). */
static void cell_gradient(oracle_tissue* T, const double* phi, double* g)
{
    const oracle_mesh* M = T->mesh;
    memset(g, 0, sizeof(double) * 3 * (size_t)T->n);
    if (!T->d.grad_gauss) {
        for (long f = 0; f < T->nf; f++) {
            const long P = M->owner[f], N = M->neigh[f];
            const double dv = phi[N] - phi[P];
            for (int k = 0; k < 3; k++) {
                g[3 * P + k] += T->lsp[3 * f + k] * dv;
                g[3 * N + k] -= T->lsn[3 * f + k] * dv;
            }
        }
        return;
    }
    for (long f = 0; f < T->nf; f++) {
        const long P = M->owner[f], N = M->neigh[f];
        const double pf = T->w[f] * (phi[P] - phi[N]) + phi[N];
        for (int k = 0; k < 3; k++) {
            g[3 * P + k] += M->sf[3 * f + k] * pf;
            g[3 * N + k] -= M->sf[3 * f + k] * pf;
        }
    }
    for (long bf = 0; bf < M->nb; bf++) {
        const long P = M->bcell[bf];
        for (int k = 0; k < 3; k++) g[3 * P + k] += M->bsf[3 * bf + k] * phi[P];
    }
    for (long c = 0; c < T->n; c++)
        for (int k = 0; k < 3; k++) g[3 * c + k] /= M->vol[c];
}

/* Boundary value of the gradient on a zeroGradient wall
 * (gaussGrad::correctBoundaryConditions): g + n (snGrad - n.g), snGrad = 0. */
static void boundary_gradient(const double* gP, const double* n, double* gb)
{
    const double ng = dot3(n, gP);
    for (int k = 0; k < 3; k++) gb[k] = gP[k] + n[k] * (0.0 - ng);
}

/* Face flux at one internal face of the explicit correction
 * (gammaSnGradCorr + SfGammaSn * correctedSnGrad::correction): the gradient
 * linearly interpolated to the face (dotInterpolate). */
static double correction_flux(const oracle_tissue* T, long f, const double* g)
{
    const oracle_mesh* M = T->mesh;
    const long P = M->owner[f], N = M->neigh[f];
    const double w = T->w[f];
    double gf[3];
    for (int k = 0; k < 3; k++) gf[k] = w * (g[3 * P + k] - g[3 * N + k]) + g[3 * N + k];
    double flux = dot3(T->sfgcorr + 3 * f, gf);
    if (!T->d.uncorrected) flux += T->sfgsn[f] * dot3(T->corrv + 3 * f, gf);
    return flux;
}

/* fvc::div of the explicit correction fluxes times V (surfaceIntegrate):
 * the Laplacian's fvMatrix source is minus this. */
static void correction_div_v(oracle_tissue* T, const double* vf, double* out)
{
    const oracle_mesh* M = T->mesh;
    double* g = T->grad;
    cell_gradient(T, vf, g);
    double* div = T->fflux;
    memset(div, 0, sizeof(double) * (size_t)T->n);
    for (long f = 0; f < T->nf; f++) {
        const double flux = correction_flux(T, f, g);
        div[M->owner[f]] += flux;
        div[M->neigh[f]] -= flux;
    }
    for (long bf = 0; bf < M->nb; bf++) {
        const long P = M->bcell[bf];
        double gb[3];
        boundary_gradient(g + 3 * P, T->bn + 3 * bf, gb);
        div[P] += dot3(T->bsfgcorr + 3 * bf, gb);
    }
    for (long c = 0; c < T->n; c++) out[c] = M->vol[c] * (div[c] / M->vol[c]);
}

oracle_tissue* oracle_tissue_new(const oracle_tissue_desc* d, const oracle_mesh* mesh)
{
    oracle_tissue* T = (oracle_tissue*)calloc(1, sizeof(oracle_tissue));
    T->d = *d;
    T->mesh = mesh;
    T->n = mesh->n;
    T->nf = mesh->nf;
    long n = T->n, nf = T->nf;
    /* ionicModel::New(coeffs, nCells, runTime.deltaT): the initial ODE step is
     * deltaT in seconds, used as milliseconds by the clamp (TNNP.C:141) */
    T->ionic = NULL;
    T->vm = (double*)malloc(sizeof(double) * (size_t)n);
    T->vm_old = (double*)malloc(sizeof(double) * (size_t)n);
    T->vm_oldold = (double*)malloc(sizeof(double) * (size_t)n);
    T->iion = (double*)calloc((size_t)n, sizeof(double));
    T->src = (double*)calloc((size_t)n, sizeof(double));
    T->act = (double*)calloc((size_t)n, sizeof(double));
    T->calc_act = (unsigned char*)malloc((size_t)n);
    T->lap = (double*)malloc(sizeof(double) * (size_t)(nf + 1));
    T->diag = (double*)malloc(sizeof(double) * (size_t)n);
    T->upper = (double*)malloc(sizeof(double) * (size_t)(nf + 1));
    T->b = (double*)malloc(sizeof(double) * (size_t)n);
    T->rA = (double*)malloc(sizeof(double) * (size_t)n);
    T->wA = (double*)malloc(sizeof(double) * (size_t)n);
    T->pA = (double*)malloc(sizeof(double) * (size_t)n);
    T->rD = (double*)malloc(sizeof(double) * (size_t)n);
    T->tmp = (double*)malloc(sizeof(double) * (size_t)n);
    for (long c = 0; c < n; c++) {
        T->vm[c] = d->vm0;
        T->calc_act[c] = 1;
    }
    if (mesh->cf) {
        T->corrected_mesh = 1;
        T->w = (double*)malloc(sizeof(double) * (size_t)(nf + 1));
        T->dcoef = (double*)malloc(sizeof(double) * (size_t)(nf + 1));
        T->corrv = (double*)malloc(sizeof(double) * 3 * (size_t)(nf + 1));
        T->sfgsn = (double*)malloc(sizeof(double) * (size_t)(nf + 1));
        T->sfgcorr = (double*)malloc(sizeof(double) * 3 * (size_t)(nf + 1));
        T->bsfgcorr = (double*)malloc(sizeof(double) * 3 * (size_t)(mesh->nb + 1));
        T->bn = (double*)malloc(sizeof(double) * 3 * (size_t)(mesh->nb + 1));
        T->lsp = (double*)malloc(sizeof(double) * 3 * (size_t)(nf + 1));
        T->lsn = (double*)malloc(sizeof(double) * 3 * (size_t)(nf + 1));
        T->grad = (double*)malloc(sizeof(double) * 3 * (size_t)n);
        T->fflux = (double*)malloc(sizeof(double) * (size_t)n);
    }
    assemble_laplacian(T);
    return T;
}

/* Per-cell conductivity [n][6] (xx xy xz yy yz zz), as read from a
 * 0/conductivity volTensorField (monodomainSolver.C:48-100); boundary faces
 * take their cell's value.  Re-assembles the Laplacian. */
void oracle_tissue_set_conductivity(oracle_tissue* T, const double* sigma6)
{
    if (!T->sigma_cell) T->sigma_cell = (double*)malloc(sizeof(double) * 6 * (size_t)T->n);
    memcpy(T->sigma_cell, sigma6, sizeof(double) * 6 * (size_t)T->n);
    assemble_laplacian(T);
}

/* Tissue flag per cell for the ionic model (before its first step). */
int oracle_tissue_set_cell_tissue(oracle_tissue* T, const unsigned char* flags)
{
    if (T->ionic) return -1;
    if (!T->tissue_cell) T->tissue_cell = (unsigned char*)malloc((size_t)T->n);
    memcpy(T->tissue_cell, flags, (size_t)T->n);
    return 0;
}

void oracle_tissue_free(oracle_tissue* T)
{
    if (!T) return;
    oracle_ionic_free(T->ionic);
    free(T->vm); free(T->vm_old); free(T->vm_oldold); free(T->iion); free(T->src);
    free(T->act); free(T->calc_act); free(T->lap); free(T->diag); free(T->upper);
    free(T->b); free(T->rA); free(T->wA); free(T->pA); free(T->rD); free(T->tmp);
    free(T->sigma_cell); free(T->tissue_cell);
    free(T->w); free(T->dcoef); free(T->corrv); free(T->sfgsn); free(T->sfgcorr);
    free(T->bsfgcorr); free(T->bn); free(T->lsp); free(T->lsn); free(T->grad); free(T->fflux);
    free(T);
}

double oracle_tissue_time(const oracle_tissue* T) { return T->t; }
double* oracle_tissue_vm(oracle_tissue* T) { return T->vm; }
double* oracle_tissue_iion(oracle_tissue* T) { return T->iion; }
double* oracle_tissue_activation(oracle_tissue* T) { return T->act; }
double* oracle_tissue_source(oracle_tissue* T) { return T->src; }
oracle_ionic* oracle_tissue_ionic(oracle_tissue* T) { return T->ionic; }

int oracle_tissue_last_solves(const oracle_tissue* T, double* ir, double* fr, int* it, int mx)
{
    int k = T->n_solves < mx ? T->n_solves : mx;
    for (int i = 0; i < k; i++) {
        ir[i] = T->init_res[i];
        fr[i] = T->final_res[i];
        it[i] = T->iters[i];
    }
    return T->n_solves;
}

/* lduMatrix::Amul for the symmetric matrix (diag, upper) */
static void amul(const oracle_tissue* T, const double* x, double* y)
{
    const int* l = T->mesh->owner;
    const int* u = T->mesh->neigh;
    for (long c = 0; c < T->n; c++) y[c] = T->diag[c] * x[c];
    for (long f = 0; f < T->nf; f++) {
        y[u[f]] += T->upper[f] * x[l[f]];
        y[l[f]] += T->upper[f] * x[u[f]];
    }
}

/* lduMatrix::solver::normFactor */
static double norm_factor(const oracle_tissue* T, const double* psi, const double* src,
                          const double* Apsi)
{
    const int* l = T->mesh->owner;
    const int* u = T->mesh->neigh;
    double* sumA = T->tmp;
    for (long c = 0; c < T->n; c++) sumA[c] = T->diag[c];
    for (long f = 0; f < T->nf; f++) {
        sumA[u[f]] += T->upper[f];
        sumA[l[f]] += T->upper[f];
    }
    double avg = 0.0;
    for (long c = 0; c < T->n; c++) avg += psi[c];
    avg /= (double)T->n;
    double nf = 0.0;
    for (long c = 0; c < T->n; c++) {
        double pa = sumA[c] * avg;
        nf += fabs(Apsi[c] - pa) + fabs(src[c] - pa);
    }
    return nf + 1e-20;
}

static void precondition(const oracle_tissue* T, double* wA, const double* rA)
{
    const double* rD = T->rD;
    for (long c = 0; c < T->n; c++) wA[c] = rD[c] * rA[c];
    if (!T->d.precond_dic) return;
    const int* l = T->mesh->owner;
    const int* u = T->mesh->neigh;
    for (long f = 0; f < T->nf; f++) wA[u[f]] -= rD[u[f]] * T->upper[f] * wA[l[f]];
    for (long f = T->nf - 1; f >= 0; f--) wA[l[f]] -= rD[l[f]] * T->upper[f] * wA[u[f]];
}

/* PCG::solve (lduMatrix), returns iterations */
static int pcg(oracle_tissue* T, double* psi, const double* src, double* init_res,
               double* final_res)
{
    long n = T->n;
    double *wA = T->wA, *rA = T->rA, *pA = T->pA;
    amul(T, psi, wA);
    for (long c = 0; c < n; c++) rA[c] = src[c] - wA[c];
    double normf = norm_factor(T, psi, src, wA);
    double s = 0.0;
    for (long c = 0; c < n; c++) s += fabs(rA[c]);
    double res = s / normf;
    *init_res = res;
    int it = 0;
    const double tol = T->d.pcg_tol, rel = T->d.pcg_rel_tol;
#define CONVERGED(r) ((r) < tol || (rel > 1e-20 && (r) < rel * (*init_res)))
    if (!CONVERGED(res)) {
        /* preconditioner set-up (DIC: calcReciprocalD; diagonal: 1/diag) */
        for (long c = 0; c < n; c++) T->rD[c] = T->diag[c];
        if (T->d.precond_dic) {
            const int* l = T->mesh->owner;
            const int* u = T->mesh->neigh;
            for (long f = 0; f < T->nf; f++)
                T->rD[u[f]] -= T->upper[f] * T->upper[f] / T->rD[l[f]];
        }
        for (long c = 0; c < n; c++) T->rD[c] = 1.0 / T->rD[c];
        double wArA = 1e300, wArAold;
        do {
            wArAold = wArA;
            precondition(T, wA, rA);
            wArA = 0.0;
            for (long c = 0; c < n; c++) wArA += wA[c] * rA[c];
            if (it == 0) {
                for (long c = 0; c < n; c++) pA[c] = wA[c];
            } else {
                double beta = wArA / wArAold;
                for (long c = 0; c < n; c++) pA[c] = wA[c] + beta * pA[c];
            }
            amul(T, pA, wA);
            double wApA = 0.0;
            for (long c = 0; c < n; c++) wApA += wA[c] * pA[c];
            if (fabs(wApA) / normf < 1e-300) break;   /* checkSingularity */
            double alpha = wArA / wApA;
            for (long c = 0; c < n; c++) {
                psi[c] += alpha * pA[c];
                rA[c] -= alpha * wA[c];
            }
            s = 0.0;
            for (long c = 0; c < n; c++) s += fabs(rA[c]);
            res = s / normf;
        } while (++it < T->d.pcg_max_iter && !CONVERGED(res));
    }
#undef CONVERGED
    *final_res = res;
    return it;
}

/* MyocardiumDomain::updateExternalStimulusCurrent (myocardiumDomain.C:307-342) */
static void update_stimulus(oracle_tissue* T, double t0)
{
    for (long c = 0; c < T->n; c++) T->src[c] = 0.0;
    for (int b = 0; b < T->d.n_boxes; b++) {
        double ts = T->d.box_start[b], te = ts + T->d.box_duration[b];
        if (t0 < ts || t0 > te) continue;
        for (long c = 0; c < T->n; c++) {
            const double* p = T->mesh->centres + 3 * c;
            if (p[0] >= T->d.box_min[b][0] && p[0] <= T->d.box_max[b][0] &&
                p[1] >= T->d.box_min[b][1] && p[1] <= T->d.box_max[b][1] &&
                p[2] >= T->d.box_min[b][2] && p[2] <= T->d.box_max[b][2])
                T->src[c] += T->d.box_intensity[b];
        }
    }
    /* PVJMapper::depositCoupling (pvjMapper.C) on top of the box stimulus */
    if (T->dep_value)
        for (long k = 0; k < T->n_dep; k++) T->src[T->dep_cell[k]] += T->dep_value[T->dep_term[k]];
}

/* ddt coefficients (EulerDdtScheme / backwardDdtScheme); backward uses
 * deltaT0 = GREAT while fewer than two old-time levels are stored */
static void ddt_coeffs(const oracle_tissue* T, double dt, double* cft, double* cft0,
                       double* cft00)
{
    if (!T->d.ddt_backward) {
        *cft = 1.0; *cft0 = 1.0; *cft00 = 0.0;
        return;
    }
    double dt0 = T->n_old < 2 ? 1e15 : dt;
    *cft = 1 + dt / (dt + dt0);
    *cft00 = dt * dt / (dt0 * (dt + dt0));
    *cft0 = *cft + *cft00;
}

/* one fvMatrix assembly + solve of chi*Cm*ddt(Vm) == laplacian - chi*Cm*Iion + src */
static int solve_implicit(oracle_tissue* T, double dt)
{
    double cft, cft0, cft00;
    /* fvm::ddt accesses Vm.oldTime() and Vm.oldTime().oldTime() (backward):
     * the first access creates each level as a copy of the newer one */
    int n_old_before = T->n_old;
    ddt_coeffs(T, dt, &cft, &cft0, &cft00);
    if (T->n_old < 1) { memcpy(T->vm_old, T->vm, sizeof(double) * (size_t)T->n); T->n_old = 1; }
    if (T->d.ddt_backward && T->n_old < 2) {
        memcpy(T->vm_oldold, T->vm_old, sizeof(double) * (size_t)T->n);
        T->n_old = 2;
    }
    (void)n_old_before;
    const double chicm = T->d.chi * T->d.cm;
    const double rdt = 1.0 / dt;
    const double* V = T->mesh->vol;
    for (long c = 0; c < T->n; c++) {
        double ddt_diag, ddt_src;
        if (T->d.ddt_backward) {
            ddt_diag = (cft * rdt) * V[c];
            ddt_src = rdt * V[c] * (cft0 * T->vm_old[c] - cft00 * T->vm_oldold[c]);
        } else {
            ddt_diag = rdt * V[c];
            ddt_src = rdt * T->vm_old[c] * V[c];
        }
        T->diag[c] = chicm * ddt_diag;
        T->b[c] = chicm * ddt_src;
    }
    /* minus the Laplacian: upper = -coef, diag += sum coef (negSumDiag) */
    const int* l = T->mesh->owner;
    const int* u = T->mesh->neigh;
    for (long f = 0; f < T->nf; f++) T->upper[f] = -T->lap[f];
    {
        double* lapdiag = T->tmp;
        for (long c = 0; c < T->n; c++) lapdiag[c] = 0.0;
        for (long f = 0; f < T->nf; f++) {
            lapdiag[l[f]] -= T->lap[f];
            lapdiag[u[f]] -= T->lap[f];
        }
        for (long c = 0; c < T->n; c++) T->diag[c] = T->diag[c] - lapdiag[c];
    }
    /* explicit sources: -(chi*Cm*Iion) + src, each times V */
    for (long c = 0; c < T->n; c++) {
        double su = -(chicm * T->iion[c]) * V[c];
        su = su + T->src[c] * V[c];
        T->b[c] = T->b[c] + su;
    }
    /* general mesh: the Laplacian's explicit correction of the current Vm
     * (fvm.source() -= V*fvc::div(faceFluxCorrection), on the other side
     * of ==) */
    if (T->corrected_mesh) {
        double* cv = T->tmp;
        correction_div_v(T, T->vm, cv);
        for (long c = 0; c < T->n; c++) T->b[c] = T->b[c] + cv[c];
    }
    if (T->extra_src)
        for (long c = 0; c < T->n; c++) T->b[c] = T->b[c] + T->extra_src[c];
    int k = T->n_solves;
    if (k >= MAX_SOLVES) return -1;
    int it = pcg(T, T->vm, T->b, &T->init_res[k], &T->final_res[k]);
    T->iters[k] = it;
    T->n_solves++;
    return it;
}

/* explicit form: chi*Cm*ddt(Vm) == fvc::laplacian(sigma,Vm) - chi*Cm*Iion + src */
static int solve_explicit(oracle_tissue* T, double dt)
{
    double cft, cft0, cft00;
    ddt_coeffs(T, dt, &cft, &cft0, &cft00);
    if (T->n_old < 1) { memcpy(T->vm_old, T->vm, sizeof(double) * (size_t)T->n); T->n_old = 1; }
    if (T->d.ddt_backward && T->n_old < 2) {
        memcpy(T->vm_oldold, T->vm_old, sizeof(double) * (size_t)T->n);
        T->n_old = 2;
    }
    const double chicm = T->d.chi * T->d.cm;
    const double rdt = 1.0 / dt;
    const double* V = T->mesh->vol;
    const int* l = T->mesh->owner;
    const int* u = T->mesh->neigh;
    double* div = T->tmp;
    for (long c = 0; c < T->n; c++) div[c] = 0.0;
    if (T->corrected_mesh) {
        /* fvc::laplacian = fvc::div(SfGammaSn*snGrad(Vm) + gammaSnGradCorr)
         * with snGrad = deltaCoeffs*(Vm_N - Vm_P) + correction */
        double* g = T->grad;
        cell_gradient(T, T->vm, g);
        for (long f = 0; f < T->nf; f++) {
            const long P = l[f], N = u[f];
            const double w = T->w[f];
            double gf[3];
            for (int k = 0; k < 3; k++) gf[k] = w * (g[3 * P + k] - g[3 * N + k]) + g[3 * N + k];
            double sn = T->dcoef[f] * (T->vm[N] - T->vm[P]);
            if (!T->d.uncorrected) sn = sn + dot3(T->corrv + 3 * f, gf);
            const double flux = T->sfgsn[f] * sn + dot3(T->sfgcorr + 3 * f, gf);
            div[P] += flux;
            div[N] -= flux;
        }
        for (long bf = 0; bf < T->mesh->nb; bf++) {
            const long P = T->mesh->bcell[bf];
            double gb[3];
            boundary_gradient(g + 3 * P, T->bn + 3 * bf, gb);
            div[P] += dot3(T->bsfgcorr + 3 * bf, gb);
        }
    } else {
        for (long f = 0; f < T->nf; f++) {
            double flux = T->lap[f] * (T->vm[u[f]] - T->vm[l[f]]);
            div[l[f]] += flux;
            div[u[f]] -= flux;
        }
    }
    for (long c = 0; c < T->n; c++) {
        double diag, src;
        if (T->d.ddt_backward) {
            diag = chicm * ((cft * rdt) * V[c]);
            src = chicm * (rdt * V[c] * (cft0 * T->vm_old[c] - cft00 * T->vm_oldold[c]));
        } else {
            diag = chicm * (rdt * V[c]);
            src = chicm * (rdt * T->vm_old[c] * V[c]);
        }
        double lapc = div[c] / V[c];
        double rhs = lapc - chicm * T->iion[c] + T->src[c];
        src = src + rhs * V[c];
        T->vm[c] = src / diag;
    }
    return 0;
}

/* fvc::laplacian(sigma, phi) per cell (the explicit form's operator),
 * for checks of the discretisation on given fields. */
void oracle_tissue_laplacian(oracle_tissue* T, const double* phi, double* out)
{
    double* save = T->vm;
    T->vm = (double*)phi;
    const int* l = T->mesh->owner;
    const int* u = T->mesh->neigh;
    double* div = out;
    for (long c = 0; c < T->n; c++) div[c] = 0.0;
    if (T->corrected_mesh) {
        double* g = T->grad;
        cell_gradient(T, phi, g);
        for (long f = 0; f < T->nf; f++) {
            const long P = l[f], N = u[f];
            const double w = T->w[f];
            double gf[3];
            for (int k = 0; k < 3; k++) gf[k] = w * (g[3 * P + k] - g[3 * N + k]) + g[3 * N + k];
            double sn = T->dcoef[f] * (phi[N] - phi[P]);
            if (!T->d.uncorrected) sn = sn + dot3(T->corrv + 3 * f, gf);
            const double flux = T->sfgsn[f] * sn + dot3(T->sfgcorr + 3 * f, gf);
            div[P] += flux;
            div[N] -= flux;
        }
        for (long bf = 0; bf < T->mesh->nb; bf++) {
            const long P = T->mesh->bcell[bf];
            double gb[3];
            boundary_gradient(g + 3 * P, T->bn + 3 * bf, gb);
            div[P] += dot3(T->bsfgcorr + 3 * bf, gb);
        }
    } else {
        for (long f = 0; f < T->nf; f++) {
            const double flux = T->lap[f] * (phi[u[f]] - phi[l[f]]);
            div[l[f]] += flux;
            div[u[f]] -= flux;
        }
    }
    for (long c = 0; c < T->n; c++) div[c] /= T->mesh->vol[c];
    T->vm = save;
}

/* Cell gradient of phi with the tissue's gradient scheme (general mesh). */
int oracle_tissue_gradient(oracle_tissue* T, const double* phi, double* g)
{
    if (!T->corrected_mesh) return -1;
    cell_gradient(T, phi, g);
    return 0;
}

/* PseudoECGSolver::compute (pseudoECGSolver.C:34-87): for each electrode P,
 * sum over cells of ((sigma_c . grad(Vm)_c) V_c) . r / |r|^3 with r = C_c - P
 * (cells at |r| <= VSMALL skipped), grad the tissue's gradient scheme. */
int oracle_tissue_pseudo_ecg(oracle_tissue* T, const double* vm, int n_el, const double* el,
                             double* out)
{
    if (!T->corrected_mesh) return -1;
    double* g = (double*)malloc(sizeof(double) * 3 * (size_t)T->n);
    cell_gradient(T, vm, g);
    const oracle_mesh* M = T->mesh;
    for (int e = 0; e < n_el; e++) out[e] = 0.0;
    for (long c = 0; c < T->n; c++) {
        double S[9];
        cell_sigma(T, c, S);
        const double* gc = g + 3 * c;
        double dip[3];
        for (int i = 0; i < 3; i++)
            dip[i] = (S[3 * i] * gc[0] + S[3 * i + 1] * gc[1] + S[3 * i + 2] * gc[2]) * M->vol[c];
        const double* C = M->centres + 3 * c;
        for (int e = 0; e < n_el; e++) {
            const double r[3] = {C[0] - el[3 * e], C[1] - el[3 * e + 1], C[2] - el[3 * e + 2]};
            const double m = sqrt(dot3(r, r));
            if (m > 1e-300) out[e] += dot3(dip, r) / (m * m * m);
        }
    }
    free(g);
    return 0;
}

/* MyocardiumDomain::updateActivationTime (myocardiumDomain.C:345-374) */
static void update_activation(oracle_tissue* T, double dt)
{
    const double old_time = T->t - dt;
    for (long c = 0; c < T->n; c++) {
        if (T->calc_act[c] && T->vm[c] > 1e-15) {
            T->calc_act[c] = 0;
            double w = (0.0 - T->vm_old[c]) / (T->vm[c] - T->vm_old[c]);
            T->act[c] = old_time + w * dt;
        }
    }
}

/* The ionic model of the tissue, constructed with initialDeltaT = dt as
 * the domain constructs it; done by the first step when not called before
 * (e.g. to import states first). */
int oracle_tissue_init_ionic(oracle_tissue* T, double dt)
{
    if (!T->ionic)
        T->ionic = oracle_ionic_new_cells(T->d.model, T->n, T->d.tissue, T->tissue_cell, dt, 0,
                                          &T->d.ode, NULL, NULL);
    return T->ionic ? 0 : -1;
}

/* Advance by dt [s]: runTime++ then electroModel::evolve with the staggered
 * advance scheme (stimulus -> ionic -> diffusion -> activation time). */
int oracle_tissue_step(oracle_tissue* T, double dt, int nthreads)
{
    if (oracle_tissue_init_ionic(T, dt)) return -1;
    /* Time::operator++ : value += deltaT; store old-time levels of Vm */
    T->t = T->t + dt;
    T->time_index++;
    if (T->n_old >= 1) {
        if (T->n_old >= 2) memcpy(T->vm_oldold, T->vm_old, sizeof(double) * (size_t)T->n);
        memcpy(T->vm_old, T->vm, sizeof(double) * (size_t)T->n);
    }
    const double t0 = T->t - dt;
    update_stimulus(T, t0);
    if (oracle_ionic_solve(T->ionic, t0, dt, T->vm, T->iion, nthreads) < 0) return -1;
    T->n_solves = 0;
    int total = 0;
    if (T->d.implicit) {
        /* pimpleControl loop: from the second corrector on, residualControl
         * compares the initial residual of the latest Vm solve with the
         * tolerance; once met, one final corrector still runs, then the loop
         * ends (pimpleLoop::loop / criteriaSatisfied, restated) */
        int converged = 0;
        for (int corr = 1; corr <= T->d.n_outer && !converged; corr++) {
            if (corr > 1 && T->init_res[T->n_solves - 1] < T->d.outer_tol) converged = 1;
            int it = solve_implicit(T, dt);
            if (it < 0) return -1;
            total += it;
        }
    } else {
        solve_explicit(T, dt);
    }
    if (T->n_old < 1) { memcpy(T->vm_old, T->vm, sizeof(double) * (size_t)T->n); T->n_old = 1; }
    update_activation(T, dt);
    return total;
}

/* ------------------------------------------------------------------------ */
/* bidomain                                                                 */

/* BidomainSolver (bidomainSolver.C:36-263) on a general mesh: the tissue Ti
 * carries Vm, the ionic model, the stimulus, the activation time and the
 * Laplacian of the intracellular conductivity Gi; Te carries the Laplacian of
 * Gi + Ge for phiE. */
struct oracle_bidomain {
    oracle_tissue* Ti;
    oracle_tissue* Te;
    double *phie, *phii, *dv, *ue, *src;
    long ref;
    double ref_value;
    double phie_tol, phie_rel_tol;
    int phie_max_iter;
    int n_solves;
    double init_res[MAX_SOLVES], final_res[MAX_SOLVES];
    int iters[MAX_SOLVES];
};

/* V fvc::div(G & fvc::grad(x)) with Gauss linear divergence: the cell
 * vectors G g linearly interpolated to the faces, the wall values
 * G (g - n (n.g)) (gaussGrad::correctBoundaryConditions on zeroGradient
 * walls; a per-cell G takes its cell's value on the wall). */
static void div_gamma_grad_v(oracle_tissue* T, const double* x, double* out, double* u)
{
    const oracle_mesh* M = T->mesh;
    double* g = T->grad;
    cell_gradient(T, x, g);
    for (long c = 0; c < T->n; c++) {
        double S[9];
        cell_sigma(T, c, S);
        const double* gc = g + 3 * c;
        for (int i = 0; i < 3; i++)
            u[3 * c + i] = S[3 * i] * gc[0] + S[3 * i + 1] * gc[1] + S[3 * i + 2] * gc[2];
    }
    double* div = T->fflux;
    memset(div, 0, sizeof(double) * (size_t)T->n);
    for (long f = 0; f < T->nf; f++) {
        const long P = M->owner[f], N = M->neigh[f];
        double uf[3];
        for (int k = 0; k < 3; k++) uf[k] = T->w[f] * (u[3 * P + k] - u[3 * N + k]) + u[3 * N + k];
        const double flux = dot3(M->sf + 3 * f, uf);
        div[P] += flux;
        div[N] -= flux;
    }
    for (long bf = 0; bf < M->nb; bf++) {
        const long P = M->bcell[bf];
        double gb[3], S[9], ub[3];
        boundary_gradient(g + 3 * P, T->bn + 3 * bf, gb);
        cell_sigma(T, P, S);
        for (int i = 0; i < 3; i++) ub[i] = S[3 * i] * gb[0] + S[3 * i + 1] * gb[1] + S[3 * i + 2] * gb[2];
        div[P] += dot3(M->bsf + 3 * bf, ub);
    }
    for (long c = 0; c < T->n; c++) out[c] = M->vol[c] * (div[c] / M->vol[c]);
}

/* polyMesh::findCell restated for the reference point: the cell whose centre
 * is nearest (the first in cell order on ties). */
static long nearest_cell(const oracle_mesh* M, const double* p)
{
    long best = -1;
    double bd = 0.0;
    for (long c = 0; c < M->n; c++) {
        const double* C = M->centres + 3 * c;
        const double d = (C[0] - p[0]) * (C[0] - p[0]) + (C[1] - p[1]) * (C[1] - p[1]) +
                         (C[2] - p[2]) * (C[2] - p[2]);
        if (best < 0 || d < bd) { best = c; bd = d; }
    }
    return best;
}

oracle_bidomain* oracle_bidomain_new(const oracle_tissue_desc* d, const double* sigma_e,
                                     const oracle_mesh* mesh, const double* ref_point,
                                     double ref_value, double phie_tol, double phie_rel_tol,
                                     int phie_max_iter)
{
    if (!mesh->cf) return NULL;
    oracle_bidomain* B = (oracle_bidomain*)calloc(1, sizeof(oracle_bidomain));
    B->Ti = oracle_tissue_new(d, mesh);
    oracle_tissue_desc de = *d;
    for (int k = 0; k < 6; k++) de.sigma[k] = d->sigma[k] + sigma_e[k];
    B->Te = oracle_tissue_new(&de, mesh);
    long n = mesh->n;
    B->phie = (double*)calloc((size_t)n, sizeof(double));
    B->phii = (double*)calloc((size_t)n, sizeof(double));
    B->dv = (double*)malloc(sizeof(double) * (size_t)n);
    B->src = (double*)malloc(sizeof(double) * (size_t)n);
    B->ue = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    B->ref = nearest_cell(mesh, ref_point);
    B->ref_value = ref_value;
    B->phie_tol = phie_tol;
    B->phie_rel_tol = phie_rel_tol;
    B->phie_max_iter = phie_max_iter;
    return B;
}

void oracle_bidomain_free(oracle_bidomain* B)
{
    if (!B) return;
    oracle_tissue_free(B->Ti);
    oracle_tissue_free(B->Te);
    free(B->phie); free(B->phii); free(B->dv); free(B->src); free(B->ue);
    free(B);
}

oracle_tissue* oracle_bidomain_tissue(oracle_bidomain* B) { return B->Ti; }
double* oracle_bidomain_phie(oracle_bidomain* B) { return B->phie; }
double* oracle_bidomain_phii(oracle_bidomain* B) { return B->phii; }
long oracle_bidomain_ref_cell(const oracle_bidomain* B) { return B->ref; }

int oracle_bidomain_last_solves(const oracle_bidomain* B, double* ir, double* fr, int* it, int mx)
{
    int k = B->n_solves < mx ? B->n_solves : mx;
    for (int i = 0; i < k; i++) {
        ir[i] = B->init_res[i];
        fr[i] = B->final_res[i];
        it[i] = B->iters[i];
    }
    return B->n_solves;
}

/* fvm::laplacian(Gi + Ge, phiE) == -fvc::div(Gi & fvc::grad(Vm)) with
 * setReference(refCell, phiEReferenceValue, true)
 * (bidomainSolver.C:222-233; fvMatrix::setReference: source += diag value,
 * diag += diag), solved in its own (negative definite) form by PCG. */
static int solve_phie(oracle_bidomain* B)
{
    oracle_tissue* Te = B->Te;
    oracle_tissue* Ti = B->Ti;
    const int* l = Te->mesh->owner;
    const int* u = Te->mesh->neigh;
    for (long c = 0; c < Te->n; c++) Te->diag[c] = 0.0;
    for (long f = 0; f < Te->nf; f++) {
        Te->upper[f] = Te->lap[f];
        Te->diag[l[f]] -= Te->lap[f];
        Te->diag[u[f]] -= Te->lap[f];
    }
    div_gamma_grad_v(Ti, Ti->vm, B->dv, B->ue);
    for (long c = 0; c < Te->n; c++) B->src[c] = -B->dv[c];
    /* the Laplacian's explicit correction of the current phiE (general
     * meshes): fvm.source() -= V fvc::div(faceFluxCorrection) */
    if (Te->corrected_mesh) {
        double* cv = Te->tmp;
        correction_div_v(Te, B->phie, cv);
        for (long c = 0; c < Te->n; c++) B->src[c] = B->src[c] - cv[c];
    }
    if (B->ref >= 0) {
        B->src[B->ref] += Te->diag[B->ref] * B->ref_value;
        Te->diag[B->ref] += Te->diag[B->ref];
    }
    const double tol = Te->d.pcg_tol, rel = Te->d.pcg_rel_tol;
    const int mx = Te->d.pcg_max_iter;
    Te->d.pcg_tol = B->phie_tol;
    Te->d.pcg_rel_tol = B->phie_rel_tol;
    Te->d.pcg_max_iter = B->phie_max_iter;
    int k = B->n_solves;
    if (k >= MAX_SOLVES) return -1;
    int it = pcg(Te, B->phie, B->src, &B->init_res[k], &B->final_res[k]);
    B->iters[k] = it;
    B->n_solves++;
    Te->d.pcg_tol = tol; Te->d.pcg_rel_tol = rel; Te->d.pcg_max_iter = mx;
    return it;
}

/* One runTime++ / evolve() of the bidomain domain: stimulus, ionic, then
 * per PIMPLE corrector the phiE solve and the Vm solve
 *   chi Cm ddt(Vm) == laplacian(Gi, Vm) + fvc::div(Gi & grad(phiE)) - chi Cm Iion + src
 * (bidomainSolver.C:215-261), phiI = Vm + phiE, activation time. */
int oracle_bidomain_step(oracle_bidomain* B, double dt, int nthreads)
{
    oracle_tissue* T = B->Ti;
    if (oracle_tissue_init_ionic(T, dt)) return -1;
    T->t = T->t + dt;
    T->time_index++;
    if (T->n_old >= 1) {
        if (T->n_old >= 2) memcpy(T->vm_oldold, T->vm_old, sizeof(double) * (size_t)T->n);
        memcpy(T->vm_old, T->vm, sizeof(double) * (size_t)T->n);
    }
    const double t0 = T->t - dt;
    update_stimulus(T, t0);
    if (oracle_ionic_solve(T->ionic, t0, dt, T->vm, T->iion, nthreads) < 0) return -1;
    T->n_solves = 0;
    B->n_solves = 0;
    int total = 0, converged = 0;
    if (!T->d.implicit) {
        /* BidomainSolver::solveDiffusionExplicit (bidomainSolver.C:183-213):
         * the phiE solve, then chi*Cm*ddt(Vm) == fvc::div(Gi & fvc::grad(Vm +
         * phiE)) - chi*Cm*Iion + src with the diagonal ddt matrix, solved as
         * source over diagonal */
        int it = solve_phie(B);
        if (it < 0) return -1;
        double cft, cft0, cft00;
        ddt_coeffs(T, dt, &cft, &cft0, &cft00);
        if (T->n_old < 1) { memcpy(T->vm_old, T->vm, sizeof(double) * (size_t)T->n); T->n_old = 1; }
        if (T->d.ddt_backward && T->n_old < 2) {
            memcpy(T->vm_oldold, T->vm_old, sizeof(double) * (size_t)T->n);
            T->n_old = 2;
        }
        for (long c = 0; c < T->n; c++) B->phii[c] = T->vm[c] + B->phie[c];
        div_gamma_grad_v(T, B->phii, B->dv, B->ue);
        const double chicm = T->d.chi * T->d.cm;
        const double rdt = 1.0 / dt;
        const double* V = T->mesh->vol;
        for (long c = 0; c < T->n; c++) {
            double ddt_diag, ddt_src;
            if (T->d.ddt_backward) {
                ddt_diag = (cft * rdt) * V[c];
                ddt_src = rdt * V[c] * (cft0 * T->vm_old[c] - cft00 * T->vm_oldold[c]);
            } else {
                ddt_diag = rdt * V[c];
                ddt_src = rdt * T->vm_old[c] * V[c];
            }
            double bb = chicm * ddt_src;
            double su = -(chicm * T->iion[c]) * V[c];
            su = su + T->src[c] * V[c];
            bb = bb + su;
            T->vm[c] = (bb + B->dv[c]) / (chicm * ddt_diag);
        }
        for (long c = 0; c < T->n; c++) B->phii[c] = T->vm[c] + B->phie[c];
        update_activation(T, dt);
        return it;
    }
    for (int corr = 1; corr <= T->d.n_outer && !converged; corr++) {
        if (corr > 1 && T->init_res[T->n_solves - 1] < T->d.outer_tol) converged = 1;
        int it = solve_phie(B);
        if (it < 0) return -1;
        total += it;
        div_gamma_grad_v(T, B->phie, B->dv, B->ue);
        T->extra_src = B->dv;
        it = solve_implicit(T, dt);
        T->extra_src = NULL;
        if (it < 0) return -1;
        total += it;
        for (long c = 0; c < T->n; c++) B->phii[c] = T->vm[c] + B->phie[c];
    }
    if (T->n_old < 1) { memcpy(T->vm_old, T->vm, sizeof(double) * (size_t)T->n); T->n_old = 1; }
    update_activation(T, dt);
    return total;
}

/* ------------------------------------------------------------------------ */
/* single cell                                                              */

long oracle_single_cell(int model, int tissue, double dt, long n_steps,
                        const oracle_ode_settings* ode, const oracle_stimulus* stim,
                        const double* scales, double* vm_trace, double* final_states)
{
    return oracle_single_cell_traces(model, tissue, dt, n_steps, ode, stim, scales, vm_trace,
                                     -1, NULL, final_states);
}

/* The same, also tracing state `state_b` (e.g. intracellular Ca) after each
 * step when b_trace is given. */
long oracle_single_cell_traces(int model, int tissue, double dt, long n_steps,
                               const oracle_ode_settings* ode, const oracle_stimulus* stim,
                               const double* scales, double* vm_trace, int state_b,
                               double* b_trace, double* final_states)
{
    oracle_ionic* io = oracle_ionic_new(model, 1, tissue, dt, 1, ode, stim, scales);
    if (!io) return -1;
    const model_info* m = io->m;
    double t = 0.0, dummy_vm = 0.0, dummy_im = 0.0;
    long total = 0;
    for (long s = 0; s < n_steps; s++) {
        t = t + dt;
        long k = oracle_ionic_solve(io, t - dt, dt, &dummy_vm, &dummy_im, 1);
        if (k < 0) { oracle_ionic_free(io); return -1; }
        total += k;
        double u = io->y[0];
        double vm = m->vm_map == 1 ? u * 100 - 80 : m->vm_map == 2 ? u * 85.7 - 84.0 : u;
        if (vm_trace) vm_trace[s] = vm;
        if (b_trace && state_b >= 0) b_trace[s] = io->y[state_b];
    }
    if (final_states) memcpy(final_states, io->y, sizeof(double) * (size_t)m->ns);
    oracle_ionic_free(io);
    return total;
}

/* ------------------------------------------------------------------------ */
/* Purkinje network                                                          */

/* ConductionSystemDomain with Monodomain1DSolver
 * (src/electroModels/electroDomains/conductionSystemDomain/conductionSystemDomain.C,
 * conductionGraph.H; src/electroModels/conductionSystemModels/monodomain1DSolver/
 * monodomain1DSolver.C:36-190) and the reaction-diffusion PVJ coupling
 * (electroCouplers/pvjCoupler/reactionDiffusion/reactionDiffusionPvjCoupler.C:36-164,
 * pvjMapper.C), restated.  The graph is a tree rooted at node 0: BFS order
 * over adjacency lists built in edge order, parent links, reverse BFS order
 * for the elimination. */
struct oracle_purkinje {
    long n, ne;
    int *ea, *eb;
    double *elen, *econd;
    int *parent, *order, *rev;
    double chi, cm;
    oracle_ionic* ionic;
    double *vm, *iion, *app;
    double *diag, *rhs, *pc, *cc, *clen;
    int root;
    double root_start, root_dur, root_int;
    long n_term;
    int* term_node;
    double* term_loc;
    double* term_current;     /* setTerminalCoupling's current [(V)/R] */
    /* coupling */
    int coupled, mode;        /* mode 0: unidirectional, 1: bidirectional */
    double r_pvj, radius;
    long* term_cell;
    long n_dep;
    long *dep_cell, *dep_term;
    double *sphere_vol, *dep_value, *tissue_vm_buf, *net_vm_buf;
};

oracle_purkinje* oracle_purkinje_new(long n_edges, const int* ea, const int* eb, const double* len,
                                     const double* cond, int model, int tissue,
                                     const oracle_ode_settings* ode, double initial_dt,
                                     double chi, double cm, int root, double root_start,
                                     double root_dur, double root_int, long n_term,
                                     const int* term_node, const double* term_loc)
{
    int maxn = 0;
    for (long e = 0; e < n_edges; e++) {
        if (ea[e] < 0 || eb[e] < 0) return NULL;
        if (ea[e] > maxn) maxn = ea[e];
        if (eb[e] > maxn) maxn = eb[e];
    }
    const long n = (long)maxn + 1;
    if (n < 1 || n_edges != n - 1) return NULL;   /* a tree: N - 1 edges */
    oracle_purkinje* P = (oracle_purkinje*)calloc(1, sizeof(oracle_purkinje));
    P->n = n;
    P->ne = n_edges;
    P->ea = (int*)malloc(sizeof(int) * (size_t)n_edges);
    P->eb = (int*)malloc(sizeof(int) * (size_t)n_edges);
    P->elen = (double*)malloc(sizeof(double) * (size_t)n_edges);
    P->econd = (double*)malloc(sizeof(double) * (size_t)n_edges);
    memcpy(P->ea, ea, sizeof(int) * (size_t)n_edges);
    memcpy(P->eb, eb, sizeof(int) * (size_t)n_edges);
    memcpy(P->elen, len, sizeof(double) * (size_t)n_edges);
    memcpy(P->econd, cond, sizeof(double) * (size_t)n_edges);
    /* adjacency in edge order (conductionGraph::buildTreeTopology) */
    int* deg = (int*)calloc((size_t)n + 1, sizeof(int));
    for (long e = 0; e < n_edges; e++) { deg[ea[e] + 1]++; deg[eb[e] + 1]++; }
    for (long i = 0; i < n; i++) deg[i + 1] += deg[i];
    int* adj = (int*)malloc(sizeof(int) * (size_t)(2 * n_edges + 1));
    int* fill = (int*)calloc((size_t)n_edges + 1, sizeof(int));
    for (long e = 0; e < n_edges; e++) {
        adj[deg[ea[e]] + fill[ea[e]]++] = eb[e];
        adj[deg[eb[e]] + fill[eb[e]]++] = ea[e];
    }
    P->parent = (int*)malloc(sizeof(int) * (size_t)n);
    P->order = (int*)malloc(sizeof(int) * (size_t)n);
    P->rev = (int*)malloc(sizeof(int) * (size_t)n);
    unsigned char* seen = (unsigned char*)calloc((size_t)n, 1);
    for (long i = 0; i < n; i++) P->parent[i] = -1;
    long head = 0, tail = 0;
    P->order[tail++] = 0;
    seen[0] = 1;
    while (head < tail) {
        const int v = P->order[head++];
        for (int k = deg[v]; k < deg[v + 1]; k++) {
            const int w = adj[k];
            if (!seen[w]) { seen[w] = 1; P->parent[w] = v; P->order[tail++] = w; }
        }
    }
    free(deg); free(adj); free(fill); free(seen);
    if (tail != n) { oracle_purkinje_free(P); return NULL; }   /* not connected */
    for (long i = 0; i < n; i++) P->rev[i] = P->order[n - 1 - i];
    P->chi = chi;
    P->cm = cm;
    P->ionic = oracle_ionic_new(model, n, tissue, initial_dt, 0, ode, NULL, NULL);
    if (!P->ionic) { oracle_purkinje_free(P); return NULL; }
    P->vm = (double*)malloc(sizeof(double) * (size_t)n);
    P->iion = (double*)calloc((size_t)n, sizeof(double));
    P->app = (double*)calloc((size_t)n, sizeof(double));
    P->diag = (double*)malloc(sizeof(double) * (size_t)n);
    P->rhs = (double*)malloc(sizeof(double) * (size_t)n);
    P->pc = (double*)malloc(sizeof(double) * (size_t)n);
    P->cc = (double*)malloc(sizeof(double) * (size_t)n);
    P->clen = (double*)malloc(sizeof(double) * (size_t)n);
    /* ionicModel::vmRest: the model's state 0 in V */
    {
        const double u = P->ionic->y[0];
        const int map = P->ionic->m->vm_map;
        const double mv = map == 1 ? u * 100 - 80 : map == 2 ? u * 85.7 - 84.0 : u;
        const double v = map == 3 ? u : mv * 1e-3;
        for (long i = 0; i < n; i++) P->vm[i] = v;
    }
    P->root = root;
    P->root_start = root_start;
    P->root_dur = root_dur;
    P->root_int = root_int;
    P->n_term = n_term;
    P->term_node = (int*)malloc(sizeof(int) * (size_t)(n_term + 1));
    P->term_loc = (double*)malloc(sizeof(double) * 3 * (size_t)(n_term + 1));
    P->term_current = (double*)calloc((size_t)n_term + 1, sizeof(double));
    if (n_term) {
        memcpy(P->term_node, term_node, sizeof(int) * (size_t)n_term);
        memcpy(P->term_loc, term_loc, sizeof(double) * 3 * (size_t)n_term);
    }
    return P;
}

void oracle_purkinje_free(oracle_purkinje* P)
{
    if (!P) return;
    free(P->ea); free(P->eb); free(P->elen); free(P->econd);
    free(P->parent); free(P->order); free(P->rev);
    if (P->ionic) oracle_ionic_free(P->ionic);
    free(P->vm); free(P->iion); free(P->app);
    free(P->diag); free(P->rhs); free(P->pc); free(P->cc); free(P->clen);
    free(P->term_node); free(P->term_loc); free(P->term_current);
    free(P->term_cell); free(P->dep_cell); free(P->dep_term); free(P->sphere_vol);
    free(P->dep_value); free(P->tissue_vm_buf); free(P->net_vm_buf);
    free(P);
}

double* oracle_purkinje_vm(oracle_purkinje* P) { return P->vm; }
double* oracle_purkinje_iion(oracle_purkinje* P) { return P->iion; }
double* oracle_purkinje_terminal_current(oracle_purkinje* P) { return P->term_current; }
long oracle_purkinje_nodes(oracle_purkinje* P) { return P->n; }
const int* oracle_purkinje_order(oracle_purkinje* P) { return P->order; }
const int* oracle_purkinje_parent(oracle_purkinje* P) { return P->parent; }

/* Monodomain1DSolver::advance (monodomain1DSolver.C:36-190): half ionic step,
 * the applied current, the implicit cable step by Hines elimination over the
 * tree, the second half ionic step. */
int oracle_purkinje_advance(oracle_purkinje* P, double t0, double dt, int nthreads)
{
    const long n = P->n;
    if (oracle_ionic_solve(P->ionic, t0, dt / 2.0, P->vm, P->iion, nthreads) < 0) return -1;
    /* ConductionSystemDomain::assembleAppliedCurrent */
    for (long i = 0; i < n; i++) P->app[i] = 0.0;
    if (t0 >= P->root_start && t0 <= (P->root_start + P->root_dur)) P->app[P->root] += P->root_int;
    for (long i = 0; i < P->n_term; i++) P->app[P->term_node[i]] -= P->term_current[i];
    const double chiCm = P->chi * P->cm;
    for (long i = 0; i < n; i++) {
        P->diag[i] = 1.0;
        P->rhs[i] = 0.0;
        P->pc[i] = 0.0;
        P->cc[i] = 0.0;
        P->clen[i] = 0.0;
    }
    for (long e = 0; e < P->ne; e++) {
        P->clen[P->ea[e]] += 0.5 * P->elen[e];
        P->clen[P->eb[e]] += 0.5 * P->elen[e];
    }
    for (long i = 0; i < n; i++)
        if (P->clen[i] <= 1e-15) return -2;       /* zero control length */
    for (long e = 0; e < P->ne; e++) {
        const int a = P->ea[e], b = P->eb[e];
        const double edgeCoeff = P->econd[e] / P->elen[e];
        const double coeffA = dt * edgeCoeff / (chiCm * P->clen[a]);
        const double coeffB = dt * edgeCoeff / (chiCm * P->clen[b]);
        P->diag[a] += coeffA;
        P->diag[b] += coeffB;
        if (P->parent[a] == b) { P->pc[a] = -coeffA; P->cc[a] = -coeffB; }
        else if (P->parent[b] == a) { P->pc[b] = -coeffB; P->cc[b] = -coeffA; }
        else return -3;
    }
    for (long i = 0; i < n; i++)
        P->rhs[i] = P->vm[i] - dt * P->iion[i] + dt * P->app[i] / chiCm;
    for (long i = 0; i < n - 1; i++) {
        const int c = P->rev[i], p = P->parent[c];
        const double factor = P->cc[c] / P->diag[c];
        P->diag[p] -= factor * P->pc[c];
        P->rhs[p] -= factor * P->rhs[c];
    }
    const int root = P->order[0];
    P->vm[root] = P->rhs[root] / P->diag[root];
    for (long i = 1; i < n; i++) {
        const int c = P->order[i], p = P->parent[c];
        P->vm[c] = (P->rhs[c] - P->pc[c] * P->vm[p]) / P->diag[c];
    }
    if (oracle_ionic_solve(P->ionic, t0 + (dt / 2.0), dt / 2.0, P->vm, P->iion, nthreads) < 0)
        return -1;
    return 0;
}

/* PVJMapper (pvjMapper.C) on the tissue mesh: per terminal the cell holding
 * the location (the nearest centre here; the first on ties), the cells whose
 * centres lie within pvjRadius and their volume. */
int oracle_purkinje_couple(oracle_purkinje* P, const oracle_mesh* M, double r_pvj, double radius,
                           int mode)
{
    const long nt = P->n_term;
    P->coupled = 1;
    P->mode = mode;
    P->r_pvj = r_pvj;
    P->radius = radius;
    P->term_cell = (long*)malloc(sizeof(long) * (size_t)(nt + 1));
    P->sphere_vol = (double*)calloc((size_t)nt + 1, sizeof(double));
    P->dep_value = (double*)calloc((size_t)nt + 1, sizeof(double));
    P->tissue_vm_buf = (double*)calloc((size_t)nt + 1, sizeof(double));
    P->net_vm_buf = (double*)calloc((size_t)nt + 1, sizeof(double));
    long cap = 16, nd = 0;
    P->dep_cell = (long*)malloc(sizeof(long) * (size_t)cap);
    P->dep_term = (long*)malloc(sizeof(long) * (size_t)cap);
    for (long i = 0; i < nt; i++) {
        const double* x = P->term_loc + 3 * i;
        long best = -1;
        double bd = 1e300;
        for (long c = 0; c < M->n; c++) {
            const double* C = M->centres + 3 * c;
            const double d[3] = {C[0] - x[0], C[1] - x[1], C[2] - x[2]};
            const double dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (dist < bd) { bd = dist; best = c; }
        }
        if (best < 0) return -1;
        if (radius < cbrt(M->vol[best])) return -2;    /* pvjRadius below the cell size */
        P->term_cell[i] = best;
        for (long c = 0; c < M->n; c++) {
            const double* C = M->centres + 3 * c;
            const double d[3] = {C[0] - x[0], C[1] - x[1], C[2] - x[2]};
            if (sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) <= radius) {
                if (nd == cap) {
                    cap *= 2;
                    P->dep_cell = (long*)realloc(P->dep_cell, sizeof(long) * (size_t)cap);
                    P->dep_term = (long*)realloc(P->dep_term, sizeof(long) * (size_t)cap);
                }
                P->dep_cell[nd] = c;
                P->dep_term[nd] = i;
                nd++;
                P->sphere_vol[i] += M->vol[c];
            }
        }
        if (P->sphere_vol[i] <= 1e-15) {
            /* no centre within the radius: the nearest cell alone */
            if (nd == cap) {
                cap *= 2;
                P->dep_cell = (long*)realloc(P->dep_cell, sizeof(long) * (size_t)cap);
                P->dep_term = (long*)realloc(P->dep_term, sizeof(long) * (size_t)cap);
            }
            P->dep_cell[nd] = best;
            P->dep_term[nd] = i;
            nd++;
            P->sphere_vol[i] = M->vol[best];
        }
    }
    P->n_dep = nd;
    return 0;
}

/* ReactionDiffusionPvjCoupler::evaluateCoupling: I = (Vnet - Vtissue)/R_pvj
 * per terminal, and its volumetric source I/sphereVolume. */
static void pvj_evaluate(oracle_purkinje* P, const double* tissue_vm)
{
    for (long i = 0; i < P->n_term; i++) {
        P->tissue_vm_buf[i] = tissue_vm[P->term_cell[i]];
        P->net_vm_buf[i] = P->vm[P->term_node[i]];
        const double I = (P->net_vm_buf[i] - P->tissue_vm_buf[i]) / P->r_pvj;
        P->term_current[i] = I;
        P->dep_value[i] = I / P->sphere_vol[i];
    }
}

/* staggeredElectrophysicsAdvanceScheme::advance with one conduction network
 * coupled to the myocardium: prepareTimeStep (box stimulus, inside the tissue
 * step), prepareSecondaryCoupling, the network's advance,
 * preparePrimaryCoupling (deposit into the source), the myocardium's advance. */
int oracle_purkinje_coupled_step(oracle_purkinje* P, oracle_tissue* T, double dt, int nthreads)
{
    if (oracle_tissue_init_ionic(T, dt)) return -1;
    const double t0 = T->t;
    /* prepareSecondaryCoupling */
    pvj_evaluate(P, T->vm);
    if (P->mode == 0)
        for (long i = 0; i < P->n_term; i++) P->term_current[i] = 0.0;
    if (oracle_purkinje_advance(P, t0, dt, nthreads) < 0) return -1;
    /* preparePrimaryCoupling: the new network Vm, deposited with the tissue's
     * stimulus; the network keeps these currents */
    pvj_evaluate(P, T->vm);
    T->n_dep = P->n_dep;
    T->dep_cell = P->dep_cell;
    T->dep_term = P->dep_term;
    T->dep_value = P->dep_value;
    const int rc = oracle_tissue_step(T, dt, nthreads);
    T->dep_value = NULL;
    return rc;
}
