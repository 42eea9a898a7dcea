/* Generated by cardiacfoam_gb300.cellml2cuda from src/ionicModels/AlievPanfilov/AlievPanfilov_1996.H.
 * Oracle form: reference calling convention and evaluation order, pow kept
 * as written.  Test infrastructure only; the product uses the CUDA form. */
#ifndef ORACLE_MODEL_ALIEVPANFILOV_H
#define ORACLE_MODEL_ALIEVPANFILOV_H
#include "../oracle_common.h"

enum { ALIEVPANFILOV_NS = 2, ALIEVPANFILOV_NA = 3, ALIEVPANFILOV_NC = 8 };
enum { ALIEVPANFILOV_S_u, ALIEVPANFILOV_S_recovery_r };
enum { ALIEVPANFILOV_A_AV_eps, ALIEVPANFILOV_A_Istim, ALIEVPANFILOV_A_Iion_cm };
enum { ALIEVPANFILOV_C_AC_Vp, ALIEVPANFILOV_C_AC_Vr, ALIEVPANFILOV_C_AC_Vth, ALIEVPANFILOV_C_AC_epsilon, ALIEVPANFILOV_C_AC_k, ALIEVPANFILOV_C_AC_mu1, ALIEVPANFILOV_C_AC_mu2, ALIEVPANFILOV_C_AC_a };
static const char* const ALIEVPANFILOV_STATE_NAMES[] = { "u", "recovery_r" };

static void alievpanfilov_init(double* CONSTANTS, double* STATES, int tissueFlag, const double* scale)
{
    (void)tissueFlag; (void)scale;
    CONSTANTS[ALIEVPANFILOV_C_AC_Vp] = 20.0;
    CONSTANTS[ALIEVPANFILOV_C_AC_Vr] = (-80.0);
    CONSTANTS[ALIEVPANFILOV_C_AC_Vth] = (-70.0);
    CONSTANTS[ALIEVPANFILOV_C_AC_epsilon] = 0.01;
    CONSTANTS[ALIEVPANFILOV_C_AC_k] = 8.0;
    CONSTANTS[ALIEVPANFILOV_C_AC_mu1] = 0.2;
    CONSTANTS[ALIEVPANFILOV_C_AC_mu2] = 0.3;
    CONSTANTS[ALIEVPANFILOV_C_AC_a] = ((CONSTANTS[ALIEVPANFILOV_C_AC_Vth] - CONSTANTS[ALIEVPANFILOV_C_AC_Vr]) / (CONSTANTS[ALIEVPANFILOV_C_AC_Vp] - CONSTANTS[ALIEVPANFILOV_C_AC_Vr]));
    STATES[ALIEVPANFILOV_S_u] = 0.05;
    STATES[ALIEVPANFILOV_S_recovery_r] = 0.0;
}

/* constants alievpanfilov_init leaves unset; NULL-equivalent when none */
static void alievpanfilov_supplement(double* CONSTANTS)
{
    (void)CONSTANTS;
}

static void alievpanfilov_rates(double VOI, const double* CONSTANTS, double* RATES, const double* STATES, double* ALGEBRAIC, int tissueFlag, int solveVm, const oracle_stimulus* stim)
{
    (void)tissueFlag; (void)solveVm; (void)stim;
    ALGEBRAIC[ALIEVPANFILOV_A_AV_eps] = (CONSTANTS[ALIEVPANFILOV_C_AC_epsilon] + ((CONSTANTS[ALIEVPANFILOV_C_AC_mu1] * STATES[ALIEVPANFILOV_S_recovery_r]) / (CONSTANTS[ALIEVPANFILOV_C_AC_mu2] + STATES[ALIEVPANFILOV_S_u])));
    RATES[ALIEVPANFILOV_S_recovery_r] = (ALGEBRAIC[ALIEVPANFILOV_A_AV_eps] * ((-STATES[ALIEVPANFILOV_S_recovery_r]) - ((CONSTANTS[ALIEVPANFILOV_C_AC_k] * STATES[ALIEVPANFILOV_S_u]) * (STATES[ALIEVPANFILOV_S_u] - (CONSTANTS[ALIEVPANFILOV_C_AC_a] + 1.0)))));
    ALGEBRAIC[ALIEVPANFILOV_A_Iion_cm] = ((((CONSTANTS[ALIEVPANFILOV_C_AC_k] * STATES[ALIEVPANFILOV_S_u]) * (STATES[ALIEVPANFILOV_S_u] - CONSTANTS[ALIEVPANFILOV_C_AC_a])) * (STATES[ALIEVPANFILOV_S_u] - 1.0)) + (STATES[ALIEVPANFILOV_S_recovery_r] * STATES[ALIEVPANFILOV_S_u]));
    ALGEBRAIC[ALIEVPANFILOV_A_Istim] = oracle_stimulus_current(VOI, stim);
    if (solveVm) {
        RATES[ALIEVPANFILOV_S_u] = ((-ALGEBRAIC[ALIEVPANFILOV_A_Iion_cm]) - ALGEBRAIC[ALIEVPANFILOV_A_Istim]);
    }
}

static void alievpanfilov_variables(double VOI, const double* CONSTANTS, double* RATES, const double* STATES, double* ALGEBRAIC, int tissueFlag, int solveVm, const oracle_stimulus* stim)
{
    (void)tissueFlag; (void)solveVm; (void)stim;
    ALGEBRAIC[ALIEVPANFILOV_A_AV_eps] = (CONSTANTS[ALIEVPANFILOV_C_AC_epsilon] + ((CONSTANTS[ALIEVPANFILOV_C_AC_mu1] * STATES[ALIEVPANFILOV_S_recovery_r]) / (CONSTANTS[ALIEVPANFILOV_C_AC_mu2] + STATES[ALIEVPANFILOV_S_u])));
    RATES[ALIEVPANFILOV_S_recovery_r] = (ALGEBRAIC[ALIEVPANFILOV_A_AV_eps] * ((-STATES[ALIEVPANFILOV_S_recovery_r]) - ((CONSTANTS[ALIEVPANFILOV_C_AC_k] * STATES[ALIEVPANFILOV_S_u]) * (STATES[ALIEVPANFILOV_S_u] - (CONSTANTS[ALIEVPANFILOV_C_AC_a] + 1.0)))));
    ALGEBRAIC[ALIEVPANFILOV_A_Iion_cm] = ((((CONSTANTS[ALIEVPANFILOV_C_AC_k] * STATES[ALIEVPANFILOV_S_u]) * (STATES[ALIEVPANFILOV_S_u] - CONSTANTS[ALIEVPANFILOV_C_AC_a])) * (STATES[ALIEVPANFILOV_S_u] - 1.0)) + (STATES[ALIEVPANFILOV_S_recovery_r] * STATES[ALIEVPANFILOV_S_u]));
    ALGEBRAIC[ALIEVPANFILOV_A_Istim] = oracle_stimulus_current(VOI, stim);
    if (solveVm) {
        RATES[ALIEVPANFILOV_S_u] = ((-ALGEBRAIC[ALIEVPANFILOV_A_Iion_cm]) - ALGEBRAIC[ALIEVPANFILOV_A_Istim]);
    }
}

#define ALIEVPANFILOV_IION_INDEX ALIEVPANFILOV_A_Iion_cm
#define ALIEVPANFILOV_IION_SCALE 100.0
#define ALIEVPANFILOV_TIME_SCALE 12.9
#endif
