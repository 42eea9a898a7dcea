/* Generated by cardiacfoam_gb300.cellml2cuda from src/ionicModels/BuenoOrovio/BuenoOrovio_2008.H.
 * Oracle form: reference calling convention and evaluation order, pow kept
 * as written.  Test infrastructure only; the product uses the CUDA form. */
#ifndef ORACLE_MODEL_BUENOOROVIO_H
#define ORACLE_MODEL_BUENOOROVIO_H
#include "../oracle_common.h"

enum { BUENOOROVIO_NS = 4, BUENOOROVIO_NA = 12, BUENOOROVIO_NC = 28 };
enum { BUENOOROVIO_S_u, BUENOOROVIO_S_v, BUENOOROVIO_S_w, BUENOOROVIO_S_s };
enum { BUENOOROVIO_A_Jfi, BUENOOROVIO_A_Jso, BUENOOROVIO_A_Jsi, BUENOOROVIO_A_Jion, BUENOOROVIO_A_Istim, BUENOOROVIO_A_tauSo, BUENOOROVIO_A_tauO, BUENOOROVIO_A_tauVMinus, BUENOOROVIO_A_tauWMinus, BUENOOROVIO_A_tauS, BUENOOROVIO_A_vInfty, BUENOOROVIO_A_wInfty };
enum { BUENOOROVIO_C_uO, BUENOOROVIO_C_uU, BUENOOROVIO_C_thetaV, BUENOOROVIO_C_thetaW, BUENOOROVIO_C_thetaVMinus, BUENOOROVIO_C_thetaO, BUENOOROVIO_C_tauV1Minus, BUENOOROVIO_C_tauV2Minus, BUENOOROVIO_C_tauVPlus, BUENOOROVIO_C_tauW1Minus, BUENOOROVIO_C_tauW2Minus, BUENOOROVIO_C_kWMinus, BUENOOROVIO_C_uWMinus, BUENOOROVIO_C_tauWPlus, BUENOOROVIO_C_tauFi, BUENOOROVIO_C_tauO1, BUENOOROVIO_C_tauO2, BUENOOROVIO_C_tauSo1, BUENOOROVIO_C_tauSo2, BUENOOROVIO_C_kSo, BUENOOROVIO_C_uSo, BUENOOROVIO_C_tauS1, BUENOOROVIO_C_tauS2, BUENOOROVIO_C_kS, BUENOOROVIO_C_uS, BUENOOROVIO_C_tauSi, BUENOOROVIO_C_tauWInfty, BUENOOROVIO_C_wInftyStar };
static const char* const BUENOOROVIO_STATE_NAMES[] = { "u", "v", "w", "s" };

static void buenoorovio_init(double* CONSTANTS, double* STATES, int tissueFlag, const double* scale)
{
    (void)tissueFlag; (void)scale;
    CONSTANTS[BUENOOROVIO_C_uO] = 0;
    CONSTANTS[BUENOOROVIO_C_uU] = ((tissueFlag == 1) ? 1.55 : ((tissueFlag == 2) ? 1.61 : 1.56));
    CONSTANTS[BUENOOROVIO_C_thetaV] = 0.3;
    CONSTANTS[BUENOOROVIO_C_thetaW] = 0.13;
    CONSTANTS[BUENOOROVIO_C_thetaVMinus] = ((tissueFlag == 1) ? 0.006 : ((tissueFlag == 2) ? 0.1 : 0.2));
    CONSTANTS[BUENOOROVIO_C_thetaO] = ((tissueFlag == 2) ? 0.005 : 0.006);
    CONSTANTS[BUENOOROVIO_C_tauV1Minus] = ((tissueFlag == 1) ? 60 : ((tissueFlag == 2) ? 80 : 75));
    CONSTANTS[BUENOOROVIO_C_tauV2Minus] = ((tissueFlag == 1) ? 1150 : ((tissueFlag == 2) ? 1.4506 : 10));
    CONSTANTS[BUENOOROVIO_C_tauVPlus] = 1.4506;
    CONSTANTS[BUENOOROVIO_C_tauW1Minus] = ((tissueFlag == 1) ? 60 : ((tissueFlag == 2) ? 70 : 6));
    CONSTANTS[BUENOOROVIO_C_tauW2Minus] = ((tissueFlag == 1) ? 15 : ((tissueFlag == 2) ? 8 : 140));
    CONSTANTS[BUENOOROVIO_C_kWMinus] = ((tissueFlag == 1) ? 65 : 200);
    CONSTANTS[BUENOOROVIO_C_uWMinus] = ((tissueFlag == 1) ? 0.03 : 0.016);
    CONSTANTS[BUENOOROVIO_C_tauWPlus] = ((tissueFlag == 1) ? 200 : 280);
    CONSTANTS[BUENOOROVIO_C_tauFi] = ((tissueFlag == 1) ? 0.11 : ((tissueFlag == 2) ? 0.078 : 0.1));
    CONSTANTS[BUENOOROVIO_C_tauO1] = ((tissueFlag == 1) ? 400 : ((tissueFlag == 2) ? 410 : 470));
    CONSTANTS[BUENOOROVIO_C_tauO2] = ((tissueFlag == 2) ? 7 : 6);
    CONSTANTS[BUENOOROVIO_C_tauSo1] = ((tissueFlag == 1) ? 30.0181 : ((tissueFlag == 2) ? 91 : 40));
    CONSTANTS[BUENOOROVIO_C_tauSo2] = ((tissueFlag == 1) ? 0.9957 : ((tissueFlag == 2) ? 0.8 : 1.2));
    CONSTANTS[BUENOOROVIO_C_kSo] = ((tissueFlag == 1) ? 2.0458 : ((tissueFlag == 2) ? 2.1 : 2));
    CONSTANTS[BUENOOROVIO_C_uSo] = ((tissueFlag == 2) ? 0.6 : 0.65);
    CONSTANTS[BUENOOROVIO_C_tauS1] = 2.7342;
    CONSTANTS[BUENOOROVIO_C_tauS2] = ((tissueFlag == 1) ? 16 : ((tissueFlag == 2) ? 4 : 2));
    CONSTANTS[BUENOOROVIO_C_kS] = 2.0994;
    CONSTANTS[BUENOOROVIO_C_uS] = 0.9087;
    CONSTANTS[BUENOOROVIO_C_tauSi] = ((tissueFlag == 1) ? 1.8875 : ((tissueFlag == 2) ? 3.3849 : 2.9013));
    CONSTANTS[BUENOOROVIO_C_tauWInfty] = ((tissueFlag == 1) ? 0.07 : ((tissueFlag == 2) ? 0.01 : 0.0273));
    CONSTANTS[BUENOOROVIO_C_wInftyStar] = ((tissueFlag == 1) ? 0.94 : ((tissueFlag == 2) ? 0.5 : 0.78));
    STATES[BUENOOROVIO_S_u] = 0;
    STATES[BUENOOROVIO_S_v] = 1.0;
    STATES[BUENOOROVIO_S_w] = 1.0;
    STATES[BUENOOROVIO_S_s] = 0.0;
}

/* constants buenoorovio_init leaves unset; NULL-equivalent when none */
static void buenoorovio_supplement(double* CONSTANTS)
{
    (void)CONSTANTS;
}

static void buenoorovio_rates(double VOI, const double* CONSTANTS, double* RATES, const double* STATES, double* ALGEBRAIC, int tissueFlag, int solveVm, const oracle_stimulus* stim)
{
    (void)tissueFlag; (void)solveVm; (void)stim;
    ALGEBRAIC[BUENOOROVIO_A_tauSo] = (CONSTANTS[BUENOOROVIO_C_tauSo1] + (((CONSTANTS[BUENOOROVIO_C_tauSo2] - CONSTANTS[BUENOOROVIO_C_tauSo1]) * (1.0 + tanh((CONSTANTS[BUENOOROVIO_C_kSo] * (STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_uSo]))))) / 2.0));
    ALGEBRAIC[BUENOOROVIO_A_tauO] = (((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaO]))) * CONSTANTS[BUENOOROVIO_C_tauO1]) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaO])) * CONSTANTS[BUENOOROVIO_C_tauO2]));
    ALGEBRAIC[BUENOOROVIO_A_Jfi] = (((((-STATES[BUENOOROVIO_S_v]) * oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaV]))) * (STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaV])) * (CONSTANTS[BUENOOROVIO_C_uU] - STATES[BUENOOROVIO_S_u])) / CONSTANTS[BUENOOROVIO_C_tauFi]);
    ALGEBRAIC[BUENOOROVIO_A_Jso] = ((((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_uO]) * (1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW])))) / ALGEBRAIC[BUENOOROVIO_A_tauO]) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW])) / ALGEBRAIC[BUENOOROVIO_A_tauSo]));
    ALGEBRAIC[BUENOOROVIO_A_Jsi] = ((((-oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW]))) * STATES[BUENOOROVIO_S_w]) * STATES[BUENOOROVIO_S_s]) / CONSTANTS[BUENOOROVIO_C_tauSi]);
    ALGEBRAIC[BUENOOROVIO_A_Jion] = ((ALGEBRAIC[BUENOOROVIO_A_Jfi] + ALGEBRAIC[BUENOOROVIO_A_Jso]) + ALGEBRAIC[BUENOOROVIO_A_Jsi]);
    ALGEBRAIC[BUENOOROVIO_A_tauVMinus] = (((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaVMinus]))) * CONSTANTS[BUENOOROVIO_C_tauV1Minus]) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaVMinus])) * CONSTANTS[BUENOOROVIO_C_tauV2Minus]));
    ALGEBRAIC[BUENOOROVIO_A_tauWMinus] = (CONSTANTS[BUENOOROVIO_C_tauW1Minus] + (((CONSTANTS[BUENOOROVIO_C_tauW2Minus] - CONSTANTS[BUENOOROVIO_C_tauW1Minus]) * (1.0 + tanh((CONSTANTS[BUENOOROVIO_C_kWMinus] * (STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_uWMinus]))))) / 2.0));
    ALGEBRAIC[BUENOOROVIO_A_tauS] = (((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW]))) * CONSTANTS[BUENOOROVIO_C_tauS1]) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW])) * CONSTANTS[BUENOOROVIO_C_tauS2]));
    ALGEBRAIC[BUENOOROVIO_A_vInfty] = oracle_heaviside((CONSTANTS[BUENOOROVIO_C_thetaVMinus] - STATES[BUENOOROVIO_S_u]));
    ALGEBRAIC[BUENOOROVIO_A_wInfty] = (((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaO]))) * (1.0 - (STATES[BUENOOROVIO_S_u] / CONSTANTS[BUENOOROVIO_C_tauWInfty]))) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaO])) * CONSTANTS[BUENOOROVIO_C_wInftyStar]));
    RATES[BUENOOROVIO_S_v] = ((((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaV]))) * (ALGEBRAIC[BUENOOROVIO_A_vInfty] - STATES[BUENOOROVIO_S_v])) / ALGEBRAIC[BUENOOROVIO_A_tauVMinus]) - ((oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaV])) * STATES[BUENOOROVIO_S_v]) / CONSTANTS[BUENOOROVIO_C_tauVPlus]));
    RATES[BUENOOROVIO_S_w] = ((((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW]))) * (ALGEBRAIC[BUENOOROVIO_A_wInfty] - STATES[BUENOOROVIO_S_w])) / ALGEBRAIC[BUENOOROVIO_A_tauWMinus]) - ((oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW])) * STATES[BUENOOROVIO_S_w]) / CONSTANTS[BUENOOROVIO_C_tauWPlus]));
    RATES[BUENOOROVIO_S_s] = ((((1.0 + tanh((CONSTANTS[BUENOOROVIO_C_kS] * (STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_uS])))) / 2.0) - STATES[BUENOOROVIO_S_s]) / ALGEBRAIC[BUENOOROVIO_A_tauS]);
    ALGEBRAIC[BUENOOROVIO_A_Istim] = oracle_stimulus_current(VOI, stim);
    if (solveVm) {
        RATES[BUENOOROVIO_S_u] = ((-ALGEBRAIC[BUENOOROVIO_A_Jion]) - ALGEBRAIC[BUENOOROVIO_A_Istim]);
    }
}

static void buenoorovio_variables(double VOI, const double* CONSTANTS, double* RATES, const double* STATES, double* ALGEBRAIC, int tissueFlag, int solveVm, const oracle_stimulus* stim)
{
    (void)tissueFlag; (void)solveVm; (void)stim;
    ALGEBRAIC[BUENOOROVIO_A_tauSo] = (CONSTANTS[BUENOOROVIO_C_tauSo1] + (((CONSTANTS[BUENOOROVIO_C_tauSo2] - CONSTANTS[BUENOOROVIO_C_tauSo1]) * (1.0 + tanh((CONSTANTS[BUENOOROVIO_C_kSo] * (STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_uSo]))))) / 2.0));
    ALGEBRAIC[BUENOOROVIO_A_tauO] = (((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaO]))) * CONSTANTS[BUENOOROVIO_C_tauO1]) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaO])) * CONSTANTS[BUENOOROVIO_C_tauO2]));
    ALGEBRAIC[BUENOOROVIO_A_Jfi] = (((((-STATES[BUENOOROVIO_S_v]) * oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaV]))) * (STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaV])) * (CONSTANTS[BUENOOROVIO_C_uU] - STATES[BUENOOROVIO_S_u])) / CONSTANTS[BUENOOROVIO_C_tauFi]);
    ALGEBRAIC[BUENOOROVIO_A_Jso] = ((((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_uO]) * (1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW])))) / ALGEBRAIC[BUENOOROVIO_A_tauO]) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW])) / ALGEBRAIC[BUENOOROVIO_A_tauSo]));
    ALGEBRAIC[BUENOOROVIO_A_Jsi] = ((((-oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW]))) * STATES[BUENOOROVIO_S_w]) * STATES[BUENOOROVIO_S_s]) / CONSTANTS[BUENOOROVIO_C_tauSi]);
    ALGEBRAIC[BUENOOROVIO_A_Jion] = ((ALGEBRAIC[BUENOOROVIO_A_Jfi] + ALGEBRAIC[BUENOOROVIO_A_Jso]) + ALGEBRAIC[BUENOOROVIO_A_Jsi]);
    ALGEBRAIC[BUENOOROVIO_A_tauVMinus] = (((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaVMinus]))) * CONSTANTS[BUENOOROVIO_C_tauV1Minus]) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaVMinus])) * CONSTANTS[BUENOOROVIO_C_tauV2Minus]));
    ALGEBRAIC[BUENOOROVIO_A_tauWMinus] = (CONSTANTS[BUENOOROVIO_C_tauW1Minus] + (((CONSTANTS[BUENOOROVIO_C_tauW2Minus] - CONSTANTS[BUENOOROVIO_C_tauW1Minus]) * (1.0 + tanh((CONSTANTS[BUENOOROVIO_C_kWMinus] * (STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_uWMinus]))))) / 2.0));
    ALGEBRAIC[BUENOOROVIO_A_tauS] = (((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW]))) * CONSTANTS[BUENOOROVIO_C_tauS1]) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW])) * CONSTANTS[BUENOOROVIO_C_tauS2]));
    ALGEBRAIC[BUENOOROVIO_A_vInfty] = oracle_heaviside((CONSTANTS[BUENOOROVIO_C_thetaVMinus] - STATES[BUENOOROVIO_S_u]));
    ALGEBRAIC[BUENOOROVIO_A_wInfty] = (((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaO]))) * (1.0 - (STATES[BUENOOROVIO_S_u] / CONSTANTS[BUENOOROVIO_C_tauWInfty]))) + (oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaO])) * CONSTANTS[BUENOOROVIO_C_wInftyStar]));
    RATES[BUENOOROVIO_S_v] = ((((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaV]))) * (ALGEBRAIC[BUENOOROVIO_A_vInfty] - STATES[BUENOOROVIO_S_v])) / ALGEBRAIC[BUENOOROVIO_A_tauVMinus]) - ((oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaV])) * STATES[BUENOOROVIO_S_v]) / CONSTANTS[BUENOOROVIO_C_tauVPlus]));
    RATES[BUENOOROVIO_S_w] = ((((1.0 - oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW]))) * (ALGEBRAIC[BUENOOROVIO_A_wInfty] - STATES[BUENOOROVIO_S_w])) / ALGEBRAIC[BUENOOROVIO_A_tauWMinus]) - ((oracle_heaviside((STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_thetaW])) * STATES[BUENOOROVIO_S_w]) / CONSTANTS[BUENOOROVIO_C_tauWPlus]));
    RATES[BUENOOROVIO_S_s] = ((((1.0 + tanh((CONSTANTS[BUENOOROVIO_C_kS] * (STATES[BUENOOROVIO_S_u] - CONSTANTS[BUENOOROVIO_C_uS])))) / 2.0) - STATES[BUENOOROVIO_S_s]) / ALGEBRAIC[BUENOOROVIO_A_tauS]);
    ALGEBRAIC[BUENOOROVIO_A_Istim] = oracle_stimulus_current(VOI, stim);
    if (solveVm) {
        RATES[BUENOOROVIO_S_u] = ((-ALGEBRAIC[BUENOOROVIO_A_Jion]) - ALGEBRAIC[BUENOOROVIO_A_Istim]);
    }
}

#define BUENOOROVIO_IION_INDEX BUENOOROVIO_A_Jion
#define BUENOOROVIO_IION_SCALE 85.7
#define BUENOOROVIO_TIME_SCALE 1.0
#endif
