// Generated by cardiacfoam_gb300.cellml2cuda from src/ionicModels/BuenoOrovio/BuenoOrovio_2008.H.
// The equations are the published cell model as cellML2foam wrote them;
// regenerate with `python -m cardiacfoam_gb300.cellml2cuda` instead of editing.
#pragma once
#include "../ionic_common.cuh"

namespace cfg { namespace buenoorovio {

constexpr int NS = 4;
constexpr int NC = 28;
constexpr int NA = 12;
enum State { S_u, S_v, S_w, S_s };
enum Constant { C_uO, C_uU, C_thetaV, C_thetaW, C_thetaVMinus, C_thetaO, C_tauV1Minus, C_tauV2Minus, C_tauVPlus, C_tauW1Minus, C_tauW2Minus, C_kWMinus, C_uWMinus, C_tauWPlus, C_tauFi, C_tauO1, C_tauO2, C_tauSo1, C_tauSo2, C_kSo, C_uSo, C_tauS1, C_tauS2, C_kS, C_uS, C_tauSi, C_tauWInfty, C_wInftyStar };
// states kept in double in the mixed form (bit i = state i)
constexpr unsigned long long WIDE_MASK = 0xfull;
constexpr double IION_SCALE = 85.7;
constexpr double TIME_SCALE = 1.0;
constexpr int VM_MAP = CFG_VM_BUENO;
constexpr int N_TISSUES = 3;
static const int TISSUES[] = {3, 2, 1, 0};
using TissueSet = TissueList<3, 2, 1>;
static const char* const STATE_NAMES[NS] = {"u", "v", "w", "s"};
CFG_HD inline bool tissue_supported(int t) { return t == 3 || t == 2 || t == 1; }

// per-cell conductance scales: index into the scale vector, or -1
constexpr int SCALE_GNa = -1;
constexpr int SCALE_GCaL = -1;
constexpr int SCALE_GKr = -1;
constexpr int SCALE_GKs = -1;
constexpr int SCALE_GK1 = -1;
constexpr int SCALE_Gto = -1;

// Constants that depend on the per-cell conductance scales and that the
// right-hand side reads: the scaled conductances and every constant
// initConsts derives from them.  sd_slot(i) is constant i's index in a
// cell's vector of them, or -1 (then the constant is the tissue's).
constexpr int NSD = 0;
CFG_HD constexpr int sd_const(int k)
{
    switch (k) {
    default: return -1;
    }
}
CFG_HD constexpr int sd_slot(int i)
{
    switch (i) {
    default: return -1;
    }
}
// intracellular calcium state (peak Ca of a beat), or -1
constexpr int CA_STATE = -1;

// Constants and initial states (initConsts).  `scale` may be null;
// otherwise scale[SCALE_x] multiplies the named conductance right after
// it is assigned, before constants derived from it are computed.
CFG_HD __forceinline__ void init_consts(double* C, double* y, int tissue, const double* scale)
{
    (void)tissue; (void)scale;
    C[C_uO] = 0;
    C[C_uU] = ((tissue == 1) ? 1.55 : ((tissue == 2) ? 1.61 : 1.56));
    C[C_thetaV] = 0.3;
    C[C_thetaW] = 0.13;
    C[C_thetaVMinus] = ((tissue == 1) ? 0.006 : ((tissue == 2) ? 0.1 : 0.2));
    C[C_thetaO] = ((tissue == 2) ? 0.005 : 0.006);
    C[C_tauV1Minus] = ((tissue == 1) ? 60 : ((tissue == 2) ? 80 : 75));
    C[C_tauV2Minus] = ((tissue == 1) ? 1150 : ((tissue == 2) ? 1.4506 : 10));
    C[C_tauVPlus] = 1.4506;
    C[C_tauW1Minus] = ((tissue == 1) ? 60 : ((tissue == 2) ? 70 : 6));
    C[C_tauW2Minus] = ((tissue == 1) ? 15 : ((tissue == 2) ? 8 : 140));
    C[C_kWMinus] = ((tissue == 1) ? 65 : 200);
    C[C_uWMinus] = ((tissue == 1) ? 0.03 : 0.016);
    C[C_tauWPlus] = ((tissue == 1) ? 200 : 280);
    C[C_tauFi] = ((tissue == 1) ? 0.11 : ((tissue == 2) ? 0.078 : 0.1));
    C[C_tauO1] = ((tissue == 1) ? 400 : ((tissue == 2) ? 410 : 470));
    C[C_tauO2] = ((tissue == 2) ? 7 : 6);
    C[C_tauSo1] = ((tissue == 1) ? 30.0181 : ((tissue == 2) ? 91 : 40));
    C[C_tauSo2] = ((tissue == 1) ? 0.9957 : ((tissue == 2) ? 0.8 : 1.2));
    C[C_kSo] = ((tissue == 1) ? 2.0458 : ((tissue == 2) ? 2.1 : 2));
    C[C_uSo] = ((tissue == 2) ? 0.6 : 0.65);
    C[C_tauS1] = 2.7342;
    C[C_tauS2] = ((tissue == 1) ? 16 : ((tissue == 2) ? 4 : 2));
    C[C_kS] = 2.0994;
    C[C_uS] = 0.9087;
    C[C_tauSi] = ((tissue == 1) ? 1.8875 : ((tissue == 2) ? 3.3849 : 2.9013));
    C[C_tauWInfty] = ((tissue == 1) ? 0.07 : ((tissue == 2) ? 0.01 : 0.0273));
    C[C_wInftyStar] = ((tissue == 1) ? 0.94 : ((tissue == 2) ? 0.5 : 0.78));
    y[S_u] = 0;
    y[S_v] = 1.0;
    y[S_w] = 1.0;
    y[S_s] = 0.0;
}

// initConsts evaluated per tissue flag (IEEE double, the header's order of
// operations): cval<T>(i) is constant i for tissue T.  Kernels for one uniform
// tissue without per-cell scales read constants from here, so the compiler
// folds them into the instructions.
template <int T> CFG_HD constexpr double cval(int i);
template <> CFG_HD constexpr double cval<3>(int i)
{
    switch (i) {
    case 0: return 0.0;
    case 1: return 1.56;
    case 2: return 0.3;
    case 3: return 0.13;
    case 4: return 0.2;
    case 5: return 0.006;
    case 6: return 75.0;
    case 7: return 10.0;
    case 8: return 1.4506;
    case 9: return 6.0;
    case 10: return 140.0;
    case 11: return 200.0;
    case 12: return 0.016;
    case 13: return 280.0;
    case 14: return 0.1;
    case 15: return 470.0;
    case 16: return 6.0;
    case 17: return 40.0;
    case 18: return 1.2;
    case 19: return 2.0;
    case 20: return 0.65;
    case 21: return 2.7342;
    case 22: return 2.0;
    case 23: return 2.0994;
    case 24: return 0.9087;
    case 25: return 2.9013;
    case 26: return 0.0273;
    case 27: return 0.78;
    default: return 0.0;
    }
}
template <> CFG_HD constexpr double cval<2>(int i)
{
    switch (i) {
    case 0: return 0.0;
    case 1: return 1.61;
    case 2: return 0.3;
    case 3: return 0.13;
    case 4: return 0.1;
    case 5: return 0.005;
    case 6: return 80.0;
    case 7: return 1.4506;
    case 8: return 1.4506;
    case 9: return 70.0;
    case 10: return 8.0;
    case 11: return 200.0;
    case 12: return 0.016;
    case 13: return 280.0;
    case 14: return 0.078;
    case 15: return 410.0;
    case 16: return 7.0;
    case 17: return 91.0;
    case 18: return 0.8;
    case 19: return 2.1;
    case 20: return 0.6;
    case 21: return 2.7342;
    case 22: return 4.0;
    case 23: return 2.0994;
    case 24: return 0.9087;
    case 25: return 3.3849;
    case 26: return 0.01;
    case 27: return 0.5;
    default: return 0.0;
    }
}
template <> CFG_HD constexpr double cval<1>(int i)
{
    switch (i) {
    case 0: return 0.0;
    case 1: return 1.55;
    case 2: return 0.3;
    case 3: return 0.13;
    case 4: return 0.006;
    case 5: return 0.006;
    case 6: return 60.0;
    case 7: return 1150.0;
    case 8: return 1.4506;
    case 9: return 60.0;
    case 10: return 15.0;
    case 11: return 65.0;
    case 12: return 0.03;
    case 13: return 200.0;
    case 14: return 0.11;
    case 15: return 400.0;
    case 16: return 6.0;
    case 17: return 30.0181;
    case 18: return 0.9957;
    case 19: return 2.0458;
    case 20: return 0.65;
    case 21: return 2.7342;
    case 22: return 16.0;
    case 23: return 2.0994;
    case 24: return 0.9087;
    case 25: return 1.8875;
    case 26: return 0.07;
    case 27: return 0.94;
    default: return 0.0;
    }
}

// Right-hand side as used by derivatives(): dydt for every state that the
// reference assigns (RATES of V only when SOLVE_VM).  Returns Iion.
// Y(i) reads state i as R (each state once, before any dydt store),
// K(i) reads constant i as R.
template <class R, bool SOLVE_VM, class YS, class KS>
__device__ __forceinline__ R rhs(double t, const YS& Y, const KS& K, R* dydt, int tissue, const CfgStimulus& stim)
{
    (void)tissue; (void)stim; (void)t;
    const R y_u = Y(S_u);
    const R y_v = Y(S_v);
    const R y_w = Y(S_w);
    const R y_s = Y(S_s);
    R a_tauSo = (K(C_tauSo1) + (((K(C_tauSo2) - K(C_tauSo1)) * (R(1.0) + cfg_tanh((K(C_kSo) * (y_u - K(C_uSo)))))) / R(2.0)));
    R a_tauO = (((R(1.0) - (((y_u - K(C_thetaO))) > R(0) ? 1 : 0)) * K(C_tauO1)) + ((((y_u - K(C_thetaO))) > R(0) ? 1 : 0) * K(C_tauO2)));
    R a_Jfi = (((((-y_v) * (((y_u - K(C_thetaV))) > R(0) ? 1 : 0)) * (y_u - K(C_thetaV))) * (K(C_uU) - y_u)) / K(C_tauFi));
    R a_Jso = ((((y_u - K(C_uO)) * (R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0))) / a_tauO) + ((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) / a_tauSo));
    R a_Jsi = ((((-(((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * y_w) * y_s) / K(C_tauSi));
    R a_Jion = ((a_Jfi + a_Jso) + a_Jsi);
    R a_tauVMinus = (((R(1.0) - (((y_u - K(C_thetaVMinus))) > R(0) ? 1 : 0)) * K(C_tauV1Minus)) + ((((y_u - K(C_thetaVMinus))) > R(0) ? 1 : 0) * K(C_tauV2Minus)));
    R a_tauWMinus = (K(C_tauW1Minus) + (((K(C_tauW2Minus) - K(C_tauW1Minus)) * (R(1.0) + cfg_tanh((K(C_kWMinus) * (y_u - K(C_uWMinus)))))) / R(2.0)));
    R a_tauS = (((R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * K(C_tauS1)) + ((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) * K(C_tauS2)));
    R a_vInfty = (((K(C_thetaVMinus) - y_u)) > R(0) ? 1 : 0);
    R a_wInfty = (((R(1.0) - (((y_u - K(C_thetaO))) > R(0) ? 1 : 0)) * (R(1.0) - (y_u / K(C_tauWInfty)))) + ((((y_u - K(C_thetaO))) > R(0) ? 1 : 0) * K(C_wInftyStar)));
    dydt[S_v] = ((((R(1.0) - (((y_u - K(C_thetaV))) > R(0) ? 1 : 0)) * (a_vInfty - y_v)) / a_tauVMinus) - (((((y_u - K(C_thetaV))) > R(0) ? 1 : 0) * y_v) / K(C_tauVPlus)));
    dydt[S_w] = ((((R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * (a_wInfty - y_w)) / a_tauWMinus) - (((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) * y_w) / K(C_tauWPlus)));
    dydt[S_s] = ((((R(1.0) + cfg_tanh((K(C_kS) * (y_u - K(C_uS))))) / R(2.0)) - y_s) / a_tauS);
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    if (SOLVE_VM) {
        dydt[S_u] = ((-a_Jion) - a_Istim);
    }
    return a_Jion;
}

// Tissue mode (solveVmWithinODESolver false): the PDE owns the membrane
// potential, so state 0 is the same at every RKF45 stage of a PDE step and
// the algebraics computed from it and constants alone are too.  hoist()
// evaluates the ones the rest of the body reads, and the special-function
// subexpressions of the rest that depend on state 0 and constants alone,
// once per cell and step into H[NH]; rhs_tissue() is the body without them,
// reading H (the same expressions in the same order: bitwise the values
// of rhs() in FP64).
constexpr int NH = 7;
enum Hoisted { H_Jso, H_vInfty, H_tauVMinus, H_wInfty, H_tauWMinus, H_tauS };
template <class R, class KS>
__device__ __forceinline__ void hoist(R y_u, const KS& K, int tissue, R* H)
{
    (void)tissue; (void)K; (void)H; (void)y_u;
    R a_tauSo = (K(C_tauSo1) + (((K(C_tauSo2) - K(C_tauSo1)) * (R(1.0) + cfg_tanh((K(C_kSo) * (y_u - K(C_uSo)))))) / R(2.0)));
    R a_tauO = (((R(1.0) - (((y_u - K(C_thetaO))) > R(0) ? 1 : 0)) * K(C_tauO1)) + ((((y_u - K(C_thetaO))) > R(0) ? 1 : 0) * K(C_tauO2)));
    R a_Jso = ((((y_u - K(C_uO)) * (R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0))) / a_tauO) + ((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) / a_tauSo));
    R a_tauVMinus = (((R(1.0) - (((y_u - K(C_thetaVMinus))) > R(0) ? 1 : 0)) * K(C_tauV1Minus)) + ((((y_u - K(C_thetaVMinus))) > R(0) ? 1 : 0) * K(C_tauV2Minus)));
    R a_tauWMinus = (K(C_tauW1Minus) + (((K(C_tauW2Minus) - K(C_tauW1Minus)) * (R(1.0) + cfg_tanh((K(C_kWMinus) * (y_u - K(C_uWMinus)))))) / R(2.0)));
    R a_tauS = (((R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * K(C_tauS1)) + ((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) * K(C_tauS2)));
    R a_vInfty = (((K(C_thetaVMinus) - y_u)) > R(0) ? 1 : 0);
    R a_wInfty = (((R(1.0) - (((y_u - K(C_thetaO))) > R(0) ? 1 : 0)) * (R(1.0) - (y_u / K(C_tauWInfty)))) + ((((y_u - K(C_thetaO))) > R(0) ? 1 : 0) * K(C_wInftyStar)));
    H[H_Jso] = a_Jso;
    H[H_vInfty] = a_vInfty;
    H[H_tauVMinus] = cfg_hrcp(a_tauVMinus);
    H[H_wInfty] = a_wInfty;
    H[H_tauWMinus] = cfg_hrcp(a_tauWMinus);
    H[H_tauS] = cfg_hrcp(a_tauS);
    H[6] = ((R(1.0) + cfg_tanh((K(C_kS) * (y_u - K(C_uS))))) / R(2.0));
}
template <class R, class YS, class KS, class HS>
__device__ __forceinline__ R rhs_tissue(double t, const YS& Y, const KS& K, const HS& H, R* dydt, int tissue, const CfgStimulus& stim)
{
    constexpr bool SOLVE_VM = false;
    (void)tissue; (void)stim; (void)t; (void)H;
    const R y_u = Y(S_u);
    const R y_v = Y(S_v);
    const R y_w = Y(S_w);
    const R y_s = Y(S_s);
    R a_Jfi = (((((-y_v) * (((y_u - K(C_thetaV))) > R(0) ? 1 : 0)) * (y_u - K(C_thetaV))) * (K(C_uU) - y_u)) / K(C_tauFi));
    R a_Jsi = ((((-(((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * y_w) * y_s) / K(C_tauSi));
    R a_Jion = ((a_Jfi + H(H_Jso)) + a_Jsi);
    dydt[S_v] = (cfg_hdiv(((R(1.0) - (((y_u - K(C_thetaV))) > R(0) ? 1 : 0)) * (H(H_vInfty) - y_v)), H(H_tauVMinus)) - (((((y_u - K(C_thetaV))) > R(0) ? 1 : 0) * y_v) / K(C_tauVPlus)));
    dydt[S_w] = (cfg_hdiv(((R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * (H(H_wInfty) - y_w)), H(H_tauWMinus)) - (((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) * y_w) / K(C_tauWPlus)));
    dydt[S_s] = cfg_hdiv((H(6) - y_s), H(H_tauS));
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    if (SOLVE_VM) {
        dydt[S_u] = ((-a_Jion) - a_Istim);
    }
    return a_Jion;
}

// Ionic current after the step (computeVariables at tEnd).
template <class R, bool SOLVE_VM, class YS, class KS>
__device__ __forceinline__ R iion(double t, const YS& Y, const KS& K, int tissue, const CfgStimulus& stim)
{
    (void)tissue; (void)stim; (void)t;
    R dydt[NS];
    const R y_u = Y(S_u);
    const R y_v = Y(S_v);
    const R y_w = Y(S_w);
    const R y_s = Y(S_s);
    R a_tauSo = (K(C_tauSo1) + (((K(C_tauSo2) - K(C_tauSo1)) * (R(1.0) + cfg_tanh((K(C_kSo) * (y_u - K(C_uSo)))))) / R(2.0)));
    R a_tauO = (((R(1.0) - (((y_u - K(C_thetaO))) > R(0) ? 1 : 0)) * K(C_tauO1)) + ((((y_u - K(C_thetaO))) > R(0) ? 1 : 0) * K(C_tauO2)));
    R a_Jfi = (((((-y_v) * (((y_u - K(C_thetaV))) > R(0) ? 1 : 0)) * (y_u - K(C_thetaV))) * (K(C_uU) - y_u)) / K(C_tauFi));
    R a_Jso = ((((y_u - K(C_uO)) * (R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0))) / a_tauO) + ((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) / a_tauSo));
    R a_Jsi = ((((-(((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * y_w) * y_s) / K(C_tauSi));
    R a_Jion = ((a_Jfi + a_Jso) + a_Jsi);
    R a_tauVMinus = (((R(1.0) - (((y_u - K(C_thetaVMinus))) > R(0) ? 1 : 0)) * K(C_tauV1Minus)) + ((((y_u - K(C_thetaVMinus))) > R(0) ? 1 : 0) * K(C_tauV2Minus)));
    R a_tauWMinus = (K(C_tauW1Minus) + (((K(C_tauW2Minus) - K(C_tauW1Minus)) * (R(1.0) + cfg_tanh((K(C_kWMinus) * (y_u - K(C_uWMinus)))))) / R(2.0)));
    R a_tauS = (((R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * K(C_tauS1)) + ((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) * K(C_tauS2)));
    R a_vInfty = (((K(C_thetaVMinus) - y_u)) > R(0) ? 1 : 0);
    R a_wInfty = (((R(1.0) - (((y_u - K(C_thetaO))) > R(0) ? 1 : 0)) * (R(1.0) - (y_u / K(C_tauWInfty)))) + ((((y_u - K(C_thetaO))) > R(0) ? 1 : 0) * K(C_wInftyStar)));
    dydt[S_v] = ((((R(1.0) - (((y_u - K(C_thetaV))) > R(0) ? 1 : 0)) * (a_vInfty - y_v)) / a_tauVMinus) - (((((y_u - K(C_thetaV))) > R(0) ? 1 : 0) * y_v) / K(C_tauVPlus)));
    dydt[S_w] = ((((R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * (a_wInfty - y_w)) / a_tauWMinus) - (((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) * y_w) / K(C_tauWPlus)));
    dydt[S_s] = ((((R(1.0) + cfg_tanh((K(C_kS) * (y_u - K(C_uS))))) / R(2.0)) - y_s) / a_tauS);
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    if (SOLVE_VM) {
        dydt[S_u] = ((-a_Jion) - a_Istim);
    }
    (void)dydt;
    return a_Jion;
}

// computeVariables with every algebraic stored: A[k] is ALGEBRAIC[k] (0 for
// the ones the body does not assign), dydt the RATES it assigns.
template <class R, bool SOLVE_VM, class YS, class KS>
__device__ __forceinline__ void variables_all(double t, const YS& Y, const KS& K, R* A, R* dydt, int tissue, const CfgStimulus& stim)
{
    (void)tissue; (void)stim; (void)t;
    const R y_u = Y(S_u);
    const R y_v = Y(S_v);
    const R y_w = Y(S_w);
    const R y_s = Y(S_s);
    R a_tauSo = (K(C_tauSo1) + (((K(C_tauSo2) - K(C_tauSo1)) * (R(1.0) + cfg_tanh((K(C_kSo) * (y_u - K(C_uSo)))))) / R(2.0)));
    R a_tauO = (((R(1.0) - (((y_u - K(C_thetaO))) > R(0) ? 1 : 0)) * K(C_tauO1)) + ((((y_u - K(C_thetaO))) > R(0) ? 1 : 0) * K(C_tauO2)));
    R a_Jfi = (((((-y_v) * (((y_u - K(C_thetaV))) > R(0) ? 1 : 0)) * (y_u - K(C_thetaV))) * (K(C_uU) - y_u)) / K(C_tauFi));
    R a_Jso = ((((y_u - K(C_uO)) * (R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0))) / a_tauO) + ((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) / a_tauSo));
    R a_Jsi = ((((-(((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * y_w) * y_s) / K(C_tauSi));
    R a_Jion = ((a_Jfi + a_Jso) + a_Jsi);
    R a_tauVMinus = (((R(1.0) - (((y_u - K(C_thetaVMinus))) > R(0) ? 1 : 0)) * K(C_tauV1Minus)) + ((((y_u - K(C_thetaVMinus))) > R(0) ? 1 : 0) * K(C_tauV2Minus)));
    R a_tauWMinus = (K(C_tauW1Minus) + (((K(C_tauW2Minus) - K(C_tauW1Minus)) * (R(1.0) + cfg_tanh((K(C_kWMinus) * (y_u - K(C_uWMinus)))))) / R(2.0)));
    R a_tauS = (((R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * K(C_tauS1)) + ((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) * K(C_tauS2)));
    R a_vInfty = (((K(C_thetaVMinus) - y_u)) > R(0) ? 1 : 0);
    R a_wInfty = (((R(1.0) - (((y_u - K(C_thetaO))) > R(0) ? 1 : 0)) * (R(1.0) - (y_u / K(C_tauWInfty)))) + ((((y_u - K(C_thetaO))) > R(0) ? 1 : 0) * K(C_wInftyStar)));
    dydt[S_v] = ((((R(1.0) - (((y_u - K(C_thetaV))) > R(0) ? 1 : 0)) * (a_vInfty - y_v)) / a_tauVMinus) - (((((y_u - K(C_thetaV))) > R(0) ? 1 : 0) * y_v) / K(C_tauVPlus)));
    dydt[S_w] = ((((R(1.0) - (((y_u - K(C_thetaW))) > R(0) ? 1 : 0)) * (a_wInfty - y_w)) / a_tauWMinus) - (((((y_u - K(C_thetaW))) > R(0) ? 1 : 0) * y_w) / K(C_tauWPlus)));
    dydt[S_s] = ((((R(1.0) + cfg_tanh((K(C_kS) * (y_u - K(C_uS))))) / R(2.0)) - y_s) / a_tauS);
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    if (SOLVE_VM) {
        dydt[S_u] = ((-a_Jion) - a_Istim);
    }
    A[0] = a_Jfi;
    A[1] = a_Jso;
    A[2] = a_Jsi;
    A[3] = a_Jion;
    A[4] = a_Istim;
    A[5] = a_tauSo;
    A[6] = a_tauO;
    A[7] = a_tauVMinus;
    A[8] = a_tauWMinus;
    A[9] = a_tauS;
    A[10] = a_vInfty;
    A[11] = a_wInfty;
}

// STATES_NAMES / ALGEBRAIC_NAMES as the header spells them; matched by
// position, entries the header leaves out are empty
static const char* const STATE_STRINGS[4] = {"u", "v", "w", "s"};
static const char* const ALG_STRINGS[12] = {"Jfi", "Jso", "Jsi", "Jion", "Istim", "tauSo", "tauO", "tauVMinus", "tauWMinus", "tauS", "vInfty", "wInfty"};
// <Model>DependencyMap(): current -> comma-separated variables, null-ended
static const char* const SWEEP_CURRENTS[] = {"Jfi", "Jso", "Jsi", "Jion", "v", "w", "s", "I_fi", "I_so", "I_si", "Iion", "I_ion", "Iion_cm", nullptr};
static const char* const SWEEP_DEPS[] = {"Jfi,v,RATES_v", "Jso,tauO,tauSo", "Jsi,w,s,RATES_s", "Jfi,Jso,Jsi,Jion", "v,vInfty,tauVMinus,RATES_v", "w,wInfty,tauWMinus,RATES_w", "s,tauS,RATES_s", "Jfi,v,RATES_v", "Jso,tauO,tauSo", "Jsi,w,s,RATES_s", "Jfi,Jso,Jsi,Jion", "Jfi,Jso,Jsi,Jion", "Jfi,Jso,Jsi,Jion", nullptr};

// traits bundle used by the kernel templates
struct Model {
    static constexpr int NS = buenoorovio::NS, NC = buenoorovio::NC;
    static constexpr unsigned long long WIDE_MASK = buenoorovio::WIDE_MASK;
    static constexpr double IION_SCALE = buenoorovio::IION_SCALE;
    static constexpr double TIME_SCALE = buenoorovio::TIME_SCALE;
    static constexpr int VM_MAP = buenoorovio::VM_MAP;
    CFG_HD static __forceinline__ void init(double* C, double* y, int tissue, const double* scale) { init_consts(C, y, tissue, scale); }
    template <int T> CFG_HD static constexpr double constant(int i) { return cval<T>(i); }
    static constexpr int NSD = buenoorovio::NSD, CA_STATE = buenoorovio::CA_STATE;
    static constexpr int NH = buenoorovio::NH;
    template <class R, class KS>
    __device__ static __forceinline__ void hoist_vm(R v, const KS& K, int tissue, R* H) { hoist<R>(v, K, tissue, H); }
    template <class R, class YS, class KS, class HS>
    __device__ static __forceinline__ R rates_tissue(double t, const YS& Y, const KS& K, const HS& H, R* dydt, int tissue, const CfgStimulus& st) { return rhs_tissue<R>(t, Y, K, H, dydt, tissue, st); }
    CFG_HD static constexpr int sd_slot(int i) { return buenoorovio::sd_slot(i); }
    static constexpr int NA = buenoorovio::NA;
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ void all_variables(double t, const YS& Y, const KS& K, R* A, R* dydt, int tissue, const CfgStimulus& st) { variables_all<R, SV>(t, Y, K, A, dydt, tissue, st); }
    CFG_HD static constexpr int sd_const(int k) { return buenoorovio::sd_const(k); }
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ R rates(double t, const YS& Y, const KS& K, R* dydt, int tissue, const CfgStimulus& st) { return rhs<R, SV>(t, Y, K, dydt, tissue, st); }
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ R current(double t, const YS& Y, const KS& K, int tissue, const CfgStimulus& st) { return iion<R, SV>(t, Y, K, tissue, st); }
};

} }  // namespace cfg::buenoorovio
