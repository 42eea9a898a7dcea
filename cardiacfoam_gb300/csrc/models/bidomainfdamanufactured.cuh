// Generated by cardiacfoam_gb300.cellml2cuda from src/ionicModels/bidomainFDAManufactured/bidomainFDAManufactured_2014.H.
// The equations are the published cell model as cellML2foam wrote them;
// regenerate with `python -m cardiacfoam_gb300.cellml2cuda` instead of editing.
#pragma once
#include "../ionic_common.cuh"

namespace cfg { namespace bidomainfdamanufactured {

constexpr int NS = 4;
constexpr int NC = 3;
constexpr int NA = 1;
enum State { S_BidomainV, S_BidomainU1, S_BidomainU2, S_BidomainU3 };
enum Constant { C_BidomainCm, C_BidomainBeta, C_BidomainChi };
// states kept in double in the mixed form (bit i = state i)
constexpr unsigned long long WIDE_MASK = 0xfull;
constexpr double IION_SCALE = 0.5;
constexpr double TIME_SCALE = 1000.0;
constexpr int VM_MAP = CFG_VM_IDENTITY;
constexpr int N_TISSUES = 3;
static const int TISSUES[] = {11, 12, 13, 0};
using TissueSet = TissueList<11, 12, 13>;
static const char* const STATE_NAMES[NS] = {"BidomainV", "BidomainU1", "BidomainU2", "BidomainU3"};
CFG_HD inline bool tissue_supported(int t) { return t == 11 || t == 12 || t == 13; }

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
    C[C_BidomainCm] = 2.0;
    C[C_BidomainChi] = 3.0;
    C[C_BidomainBeta] = 0.0;
    if (((tissue - 10) == 1)) {
        C[C_BidomainBeta] = (-1.1);
    } else {
        if (((tissue - 10) == 2)) {
            C[C_BidomainBeta] = (-5.9);
        } else {
            if (((tissue - 10) == 3)) {
                C[C_BidomainBeta] = (-8.6);
            } else {
                /* unsupported configuration in the reference */
            }
        }
    }
    C[C_BidomainBeta] = (C[C_BidomainBeta] * (1.0 - 0.7071067811865476));
}

// initConsts evaluated per tissue flag (IEEE double, the header's order of
// operations): cval<T>(i) is constant i for tissue T.  Kernels for one uniform
// tissue without per-cell scales read constants from here, so the compiler
// folds them into the instructions.
template <int T> CFG_HD constexpr double cval(int i);
template <> CFG_HD constexpr double cval<11>(int i)
{
    switch (i) {
    case 0: return 2.0;
    case 1: return -0.3221825406947977;
    case 2: return 3.0;
    default: return 0.0;
    }
}
template <> CFG_HD constexpr double cval<12>(int i)
{
    switch (i) {
    case 0: return 2.0;
    case 1: return -1.7280699909993695;
    case 2: return 3.0;
    default: return 0.0;
    }
}
template <> CFG_HD constexpr double cval<13>(int i)
{
    switch (i) {
    case 0: return 2.0;
    case 1: return -2.518881681795691;
    case 2: return 3.0;
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
    const R y_BidomainV = Y(S_BidomainV);
    const R y_BidomainU1 = Y(S_BidomainU1);
    const R y_BidomainU2 = Y(S_BidomainU2);
    const R y_BidomainU3 = Y(S_BidomainU3);
    dydt[S_BidomainV] = R(0.0);
    dydt[S_BidomainU1] = ((cfg_ipow<2>(((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<2>(y_BidomainU2)) + (((R(0.5) * ((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<2>(y_BidomainU2)) * (y_BidomainV - y_BidomainU3)));
    dydt[S_BidomainU2] = ((-((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<3>(y_BidomainU2));
    dydt[S_BidomainU3] = R(0.0);
    R a_BidomainIion = ((((((-R(0.5)) * K(C_BidomainCm)) * ((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<2>(y_BidomainU2)) * (y_BidomainV - y_BidomainU3)) + ((K(C_BidomainBeta) * (y_BidomainV - y_BidomainU3)) / K(C_BidomainChi)));
    return a_BidomainIion;
}

// Tissue mode (solveVmWithinODESolver false): the PDE owns the membrane
// potential, so state 0 is the same at every RKF45 stage of a PDE step and
// the algebraics computed from it and constants alone are too.  hoist()
// evaluates the ones the rest of the body reads, and the special-function
// subexpressions of the rest that depend on state 0 and constants alone,
// once per cell and step into H[NH]; rhs_tissue() is the body without them,
// reading H (the same expressions in the same order: bitwise the values
// of rhs() in FP64).
constexpr int NH = 0;
template <class R, class KS>
__device__ __forceinline__ void hoist(R y_BidomainV, const KS& K, int tissue, R* H)
{
    (void)tissue; (void)K; (void)H; (void)y_BidomainV;
}
template <class R, class YS, class KS, class HS>
__device__ __forceinline__ R rhs_tissue(double t, const YS& Y, const KS& K, const HS& H, R* dydt, int tissue, const CfgStimulus& stim)
{
    (void)H;
    return rhs<R, false>(t, Y, K, dydt, tissue, stim);
}

// Ionic current after the step (computeVariables at tEnd).
template <class R, bool SOLVE_VM, class YS, class KS>
__device__ __forceinline__ R iion(double t, const YS& Y, const KS& K, int tissue, const CfgStimulus& stim)
{
    (void)tissue; (void)stim; (void)t;
    R dydt[NS];
    const R y_BidomainV = Y(S_BidomainV);
    const R y_BidomainU1 = Y(S_BidomainU1);
    const R y_BidomainU2 = Y(S_BidomainU2);
    const R y_BidomainU3 = Y(S_BidomainU3);
    dydt[S_BidomainV] = R(0.0);
    dydt[S_BidomainU1] = ((cfg_ipow<2>(((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<2>(y_BidomainU2)) + (((R(0.5) * ((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<2>(y_BidomainU2)) * (y_BidomainV - y_BidomainU3)));
    dydt[S_BidomainU2] = ((-((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<3>(y_BidomainU2));
    dydt[S_BidomainU3] = R(0.0);
    R a_BidomainIion = ((((((-R(0.5)) * K(C_BidomainCm)) * ((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<2>(y_BidomainU2)) * (y_BidomainV - y_BidomainU3)) + ((K(C_BidomainBeta) * (y_BidomainV - y_BidomainU3)) / K(C_BidomainChi)));
    (void)dydt;
    return a_BidomainIion;
}

// computeVariables with every algebraic stored: A[k] is ALGEBRAIC[k] (0 for
// the ones the body does not assign), dydt the RATES it assigns.
template <class R, bool SOLVE_VM, class YS, class KS>
__device__ __forceinline__ void variables_all(double t, const YS& Y, const KS& K, R* A, R* dydt, int tissue, const CfgStimulus& stim)
{
    (void)tissue; (void)stim; (void)t;
    const R y_BidomainV = Y(S_BidomainV);
    const R y_BidomainU1 = Y(S_BidomainU1);
    const R y_BidomainU2 = Y(S_BidomainU2);
    const R y_BidomainU3 = Y(S_BidomainU3);
    dydt[S_BidomainV] = R(0.0);
    dydt[S_BidomainU1] = ((cfg_ipow<2>(((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<2>(y_BidomainU2)) + (((R(0.5) * ((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<2>(y_BidomainU2)) * (y_BidomainV - y_BidomainU3)));
    dydt[S_BidomainU2] = ((-((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<3>(y_BidomainU2));
    dydt[S_BidomainU3] = R(0.0);
    R a_BidomainIion = ((((((-R(0.5)) * K(C_BidomainCm)) * ((y_BidomainU1 + y_BidomainU3) - y_BidomainV)) * cfg_ipow<2>(y_BidomainU2)) * (y_BidomainV - y_BidomainU3)) + ((K(C_BidomainBeta) * (y_BidomainV - y_BidomainU3)) / K(C_BidomainChi)));
    A[0] = a_BidomainIion;
}

// STATES_NAMES / ALGEBRAIC_NAMES as the header spells them; matched by
// position, entries the header leaves out are empty
static const char* const STATE_STRINGS[4] = {"V", "u1", "u2", "u3"};
static const char* const ALG_STRINGS[1] = {"Iion"};
// <Model>DependencyMap(): current -> comma-separated variables, null-ended
static const char* const SWEEP_CURRENTS[] = {nullptr};
static const char* const SWEEP_DEPS[] = {nullptr};

// traits bundle used by the kernel templates
struct Model {
    static constexpr int NS = bidomainfdamanufactured::NS, NC = bidomainfdamanufactured::NC;
    static constexpr unsigned long long WIDE_MASK = bidomainfdamanufactured::WIDE_MASK;
    static constexpr double IION_SCALE = bidomainfdamanufactured::IION_SCALE;
    static constexpr double TIME_SCALE = bidomainfdamanufactured::TIME_SCALE;
    static constexpr int VM_MAP = bidomainfdamanufactured::VM_MAP;
    CFG_HD static __forceinline__ void init(double* C, double* y, int tissue, const double* scale) { init_consts(C, y, tissue, scale); }
    template <int T> CFG_HD static constexpr double constant(int i) { return cval<T>(i); }
    static constexpr int NSD = bidomainfdamanufactured::NSD, CA_STATE = bidomainfdamanufactured::CA_STATE;
    static constexpr int NH = bidomainfdamanufactured::NH;
    template <class R, class KS>
    __device__ static __forceinline__ void hoist_vm(R v, const KS& K, int tissue, R* H) { hoist<R>(v, K, tissue, H); }
    template <class R, class YS, class KS, class HS>
    __device__ static __forceinline__ R rates_tissue(double t, const YS& Y, const KS& K, const HS& H, R* dydt, int tissue, const CfgStimulus& st) { return rhs_tissue<R>(t, Y, K, H, dydt, tissue, st); }
    CFG_HD static constexpr int sd_slot(int i) { return bidomainfdamanufactured::sd_slot(i); }
    static constexpr int NA = bidomainfdamanufactured::NA;
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ void all_variables(double t, const YS& Y, const KS& K, R* A, R* dydt, int tissue, const CfgStimulus& st) { variables_all<R, SV>(t, Y, K, A, dydt, tissue, st); }
    CFG_HD static constexpr int sd_const(int k) { return bidomainfdamanufactured::sd_const(k); }
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ R rates(double t, const YS& Y, const KS& K, R* dydt, int tissue, const CfgStimulus& st) { return rhs<R, SV>(t, Y, K, dydt, tissue, st); }
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ R current(double t, const YS& Y, const KS& K, int tissue, const CfgStimulus& st) { return iion<R, SV>(t, Y, K, tissue, st); }
};

} }  // namespace cfg::bidomainfdamanufactured
