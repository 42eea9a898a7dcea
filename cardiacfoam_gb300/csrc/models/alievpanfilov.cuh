// Generated by cardiacfoam_gb300.cellml2cuda from src/ionicModels/AlievPanfilov/AlievPanfilov_1996.H.
// The equations are the published cell model as cellML2foam wrote them;
// regenerate with `python -m cardiacfoam_gb300.cellml2cuda` instead of editing.
#pragma once
#include "../ionic_common.cuh"

namespace cfg { namespace alievpanfilov {

constexpr int NS = 2;
constexpr int NC = 8;
constexpr int NA = 3;
enum State { S_u, S_recovery_r };
enum Constant { C_AC_Vp, C_AC_Vr, C_AC_Vth, C_AC_epsilon, C_AC_k, C_AC_mu1, C_AC_mu2, C_AC_a };
// states kept in double in the mixed form (bit i = state i)
constexpr unsigned long long WIDE_MASK = 0x3ull;
constexpr double IION_SCALE = 100.0;
constexpr double TIME_SCALE = 12.9;
constexpr int VM_MAP = CFG_VM_ALIEV;
constexpr int N_TISSUES = 1;
static const int TISSUES[] = {4, 0};
using TissueSet = TissueList<4>;
static const char* const STATE_NAMES[NS] = {"u", "recovery_r"};
CFG_HD inline bool tissue_supported(int t) { return t == 4; }

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
    C[C_AC_Vp] = 20.0;
    C[C_AC_Vr] = (-80.0);
    C[C_AC_Vth] = (-70.0);
    C[C_AC_epsilon] = 0.01;
    C[C_AC_k] = 8.0;
    C[C_AC_mu1] = 0.2;
    C[C_AC_mu2] = 0.3;
    C[C_AC_a] = ((C[C_AC_Vth] - C[C_AC_Vr]) / (C[C_AC_Vp] - C[C_AC_Vr]));
    y[S_u] = 0.05;
    y[S_recovery_r] = 0.0;
}

// initConsts evaluated per tissue flag (IEEE double, the header's order of
// operations): cval<T>(i) is constant i for tissue T.  Kernels for one uniform
// tissue without per-cell scales read constants from here, so the compiler
// folds them into the instructions.
template <int T> CFG_HD constexpr double cval(int i);
template <> CFG_HD constexpr double cval<4>(int i)
{
    switch (i) {
    case 0: return 20.0;
    case 1: return -80.0;
    case 2: return -70.0;
    case 3: return 0.01;
    case 4: return 8.0;
    case 5: return 0.2;
    case 6: return 0.3;
    case 7: return 0.1;
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
    const R y_recovery_r = Y(S_recovery_r);
    R a_AV_eps = (K(C_AC_epsilon) + ((K(C_AC_mu1) * y_recovery_r) / (K(C_AC_mu2) + y_u)));
    dydt[S_recovery_r] = (a_AV_eps * ((-y_recovery_r) - ((K(C_AC_k) * y_u) * (y_u - (K(C_AC_a) + R(1.0))))));
    R a_Iion_cm = ((((K(C_AC_k) * y_u) * (y_u - K(C_AC_a))) * (y_u - R(1.0))) + (y_recovery_r * y_u));
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    if (SOLVE_VM) {
        dydt[S_u] = ((-a_Iion_cm) - a_Istim);
    }
    return a_Iion_cm;
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
__device__ __forceinline__ void hoist(R y_u, const KS& K, int tissue, R* H)
{
    (void)tissue; (void)K; (void)H; (void)y_u;
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
    const R y_u = Y(S_u);
    const R y_recovery_r = Y(S_recovery_r);
    R a_AV_eps = (K(C_AC_epsilon) + ((K(C_AC_mu1) * y_recovery_r) / (K(C_AC_mu2) + y_u)));
    dydt[S_recovery_r] = (a_AV_eps * ((-y_recovery_r) - ((K(C_AC_k) * y_u) * (y_u - (K(C_AC_a) + R(1.0))))));
    R a_Iion_cm = ((((K(C_AC_k) * y_u) * (y_u - K(C_AC_a))) * (y_u - R(1.0))) + (y_recovery_r * y_u));
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    if (SOLVE_VM) {
        dydt[S_u] = ((-a_Iion_cm) - a_Istim);
    }
    (void)dydt;
    return a_Iion_cm;
}

// computeVariables with every algebraic stored: A[k] is ALGEBRAIC[k] (0 for
// the ones the body does not assign), dydt the RATES it assigns.
template <class R, bool SOLVE_VM, class YS, class KS>
__device__ __forceinline__ void variables_all(double t, const YS& Y, const KS& K, R* A, R* dydt, int tissue, const CfgStimulus& stim)
{
    (void)tissue; (void)stim; (void)t;
    const R y_u = Y(S_u);
    const R y_recovery_r = Y(S_recovery_r);
    R a_AV_eps = (K(C_AC_epsilon) + ((K(C_AC_mu1) * y_recovery_r) / (K(C_AC_mu2) + y_u)));
    dydt[S_recovery_r] = (a_AV_eps * ((-y_recovery_r) - ((K(C_AC_k) * y_u) * (y_u - (K(C_AC_a) + R(1.0))))));
    R a_Iion_cm = ((((K(C_AC_k) * y_u) * (y_u - K(C_AC_a))) * (y_u - R(1.0))) + (y_recovery_r * y_u));
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    if (SOLVE_VM) {
        dydt[S_u] = ((-a_Iion_cm) - a_Istim);
    }
    A[0] = a_AV_eps;
    A[1] = a_Istim;
    A[2] = a_Iion_cm;
}

// STATES_NAMES / ALGEBRAIC_NAMES as the header spells them; matched by
// position, entries the header leaves out are empty
static const char* const STATE_STRINGS[2] = {"u", "recovery_r"};
static const char* const ALG_STRINGS[3] = {"AV_eps", "Istim", "Iion_cm"};
// <Model>DependencyMap(): current -> comma-separated variables, null-ended
static const char* const SWEEP_CURRENTS[] = {"Iion", "I_ion", "Iion_cm", "u", "recovery_r", nullptr};
static const char* const SWEEP_DEPS[] = {"Iion_cm,u,recovery_r,AV_eps", "Iion_cm,u,recovery_r,AV_eps", "Iion_cm,u,recovery_r,AV_eps", "u,RATES_u", "recovery_r,AV_eps,RATES_recovery_r", nullptr};

// traits bundle used by the kernel templates
struct Model {
    static constexpr int NS = alievpanfilov::NS, NC = alievpanfilov::NC;
    static constexpr unsigned long long WIDE_MASK = alievpanfilov::WIDE_MASK;
    static constexpr double IION_SCALE = alievpanfilov::IION_SCALE;
    static constexpr double TIME_SCALE = alievpanfilov::TIME_SCALE;
    static constexpr int VM_MAP = alievpanfilov::VM_MAP;
    CFG_HD static __forceinline__ void init(double* C, double* y, int tissue, const double* scale) { init_consts(C, y, tissue, scale); }
    template <int T> CFG_HD static constexpr double constant(int i) { return cval<T>(i); }
    static constexpr int NSD = alievpanfilov::NSD, CA_STATE = alievpanfilov::CA_STATE;
    static constexpr int NH = alievpanfilov::NH;
    template <class R, class KS>
    __device__ static __forceinline__ void hoist_vm(R v, const KS& K, int tissue, R* H) { hoist<R>(v, K, tissue, H); }
    template <class R, class YS, class KS, class HS>
    __device__ static __forceinline__ R rates_tissue(double t, const YS& Y, const KS& K, const HS& H, R* dydt, int tissue, const CfgStimulus& st) { return rhs_tissue<R>(t, Y, K, H, dydt, tissue, st); }
    CFG_HD static constexpr int sd_slot(int i) { return alievpanfilov::sd_slot(i); }
    static constexpr int NA = alievpanfilov::NA;
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ void all_variables(double t, const YS& Y, const KS& K, R* A, R* dydt, int tissue, const CfgStimulus& st) { variables_all<R, SV>(t, Y, K, A, dydt, tissue, st); }
    CFG_HD static constexpr int sd_const(int k) { return alievpanfilov::sd_const(k); }
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ R rates(double t, const YS& Y, const KS& K, R* dydt, int tissue, const CfgStimulus& st) { return rhs<R, SV>(t, Y, K, dydt, tissue, st); }
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ R current(double t, const YS& Y, const KS& K, int tissue, const CfgStimulus& st) { return iion<R, SV>(t, Y, K, tissue, st); }
};

} }  // namespace cfg::alievpanfilov
