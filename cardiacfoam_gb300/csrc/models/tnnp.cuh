// Generated by cardiacfoam_gb300.cellml2cuda from src/ionicModels/TNNP/TNNP_2004.H.
// The equations are the published cell model as cellML2foam wrote them;
// regenerate with `python -m cardiacfoam_gb300.cellml2cuda` instead of editing.
#pragma once
#include "../ionic_common.cuh"

namespace cfg { namespace tnnp {

constexpr int NS = 17;
constexpr int NC = 42;
constexpr int NA = 70;
enum State { S_V, S_K_i, S_Na_i, S_Ca_i, S_Xr1, S_Xr2, S_Xs, S_m, S_h, S_j, S_d, S_f, S_fCa, S_s, S_r, S_Ca_SR, S_g };
enum Constant { C_R, C_T, C_F, C_Cm, C_V_c, C_P_kna, C_K_o, C_Na_o, C_Ca_o, C_g_K1, C_g_Kr, C_g_Ks, C_g_Na, C_g_bNa, C_g_CaL, C_g_bCa, C_g_to, C_P_NaK, C_K_mk, C_K_mNa, C_K_NaCa, C_K_sat, C_alpha_NCX, C_gamma_NCX, C_Km_Ca, C_Km_Nai, C_g_pCa, C_K_pCa, C_g_pK, C_tau_g, C_a_rel, C_b_rel, C_c_rel, C_K_up, C_V_leak, C_Vmax_up, C_Buf_c, C_K_buf_c, C_Buf_sr, C_K_buf_sr, C_V_sr, C_tau_fCa };
// states kept in double in the mixed form (bit i = state i)
constexpr unsigned long long WIDE_MASK = 0x800full;
constexpr double IION_SCALE = 1.0;
constexpr double TIME_SCALE = 1.0;
constexpr int VM_MAP = CFG_VM_MV;
constexpr int N_TISSUES = 3;
static const int TISSUES[] = {3, 2, 1, 0};
using TissueSet = TissueList<3, 2, 1>;
static const char* const STATE_NAMES[NS] = {"V", "K_i", "Na_i", "Ca_i", "Xr1", "Xr2", "Xs", "m", "h", "j", "d", "f", "fCa", "s", "r", "Ca_SR", "g"};
CFG_HD inline bool tissue_supported(int t) { return t == 3 || t == 2 || t == 1; }

// per-cell conductance scales: index into the scale vector, or -1
constexpr int SCALE_GNa = 0;
constexpr int SCALE_GCaL = 1;
constexpr int SCALE_GKr = 2;
constexpr int SCALE_GKs = 3;
constexpr int SCALE_GK1 = 4;
constexpr int SCALE_Gto = 5;

// Constants that depend on the per-cell conductance scales and that the
// right-hand side reads: the scaled conductances and every constant
// initConsts derives from them.  sd_slot(i) is constant i's index in a
// cell's vector of them, or -1 (then the constant is the tissue's).
constexpr int NSD = 6;
CFG_HD constexpr int sd_const(int k)
{
    switch (k) {
    case 0: return C_g_K1;
    case 1: return C_g_Kr;
    case 2: return C_g_Ks;
    case 3: return C_g_Na;
    case 4: return C_g_CaL;
    case 5: return C_g_to;
    default: return -1;
    }
}
CFG_HD constexpr int sd_slot(int i)
{
    switch (i) {
    case C_g_K1: return 0;
    case C_g_Kr: return 1;
    case C_g_Ks: return 2;
    case C_g_Na: return 3;
    case C_g_CaL: return 4;
    case C_g_to: return 5;
    default: return -1;
    }
}
// intracellular calcium state (peak Ca of a beat), or -1
constexpr int CA_STATE = S_Ca_i;

// Constants and initial states (initConsts).  `scale` may be null;
// otherwise scale[SCALE_x] multiplies the named conductance right after
// it is assigned, before constants derived from it are computed.
CFG_HD __forceinline__ void init_consts(double* C, double* y, int tissue, const double* scale)
{
    (void)tissue; (void)scale;
    y[S_V] = (-86.2);
    C[C_R] = 8.314;
    C[C_T] = 310;
    C[C_F] = 96.485;
    C[C_Cm] = 185;
    C[C_V_c] = 16404;
    C[C_P_kna] = 0.03;
    C[C_K_o] = 5.4;
    C[C_Na_o] = 140;
    y[S_K_i] = 138.3;
    y[S_Na_i] = 11.6;
    C[C_Ca_o] = 2;
    y[S_Ca_i] = 0.0002;
    C[C_g_K1] = 5.405;
    if (scale) C[C_g_K1] *= scale[SCALE_GK1];
    C[C_g_Kr] = 0.096;
    if (scale) C[C_g_Kr] *= scale[SCALE_GKr];
    y[S_Xr1] = 0;
    y[S_Xr2] = 1;
    C[C_g_Ks] = ((tissue == 2) ? 0.062 : 0.245);
    if (scale) C[C_g_Ks] *= scale[SCALE_GKs];
    y[S_Xs] = 0;
    C[C_g_Na] = 14.838;
    if (scale) C[C_g_Na] *= scale[SCALE_GNa];
    y[S_m] = 0;
    y[S_h] = 0.75;
    y[S_j] = 0.75;
    C[C_g_bNa] = 0.00029;
    C[C_g_CaL] = 0.175;
    if (scale) C[C_g_CaL] *= scale[SCALE_GCaL];
    y[S_d] = 0;
    y[S_f] = 1;
    y[S_fCa] = 1;
    C[C_g_bCa] = 0.000592;
    C[C_g_to] = ((tissue == 3) ? 0.073 : 0.294);
    if (scale) C[C_g_to] *= scale[SCALE_Gto];
    y[S_s] = 1;
    y[S_r] = 0;
    C[C_P_NaK] = 1.362;
    C[C_K_mk] = 1;
    C[C_K_mNa] = 40;
    C[C_K_NaCa] = 1000;
    C[C_K_sat] = 0.1;
    C[C_alpha_NCX] = 2.5;
    C[C_gamma_NCX] = 0.35;
    C[C_Km_Ca] = 1.38;
    C[C_Km_Nai] = 87.5;
    C[C_g_pCa] = 0.825;
    C[C_K_pCa] = 0.0005;
    C[C_g_pK] = 0.0146;
    y[S_Ca_SR] = 0.2;
    y[S_g] = 1;
    C[C_tau_g] = 2;
    C[C_a_rel] = 0.016464;
    C[C_b_rel] = 0.25;
    C[C_c_rel] = 0.008232;
    C[C_K_up] = 0.00025;
    C[C_V_leak] = 8e-5;
    C[C_Vmax_up] = 0.000425;
    C[C_Buf_c] = 0.15;
    C[C_K_buf_c] = 0.001;
    C[C_Buf_sr] = 10;
    C[C_K_buf_sr] = 0.3;
    C[C_V_sr] = 1094;
    C[C_tau_fCa] = 2.00000;
}

// initConsts evaluated per tissue flag (IEEE double, the header's order of
// operations): cval<T>(i) is constant i for tissue T.  Kernels for one uniform
// tissue without per-cell scales read constants from here, so the compiler
// folds them into the instructions.
template <int T> CFG_HD constexpr double cval(int i);
template <> CFG_HD constexpr double cval<3>(int i)
{
    switch (i) {
    case 0: return 8.314;
    case 1: return 310.0;
    case 2: return 96.485;
    case 3: return 185.0;
    case 4: return 16404.0;
    case 5: return 0.03;
    case 6: return 5.4;
    case 7: return 140.0;
    case 8: return 2.0;
    case 9: return 5.405;
    case 10: return 0.096;
    case 11: return 0.245;
    case 12: return 14.838;
    case 13: return 0.00029;
    case 14: return 0.175;
    case 15: return 0.000592;
    case 16: return 0.073;
    case 17: return 1.362;
    case 18: return 1.0;
    case 19: return 40.0;
    case 20: return 1000.0;
    case 21: return 0.1;
    case 22: return 2.5;
    case 23: return 0.35;
    case 24: return 1.38;
    case 25: return 87.5;
    case 26: return 0.825;
    case 27: return 0.0005;
    case 28: return 0.0146;
    case 29: return 2.0;
    case 30: return 0.016464;
    case 31: return 0.25;
    case 32: return 0.008232;
    case 33: return 0.00025;
    case 34: return 8e-05;
    case 35: return 0.000425;
    case 36: return 0.15;
    case 37: return 0.001;
    case 38: return 10.0;
    case 39: return 0.3;
    case 40: return 1094.0;
    case 41: return 2.0;
    default: return 0.0;
    }
}
template <> CFG_HD constexpr double cval<2>(int i)
{
    switch (i) {
    case 0: return 8.314;
    case 1: return 310.0;
    case 2: return 96.485;
    case 3: return 185.0;
    case 4: return 16404.0;
    case 5: return 0.03;
    case 6: return 5.4;
    case 7: return 140.0;
    case 8: return 2.0;
    case 9: return 5.405;
    case 10: return 0.096;
    case 11: return 0.062;
    case 12: return 14.838;
    case 13: return 0.00029;
    case 14: return 0.175;
    case 15: return 0.000592;
    case 16: return 0.294;
    case 17: return 1.362;
    case 18: return 1.0;
    case 19: return 40.0;
    case 20: return 1000.0;
    case 21: return 0.1;
    case 22: return 2.5;
    case 23: return 0.35;
    case 24: return 1.38;
    case 25: return 87.5;
    case 26: return 0.825;
    case 27: return 0.0005;
    case 28: return 0.0146;
    case 29: return 2.0;
    case 30: return 0.016464;
    case 31: return 0.25;
    case 32: return 0.008232;
    case 33: return 0.00025;
    case 34: return 8e-05;
    case 35: return 0.000425;
    case 36: return 0.15;
    case 37: return 0.001;
    case 38: return 10.0;
    case 39: return 0.3;
    case 40: return 1094.0;
    case 41: return 2.0;
    default: return 0.0;
    }
}
template <> CFG_HD constexpr double cval<1>(int i)
{
    switch (i) {
    case 0: return 8.314;
    case 1: return 310.0;
    case 2: return 96.485;
    case 3: return 185.0;
    case 4: return 16404.0;
    case 5: return 0.03;
    case 6: return 5.4;
    case 7: return 140.0;
    case 8: return 2.0;
    case 9: return 5.405;
    case 10: return 0.096;
    case 11: return 0.245;
    case 12: return 14.838;
    case 13: return 0.00029;
    case 14: return 0.175;
    case 15: return 0.000592;
    case 16: return 0.294;
    case 17: return 1.362;
    case 18: return 1.0;
    case 19: return 40.0;
    case 20: return 1000.0;
    case 21: return 0.1;
    case 22: return 2.5;
    case 23: return 0.35;
    case 24: return 1.38;
    case 25: return 87.5;
    case 26: return 0.825;
    case 27: return 0.0005;
    case 28: return 0.0146;
    case 29: return 2.0;
    case 30: return 0.016464;
    case 31: return 0.25;
    case 32: return 0.008232;
    case 33: return 0.00025;
    case 34: return 8e-05;
    case 35: return 0.000425;
    case 36: return 0.15;
    case 37: return 0.001;
    case 38: return 10.0;
    case 39: return 0.3;
    case 40: return 1094.0;
    case 41: return 2.0;
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
    const R y_V = Y(S_V);
    const R y_K_i = Y(S_K_i);
    const R y_Na_i = Y(S_Na_i);
    const R y_Ca_i = Y(S_Ca_i);
    const R y_Xr1 = Y(S_Xr1);
    const R y_Xr2 = Y(S_Xr2);
    const R y_Xs = Y(S_Xs);
    const R y_m = Y(S_m);
    const R y_h = Y(S_h);
    const R y_j = Y(S_j);
    const R y_d = Y(S_d);
    const R y_f = Y(S_f);
    const R y_fCa = Y(S_fCa);
    const R y_s = Y(S_s);
    const R y_r = Y(S_r);
    const R y_Ca_SR = Y(S_Ca_SR);
    const R y_g = Y(S_g);
    R a_m_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp((((-R(56.8600)) - y_V) / R(9.03000))))));
    R a_alpha_m = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(5.00000)))));
    R a_beta_m = ((R(0.100000) / (R(1.00000) + cfg_exp(((y_V + R(35.0000)) / R(5.00000))))) + (R(0.100000) / (R(1.00000) + cfg_exp(((y_V - R(50.0000)) / R(200.000))))));
    R a_tau_m = ((R(1.00000) * a_alpha_m) * a_beta_m);
    dydt[S_m] = ((a_m_inf - y_m) / a_tau_m);
    R a_h_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    R a_alpha_h = ((y_V < (-R(40.0000))) ? (R(0.0570000) * cfg_exp(((-(y_V + R(80.0000))) / R(6.80000)))) : R(0.00000));
    R a_beta_h = ((y_V < (-R(40.0000))) ? ((R(2.70000) * cfg_exp((R(0.0790000) * y_V))) + (R(310000.) * cfg_exp((R(0.348500) * y_V)))) : (R(0.770000) / (R(0.130000) * (R(1.00000) + cfg_exp(((y_V + R(10.6600)) / (-R(11.1000))))))));
    R a_tau_h = (R(1.00000) / (a_alpha_h + a_beta_h));
    dydt[S_h] = ((a_h_inf - y_h) / a_tau_h);
    R a_j_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    R a_alpha_j = ((y_V < (-R(40.0000))) ? ((((((-R(25428.0)) * cfg_exp((R(0.244400) * y_V))) - (R(6.94800e-06) * cfg_exp(((-R(0.0439100)) * y_V)))) * (y_V + R(37.7800))) / R(1.00000)) / (R(1.00000) + cfg_exp((R(0.311000) * (y_V + R(79.2300)))))) : R(0.00000));
    R a_beta_j = ((y_V < (-R(40.0000))) ? ((R(0.0242400) * cfg_exp(((-R(0.0105200)) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.137800)) * (y_V + R(40.1400)))))) : ((R(0.600000) * cfg_exp((R(0.0570000) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.100000)) * (y_V + R(32.0000)))))));
    R a_tau_j = (R(1.00000) / (a_alpha_j + a_beta_j));
    dydt[S_j] = ((a_j_inf - y_j) / a_tau_j);
    R a_d_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(7.50000)))));
    R a_alpha_d = ((R(1.40000) / (R(1.00000) + cfg_exp((((-R(35.0000)) - y_V) / R(13.0000))))) + R(0.250000));
    R a_gama_fCa = (R(1.40000) / (R(1.00000) + cfg_exp(((y_V + R(5.00000)) / R(5.00000)))));
    R a_gamma_d = (R(1.00000) / (R(1.00000) + cfg_exp(((R(50.0000) - y_V) / R(20.0000)))));
    R a_tau_d = (((R(1.00000) * a_alpha_d) * a_gama_fCa) + a_gamma_d);
    dydt[S_d] = ((a_d_inf - y_d) / a_tau_d);
    R a_f_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(7.00000)))));
    R a_tau_f = (((R(1125.00) * cfg_exp(((-cfg_ipow<2>((y_V + R(27.0000)))) / R(240.000)))) + R(80.0000)) + (R(165.000) / (R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(10.0000))))));
    dydt[S_f] = ((a_f_inf - y_f) / a_tau_f);
    R a_alpha_fCa = (R(1.00000) / (R(1.00000) + cfg_ipow<8>((y_Ca_i / R(0.000325000)))));
    R a_beta_fCa = (R(0.100000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000500000)) / R(0.000100000)))));
    R a_beta_d = (R(0.200000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000750000)) / R(0.000800000)))));
    R a_fCa_inf = ((((a_alpha_fCa + a_beta_fCa) + a_beta_d) + R(0.230000)) / R(1.46000));
    R a_d_fCa = ((a_fCa_inf - y_fCa) / K(C_tau_fCa));
    dydt[S_fCa] = (((a_fCa_inf > y_fCa) && (y_V > (-R(60.0000)))) ? R(0.00000) : a_d_fCa);
    R a_s_inf = ((tissue == 1) ? (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(5.00000))))) : (R(1.10000) / (R(1.00000) + cfg_exp(((y_V + R(28.0000)) / R(6.00000))))));
    R a_tau_s = ((tissue == 1) ? (((R(85.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(45.0000)))) / R(320.000)))) + (R(5.00000) / (R(1.00000) + cfg_exp(((y_V - R(20.0000)) / R(5.00000)))))) + R(3.00000)) : ((R(1000.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(67.0000)))) / R(1000.000)))) + R(8.00000)));
    dydt[S_s] = ((a_s_inf - y_s) / a_tau_s);
    R a_r_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((R(20.0000) - y_V) / R(6.00000)))));
    R a_tau_r = ((R(9.50000) * cfg_exp(((-cfg_ipow<2>((y_V + R(40.0000)))) / R(1800.00)))) + R(0.800000));
    dydt[S_r] = ((a_r_inf - y_r) / a_tau_r);
    R a_xr1_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(26.0000)) - y_V) / R(7.00000)))));
    R a_alpha_xr1 = (R(450.000) / (R(1.00000) + cfg_exp((((-R(45.0000)) - y_V) / R(10.0000)))));
    R a_beta_xr1 = (R(6.00000) / (R(1.00000) + cfg_exp(((y_V + R(30.0000)) / R(11.5000)))));
    R a_tau_xr1 = ((R(1.00000) * a_alpha_xr1) * a_beta_xr1);
    dydt[S_Xr1] = ((a_xr1_inf - y_Xr1) / a_tau_xr1);
    R a_xr2_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(88.0000)) / R(24.0000)))));
    R a_alpha_xr2 = (R(3.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(20.0000)))));
    R a_beta_xr2 = (R(1.12000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    R a_tau_xr2 = ((R(1.00000) * a_alpha_xr2) * a_beta_xr2);
    dydt[S_Xr2] = ((a_xr2_inf - y_Xr2) / a_tau_xr2);
    R a_xs_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(14.0000)))));
    R a_alpha_xs = (R(1100.00) / cfg_sqrt((R(1.00000) + cfg_exp((((-R(10.0000)) - y_V) / R(6.00000))))));
    R a_beta_xs = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    R a_tau_xs = ((R(1.00000) * a_alpha_xs) * a_beta_xs);
    dydt[S_Xs] = ((a_xs_inf - y_Xs) / a_tau_xs);
    R a_g_inf = ((y_Ca_i < R(0.000350000)) ? (R(1.00000) / (R(1.00000) + cfg_ipow<6>((y_Ca_i / R(0.000350000))))) : (R(1.00000) / (R(1.00000) + cfg_ipow<16>((y_Ca_i / R(0.000350000))))));
    R a_d_g = ((a_g_inf - y_g) / K(C_tau_g));
    dydt[S_g] = (((a_g_inf > y_g) && (y_V > (-R(60.0000)))) ? R(0.00000) : a_d_g);
    R a_i_NaK = (((((K(C_P_NaK) * K(C_K_o)) / (K(C_K_o) + K(C_K_mk))) * y_Na_i) / (y_Na_i + K(C_K_mNa))) / ((R(1.00000) + (R(0.124500) * cfg_exp(((((-R(0.100000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))))) + (R(0.0353000) * cfg_exp((((-y_V) * K(C_F)) / (K(C_R) * K(C_T)))))));
    R a_E_Na = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_Na_o) / y_Na_i)));
    R a_i_Na = ((((K(C_g_Na) * cfg_ipow<3>(y_m)) * y_h) * y_j) * (y_V - a_E_Na));
    R a_i_b_Na = (K(C_g_bNa) * (y_V - a_E_Na));
    R a_i_NaCa = ((K(C_K_NaCa) * (((cfg_exp((((K(C_gamma_NCX) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))) * cfg_ipow<3>(y_Na_i)) * K(C_Ca_o)) - (((cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))) * cfg_ipow<3>(K(C_Na_o))) * y_Ca_i) * K(C_alpha_NCX)))) / (((cfg_ipow<3>(K(C_Km_Nai)) + cfg_ipow<3>(K(C_Na_o))) * (K(C_Km_Ca) + K(C_Ca_o))) * (R(1.00000) + (K(C_K_sat) * cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T))))))));
    dydt[S_Na_i] = (((-(((a_i_Na + a_i_b_Na) + (R(3.00000) * a_i_NaK)) + (R(3.00000) * a_i_NaCa))) * K(C_Cm)) / (K(C_V_c) * K(C_F)));
    R a_E_K = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_K_o) / y_K_i)));
    R a_alpha_K1 = (R(0.100000) / (R(1.00000) + cfg_exp((R(0.0600000) * ((y_V - a_E_K) - R(200.000))))));
    R a_beta_K1 = (((R(3.00000) * cfg_exp((R(0.000200000) * ((y_V - a_E_K) + R(100.000))))) + (R(1.00000) * cfg_exp((R(0.100000) * ((y_V - a_E_K) - R(10.0000)))))) / (R(1.00000) + cfg_exp(((-R(0.500000)) * (y_V - a_E_K)))));
    R a_xK1_inf = (a_alpha_K1 / (a_alpha_K1 + a_beta_K1));
    R a_i_K1 = (((K(C_g_K1) * a_xK1_inf) * cfg_sqrt((K(C_K_o) / R(5.40000)))) * (y_V - a_E_K));
    R a_i_to = (((K(C_g_to) * y_r) * y_s) * (y_V - a_E_K));
    R a_i_Kr = ((((K(C_g_Kr) * cfg_sqrt((K(C_K_o) / R(5.40000)))) * y_Xr1) * y_Xr2) * (y_V - a_E_K));
    R a_E_Ks = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log(((K(C_K_o) + (K(C_P_kna) * K(C_Na_o))) / (y_K_i + (K(C_P_kna) * y_Na_i)))));
    R a_i_Ks = ((K(C_g_Ks) * cfg_ipow<2>(y_Xs)) * (y_V - a_E_Ks));
    R a_i_CaL = (((((((((K(C_g_CaL) * y_d) * y_f) * y_fCa) * R(4.00000)) * y_V) * cfg_ipow<2>(K(C_F))) / (K(C_R) * K(C_T))) * ((y_Ca_i * cfg_exp((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T))))) - (R(0.341000) * K(C_Ca_o)))) / cfg_expm1((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))));
    R a_E_Ca = ((((R(0.500000) * K(C_R)) * K(C_T)) / K(C_F)) * cfg_log((K(C_Ca_o) / y_Ca_i)));
    R a_i_b_Ca = (K(C_g_bCa) * (y_V - a_E_Ca));
    R a_i_p_K = ((K(C_g_pK) * (y_V - a_E_K)) / (R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(5.98000)))));
    R a_i_p_Ca = ((K(C_g_pCa) * y_Ca_i) / (y_Ca_i + K(C_K_pCa)));
    R a_Iion_cm = (((((((((((a_i_K1 + a_i_to) + a_i_Kr) + a_i_Ks) + a_i_CaL) + a_i_NaK) + a_i_Na) + a_i_b_Na) + a_i_NaCa) + a_i_b_Ca) + a_i_p_K) + a_i_p_Ca);
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    dydt[S_V] = R(0.0);
    if (SOLVE_VM) {
        dydt[S_V] = ((-a_Iion_cm) - a_Istim);
    }
    dydt[S_K_i] = (((-((((((a_i_K1 + a_i_to) + a_i_Kr) + a_i_Ks) + a_i_p_K) + a_Istim) - (R(2.00000) * a_i_NaK))) * K(C_Cm)) / (K(C_V_c) * K(C_F)));
    R a_i_rel = (((((K(C_a_rel) * cfg_ipow<2>(y_Ca_SR)) / (cfg_ipow<2>(K(C_b_rel)) + cfg_ipow<2>(y_Ca_SR))) + K(C_c_rel)) * y_d) * y_g);
    R a_i_up = (K(C_Vmax_up) / (R(1.00000) + (cfg_ipow<2>(K(C_K_up)) / cfg_ipow<2>(y_Ca_i))));
    R a_i_leak = (K(C_V_leak) * (y_Ca_SR - y_Ca_i));
    R a_ddt_Ca_i_total = ((((((-(((a_i_CaL + a_i_b_Ca) + a_i_p_Ca) - (R(2.00000) * a_i_NaCa))) / ((R(2.00000) * K(C_V_c)) * K(C_F))) * K(C_Cm)) + a_i_leak) - a_i_up) + a_i_rel);
    R a_f_JCa_i_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_c) * K(C_K_buf_c)) / cfg_ipow<2>((y_Ca_i + K(C_K_buf_c))))));
    dydt[S_Ca_i] = (a_ddt_Ca_i_total * a_f_JCa_i_free);
    R a_ddt_Ca_sr_total = ((K(C_V_c) / K(C_V_sr)) * (a_i_up - (a_i_rel + a_i_leak)));
    R a_f_JCa_sr_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_sr) * K(C_K_buf_sr)) / cfg_ipow<2>((y_Ca_SR + K(C_K_buf_sr))))));
    dydt[S_Ca_SR] = (a_ddt_Ca_sr_total * a_f_JCa_sr_free);
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
constexpr int NH = 29;
enum Hoisted { H_m_inf, H_tau_m, H_h_inf, H_tau_h, H_j_inf, H_tau_j, H_d_inf, H_tau_d, H_f_inf, H_tau_f, H_s_inf, H_tau_s, H_r_inf, H_tau_r, H_xr1_inf, H_tau_xr1, H_xr2_inf, H_tau_xr2, H_xs_inf, H_tau_xs };
template <class R, class KS>
__device__ __forceinline__ void hoist(R y_V, const KS& K, int tissue, R* H)
{
    (void)tissue; (void)K; (void)H; (void)y_V;
    R a_m_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp((((-R(56.8600)) - y_V) / R(9.03000))))));
    R a_alpha_m = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(5.00000)))));
    R a_beta_m = ((R(0.100000) / (R(1.00000) + cfg_exp(((y_V + R(35.0000)) / R(5.00000))))) + (R(0.100000) / (R(1.00000) + cfg_exp(((y_V - R(50.0000)) / R(200.000))))));
    R a_tau_m = ((R(1.00000) * a_alpha_m) * a_beta_m);
    R a_h_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    R a_alpha_h = ((y_V < (-R(40.0000))) ? (R(0.0570000) * cfg_exp(((-(y_V + R(80.0000))) / R(6.80000)))) : R(0.00000));
    R a_beta_h = ((y_V < (-R(40.0000))) ? ((R(2.70000) * cfg_exp((R(0.0790000) * y_V))) + (R(310000.) * cfg_exp((R(0.348500) * y_V)))) : (R(0.770000) / (R(0.130000) * (R(1.00000) + cfg_exp(((y_V + R(10.6600)) / (-R(11.1000))))))));
    R a_tau_h = (R(1.00000) / (a_alpha_h + a_beta_h));
    R a_j_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    R a_alpha_j = ((y_V < (-R(40.0000))) ? ((((((-R(25428.0)) * cfg_exp((R(0.244400) * y_V))) - (R(6.94800e-06) * cfg_exp(((-R(0.0439100)) * y_V)))) * (y_V + R(37.7800))) / R(1.00000)) / (R(1.00000) + cfg_exp((R(0.311000) * (y_V + R(79.2300)))))) : R(0.00000));
    R a_beta_j = ((y_V < (-R(40.0000))) ? ((R(0.0242400) * cfg_exp(((-R(0.0105200)) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.137800)) * (y_V + R(40.1400)))))) : ((R(0.600000) * cfg_exp((R(0.0570000) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.100000)) * (y_V + R(32.0000)))))));
    R a_tau_j = (R(1.00000) / (a_alpha_j + a_beta_j));
    R a_d_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(7.50000)))));
    R a_alpha_d = ((R(1.40000) / (R(1.00000) + cfg_exp((((-R(35.0000)) - y_V) / R(13.0000))))) + R(0.250000));
    R a_gama_fCa = (R(1.40000) / (R(1.00000) + cfg_exp(((y_V + R(5.00000)) / R(5.00000)))));
    R a_gamma_d = (R(1.00000) / (R(1.00000) + cfg_exp(((R(50.0000) - y_V) / R(20.0000)))));
    R a_tau_d = (((R(1.00000) * a_alpha_d) * a_gama_fCa) + a_gamma_d);
    R a_f_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(7.00000)))));
    R a_tau_f = (((R(1125.00) * cfg_exp(((-cfg_ipow<2>((y_V + R(27.0000)))) / R(240.000)))) + R(80.0000)) + (R(165.000) / (R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(10.0000))))));
    R a_s_inf = ((tissue == 1) ? (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(5.00000))))) : (R(1.10000) / (R(1.00000) + cfg_exp(((y_V + R(28.0000)) / R(6.00000))))));
    R a_tau_s = ((tissue == 1) ? (((R(85.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(45.0000)))) / R(320.000)))) + (R(5.00000) / (R(1.00000) + cfg_exp(((y_V - R(20.0000)) / R(5.00000)))))) + R(3.00000)) : ((R(1000.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(67.0000)))) / R(1000.000)))) + R(8.00000)));
    R a_r_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((R(20.0000) - y_V) / R(6.00000)))));
    R a_tau_r = ((R(9.50000) * cfg_exp(((-cfg_ipow<2>((y_V + R(40.0000)))) / R(1800.00)))) + R(0.800000));
    R a_xr1_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(26.0000)) - y_V) / R(7.00000)))));
    R a_alpha_xr1 = (R(450.000) / (R(1.00000) + cfg_exp((((-R(45.0000)) - y_V) / R(10.0000)))));
    R a_beta_xr1 = (R(6.00000) / (R(1.00000) + cfg_exp(((y_V + R(30.0000)) / R(11.5000)))));
    R a_tau_xr1 = ((R(1.00000) * a_alpha_xr1) * a_beta_xr1);
    R a_xr2_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(88.0000)) / R(24.0000)))));
    R a_alpha_xr2 = (R(3.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(20.0000)))));
    R a_beta_xr2 = (R(1.12000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    R a_tau_xr2 = ((R(1.00000) * a_alpha_xr2) * a_beta_xr2);
    R a_xs_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(14.0000)))));
    R a_alpha_xs = (R(1100.00) / cfg_sqrt((R(1.00000) + cfg_exp((((-R(10.0000)) - y_V) / R(6.00000))))));
    R a_beta_xs = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    R a_tau_xs = ((R(1.00000) * a_alpha_xs) * a_beta_xs);
    H[H_m_inf] = a_m_inf;
    H[H_tau_m] = cfg_hrcp(a_tau_m);
    H[H_h_inf] = a_h_inf;
    H[H_tau_h] = cfg_hrcp(a_tau_h);
    H[H_j_inf] = a_j_inf;
    H[H_tau_j] = cfg_hrcp(a_tau_j);
    H[H_d_inf] = a_d_inf;
    H[H_tau_d] = cfg_hrcp(a_tau_d);
    H[H_f_inf] = a_f_inf;
    H[H_tau_f] = cfg_hrcp(a_tau_f);
    H[H_s_inf] = a_s_inf;
    H[H_tau_s] = cfg_hrcp(a_tau_s);
    H[H_r_inf] = a_r_inf;
    H[H_tau_r] = cfg_hrcp(a_tau_r);
    H[H_xr1_inf] = a_xr1_inf;
    H[H_tau_xr1] = cfg_hrcp(a_tau_xr1);
    H[H_xr2_inf] = a_xr2_inf;
    H[H_tau_xr2] = cfg_hrcp(a_tau_xr2);
    H[H_xs_inf] = a_xs_inf;
    H[H_tau_xs] = cfg_hrcp(a_tau_xs);
    H[20] = cfg_hrcp(((R(1.00000) + (R(0.124500) * cfg_exp(((((-R(0.100000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))))) + (R(0.0353000) * cfg_exp((((-y_V) * K(C_F)) / (K(C_R) * K(C_T)))))));
    H[21] = cfg_hrcp((((cfg_ipow<3>(K(C_Km_Nai)) + cfg_ipow<3>(K(C_Na_o))) * (K(C_Km_Ca) + K(C_Ca_o))) * (R(1.00000) + (K(C_K_sat) * cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T))))))));
    H[22] = cfg_exp((((K(C_gamma_NCX) * y_V) * K(C_F)) / (K(C_R) * K(C_T))));
    H[23] = (cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))) * cfg_ipow<3>(K(C_Na_o)));
    H[24] = cfg_sqrt((K(C_K_o) / R(5.40000)));
    H[25] = (K(C_g_Kr) * cfg_sqrt((K(C_K_o) / R(5.40000))));
    H[26] = cfg_hrcp(cfg_expm1((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))));
    H[27] = cfg_exp((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T))));
    H[28] = cfg_hrcp((R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(5.98000)))));
}
template <class R, class YS, class KS, class HS>
__device__ __forceinline__ R rhs_tissue(double t, const YS& Y, const KS& K, const HS& H, R* dydt, int tissue, const CfgStimulus& stim)
{
    constexpr bool SOLVE_VM = false;
    (void)tissue; (void)stim; (void)t; (void)H;
    const R y_V = Y(S_V);
    const R y_K_i = Y(S_K_i);
    const R y_Na_i = Y(S_Na_i);
    const R y_Ca_i = Y(S_Ca_i);
    const R y_Xr1 = Y(S_Xr1);
    const R y_Xr2 = Y(S_Xr2);
    const R y_Xs = Y(S_Xs);
    const R y_m = Y(S_m);
    const R y_h = Y(S_h);
    const R y_j = Y(S_j);
    const R y_d = Y(S_d);
    const R y_f = Y(S_f);
    const R y_fCa = Y(S_fCa);
    const R y_s = Y(S_s);
    const R y_r = Y(S_r);
    const R y_Ca_SR = Y(S_Ca_SR);
    const R y_g = Y(S_g);
    dydt[S_m] = cfg_hdiv((H(H_m_inf) - y_m), H(H_tau_m));
    dydt[S_h] = cfg_hdiv((H(H_h_inf) - y_h), H(H_tau_h));
    dydt[S_j] = cfg_hdiv((H(H_j_inf) - y_j), H(H_tau_j));
    dydt[S_d] = cfg_hdiv((H(H_d_inf) - y_d), H(H_tau_d));
    dydt[S_f] = cfg_hdiv((H(H_f_inf) - y_f), H(H_tau_f));
    R a_alpha_fCa = (R(1.00000) / (R(1.00000) + cfg_ipow<8>((y_Ca_i / R(0.000325000)))));
    R a_beta_fCa = (R(0.100000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000500000)) / R(0.000100000)))));
    R a_beta_d = (R(0.200000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000750000)) / R(0.000800000)))));
    R a_fCa_inf = ((((a_alpha_fCa + a_beta_fCa) + a_beta_d) + R(0.230000)) / R(1.46000));
    R a_d_fCa = ((a_fCa_inf - y_fCa) / K(C_tau_fCa));
    dydt[S_fCa] = (((a_fCa_inf > y_fCa) && (y_V > (-R(60.0000)))) ? R(0.00000) : a_d_fCa);
    dydt[S_s] = cfg_hdiv((H(H_s_inf) - y_s), H(H_tau_s));
    dydt[S_r] = cfg_hdiv((H(H_r_inf) - y_r), H(H_tau_r));
    dydt[S_Xr1] = cfg_hdiv((H(H_xr1_inf) - y_Xr1), H(H_tau_xr1));
    dydt[S_Xr2] = cfg_hdiv((H(H_xr2_inf) - y_Xr2), H(H_tau_xr2));
    dydt[S_Xs] = cfg_hdiv((H(H_xs_inf) - y_Xs), H(H_tau_xs));
    R a_g_inf = ((y_Ca_i < R(0.000350000)) ? (R(1.00000) / (R(1.00000) + cfg_ipow<6>((y_Ca_i / R(0.000350000))))) : (R(1.00000) / (R(1.00000) + cfg_ipow<16>((y_Ca_i / R(0.000350000))))));
    R a_d_g = ((a_g_inf - y_g) / K(C_tau_g));
    dydt[S_g] = (((a_g_inf > y_g) && (y_V > (-R(60.0000)))) ? R(0.00000) : a_d_g);
    R a_i_NaK = cfg_hdiv(((((K(C_P_NaK) * K(C_K_o)) / (K(C_K_o) + K(C_K_mk))) * y_Na_i) / (y_Na_i + K(C_K_mNa))), H(20));
    R a_E_Na = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_Na_o) / y_Na_i)));
    R a_i_Na = ((((K(C_g_Na) * cfg_ipow<3>(y_m)) * y_h) * y_j) * (y_V - a_E_Na));
    R a_i_b_Na = (K(C_g_bNa) * (y_V - a_E_Na));
    R a_i_NaCa = cfg_hdiv((K(C_K_NaCa) * (((H(22) * cfg_ipow<3>(y_Na_i)) * K(C_Ca_o)) - ((H(23) * y_Ca_i) * K(C_alpha_NCX)))), H(21));
    dydt[S_Na_i] = (((-(((a_i_Na + a_i_b_Na) + (R(3.00000) * a_i_NaK)) + (R(3.00000) * a_i_NaCa))) * K(C_Cm)) / (K(C_V_c) * K(C_F)));
    R a_E_K = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_K_o) / y_K_i)));
    R a_alpha_K1 = (R(0.100000) / (R(1.00000) + cfg_exp((R(0.0600000) * ((y_V - a_E_K) - R(200.000))))));
    R a_beta_K1 = (((R(3.00000) * cfg_exp((R(0.000200000) * ((y_V - a_E_K) + R(100.000))))) + (R(1.00000) * cfg_exp((R(0.100000) * ((y_V - a_E_K) - R(10.0000)))))) / (R(1.00000) + cfg_exp(((-R(0.500000)) * (y_V - a_E_K)))));
    R a_xK1_inf = (a_alpha_K1 / (a_alpha_K1 + a_beta_K1));
    R a_i_K1 = (((K(C_g_K1) * a_xK1_inf) * H(24)) * (y_V - a_E_K));
    R a_i_to = (((K(C_g_to) * y_r) * y_s) * (y_V - a_E_K));
    R a_i_Kr = (((H(25) * y_Xr1) * y_Xr2) * (y_V - a_E_K));
    R a_E_Ks = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log(((K(C_K_o) + (K(C_P_kna) * K(C_Na_o))) / (y_K_i + (K(C_P_kna) * y_Na_i)))));
    R a_i_Ks = ((K(C_g_Ks) * cfg_ipow<2>(y_Xs)) * (y_V - a_E_Ks));
    R a_i_CaL = cfg_hdiv(((((((((K(C_g_CaL) * y_d) * y_f) * y_fCa) * R(4.00000)) * y_V) * cfg_ipow<2>(K(C_F))) / (K(C_R) * K(C_T))) * ((y_Ca_i * H(27)) - (R(0.341000) * K(C_Ca_o)))), H(26));
    R a_E_Ca = ((((R(0.500000) * K(C_R)) * K(C_T)) / K(C_F)) * cfg_log((K(C_Ca_o) / y_Ca_i)));
    R a_i_b_Ca = (K(C_g_bCa) * (y_V - a_E_Ca));
    R a_i_p_K = cfg_hdiv((K(C_g_pK) * (y_V - a_E_K)), H(28));
    R a_i_p_Ca = ((K(C_g_pCa) * y_Ca_i) / (y_Ca_i + K(C_K_pCa)));
    R a_Iion_cm = (((((((((((a_i_K1 + a_i_to) + a_i_Kr) + a_i_Ks) + a_i_CaL) + a_i_NaK) + a_i_Na) + a_i_b_Na) + a_i_NaCa) + a_i_b_Ca) + a_i_p_K) + a_i_p_Ca);
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    dydt[S_V] = R(0.0);
    if (SOLVE_VM) {
        dydt[S_V] = ((-a_Iion_cm) - a_Istim);
    }
    dydt[S_K_i] = (((-((((((a_i_K1 + a_i_to) + a_i_Kr) + a_i_Ks) + a_i_p_K) + a_Istim) - (R(2.00000) * a_i_NaK))) * K(C_Cm)) / (K(C_V_c) * K(C_F)));
    R a_i_rel = (((((K(C_a_rel) * cfg_ipow<2>(y_Ca_SR)) / (cfg_ipow<2>(K(C_b_rel)) + cfg_ipow<2>(y_Ca_SR))) + K(C_c_rel)) * y_d) * y_g);
    R a_i_up = (K(C_Vmax_up) / (R(1.00000) + (cfg_ipow<2>(K(C_K_up)) / cfg_ipow<2>(y_Ca_i))));
    R a_i_leak = (K(C_V_leak) * (y_Ca_SR - y_Ca_i));
    R a_ddt_Ca_i_total = ((((((-(((a_i_CaL + a_i_b_Ca) + a_i_p_Ca) - (R(2.00000) * a_i_NaCa))) / ((R(2.00000) * K(C_V_c)) * K(C_F))) * K(C_Cm)) + a_i_leak) - a_i_up) + a_i_rel);
    R a_f_JCa_i_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_c) * K(C_K_buf_c)) / cfg_ipow<2>((y_Ca_i + K(C_K_buf_c))))));
    dydt[S_Ca_i] = (a_ddt_Ca_i_total * a_f_JCa_i_free);
    R a_ddt_Ca_sr_total = ((K(C_V_c) / K(C_V_sr)) * (a_i_up - (a_i_rel + a_i_leak)));
    R a_f_JCa_sr_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_sr) * K(C_K_buf_sr)) / cfg_ipow<2>((y_Ca_SR + K(C_K_buf_sr))))));
    dydt[S_Ca_SR] = (a_ddt_Ca_sr_total * a_f_JCa_sr_free);
    return a_Iion_cm;
}

// Ionic current after the step (computeVariables at tEnd).
template <class R, bool SOLVE_VM, class YS, class KS>
__device__ __forceinline__ R iion(double t, const YS& Y, const KS& K, int tissue, const CfgStimulus& stim)
{
    (void)tissue; (void)stim; (void)t;
    R dydt[NS];
    const R y_V = Y(S_V);
    const R y_K_i = Y(S_K_i);
    const R y_Na_i = Y(S_Na_i);
    const R y_Ca_i = Y(S_Ca_i);
    const R y_Xr1 = Y(S_Xr1);
    const R y_Xr2 = Y(S_Xr2);
    const R y_Xs = Y(S_Xs);
    const R y_m = Y(S_m);
    const R y_h = Y(S_h);
    const R y_j = Y(S_j);
    const R y_d = Y(S_d);
    const R y_f = Y(S_f);
    const R y_fCa = Y(S_fCa);
    const R y_s = Y(S_s);
    const R y_r = Y(S_r);
    const R y_Ca_SR = Y(S_Ca_SR);
    const R y_g = Y(S_g);
    R a_f_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(7.00000)))));
    R a_tau_f = (((R(1125.00) * cfg_exp(((-cfg_ipow<2>((y_V + R(27.0000)))) / R(240.000)))) + R(80.0000)) + (R(165.000) / (R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(10.0000))))));
    R a_s_inf = ((tissue == 1) ? (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(5.00000))))) : (R(1.10000) / (R(1.00000) + cfg_exp(((y_V + R(28.0000)) / R(6.00000))))));
    R a_tau_s = ((tissue == 1) ? (((R(85.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(45.0000)))) / R(320.000)))) + (R(5.00000) / (R(1.00000) + cfg_exp(((y_V - R(20.0000)) / R(5.00000)))))) + R(3.00000)) : ((R(1000.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(67.0000)))) / R(1000.000)))) + R(8.00000)));
    R a_r_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((R(20.0000) - y_V) / R(6.00000)))));
    R a_tau_r = ((R(9.50000) * cfg_exp(((-cfg_ipow<2>((y_V + R(40.0000)))) / R(1800.00)))) + R(0.800000));
    R a_g_inf = ((y_Ca_i < R(0.000350000)) ? (R(1.00000) / (R(1.00000) + cfg_ipow<6>((y_Ca_i / R(0.000350000))))) : (R(1.00000) / (R(1.00000) + cfg_ipow<16>((y_Ca_i / R(0.000350000))))));
    R a_d_g = ((a_g_inf - y_g) / K(C_tau_g));
    R a_xr1_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(26.0000)) - y_V) / R(7.00000)))));
    R a_alpha_xr1 = (R(450.000) / (R(1.00000) + cfg_exp((((-R(45.0000)) - y_V) / R(10.0000)))));
    R a_beta_xr1 = (R(6.00000) / (R(1.00000) + cfg_exp(((y_V + R(30.0000)) / R(11.5000)))));
    R a_tau_xr1 = ((R(1.00000) * a_alpha_xr1) * a_beta_xr1);
    R a_xr2_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(88.0000)) / R(24.0000)))));
    R a_alpha_xr2 = (R(3.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(20.0000)))));
    R a_beta_xr2 = (R(1.12000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    R a_tau_xr2 = ((R(1.00000) * a_alpha_xr2) * a_beta_xr2);
    R a_xs_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(14.0000)))));
    R a_alpha_xs = (R(1100.00) / cfg_sqrt((R(1.00000) + cfg_exp((((-R(10.0000)) - y_V) / R(6.00000))))));
    R a_beta_xs = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    R a_tau_xs = ((R(1.00000) * a_alpha_xs) * a_beta_xs);
    R a_m_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp((((-R(56.8600)) - y_V) / R(9.03000))))));
    R a_alpha_m = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(5.00000)))));
    R a_beta_m = ((R(0.100000) / (R(1.00000) + cfg_exp(((y_V + R(35.0000)) / R(5.00000))))) + (R(0.100000) / (R(1.00000) + cfg_exp(((y_V - R(50.0000)) / R(200.000))))));
    R a_tau_m = ((R(1.00000) * a_alpha_m) * a_beta_m);
    R a_h_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    R a_alpha_h = ((y_V < (-R(40.0000))) ? (R(0.0570000) * cfg_exp(((-(y_V + R(80.0000))) / R(6.80000)))) : R(0.00000));
    R a_beta_h = ((y_V < (-R(40.0000))) ? ((R(2.70000) * cfg_exp((R(0.0790000) * y_V))) + (R(310000.) * cfg_exp((R(0.348500) * y_V)))) : (R(0.770000) / (R(0.130000) * (R(1.00000) + cfg_exp(((y_V + R(10.6600)) / (-R(11.1000))))))));
    R a_tau_h = (R(1.00000) / (a_alpha_h + a_beta_h));
    R a_j_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    R a_alpha_j = ((y_V < (-R(40.0000))) ? ((((((-R(25428.0)) * cfg_exp((R(0.244400) * y_V))) - (R(6.94800e-06) * cfg_exp(((-R(0.0439100)) * y_V)))) * (y_V + R(37.7800))) / R(1.00000)) / (R(1.00000) + cfg_exp((R(0.311000) * (y_V + R(79.2300)))))) : R(0.00000));
    R a_beta_j = ((y_V < (-R(40.0000))) ? ((R(0.0242400) * cfg_exp(((-R(0.0105200)) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.137800)) * (y_V + R(40.1400)))))) : ((R(0.600000) * cfg_exp((R(0.0570000) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.100000)) * (y_V + R(32.0000)))))));
    R a_tau_j = (R(1.00000) / (a_alpha_j + a_beta_j));
    R a_d_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(7.50000)))));
    R a_alpha_d = ((R(1.40000) / (R(1.00000) + cfg_exp((((-R(35.0000)) - y_V) / R(13.0000))))) + R(0.250000));
    R a_gama_fCa = (R(1.40000) / (R(1.00000) + cfg_exp(((y_V + R(5.00000)) / R(5.00000)))));
    R a_gamma_d = (R(1.00000) / (R(1.00000) + cfg_exp(((R(50.0000) - y_V) / R(20.0000)))));
    R a_tau_d = (((R(1.00000) * a_alpha_d) * a_gama_fCa) + a_gamma_d);
    R a_alpha_fCa = (R(1.00000) / (R(1.00000) + cfg_ipow<8>((y_Ca_i / R(0.000325000)))));
    R a_beta_fCa = (R(0.100000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000500000)) / R(0.000100000)))));
    R a_beta_d = (R(0.200000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000750000)) / R(0.000800000)))));
    R a_fCa_inf = ((((a_alpha_fCa + a_beta_fCa) + a_beta_d) + R(0.230000)) / R(1.46000));
    R a_d_fCa = ((a_fCa_inf - y_fCa) / K(C_tau_fCa));
    R a_i_NaK = (((((K(C_P_NaK) * K(C_K_o)) / (K(C_K_o) + K(C_K_mk))) * y_Na_i) / (y_Na_i + K(C_K_mNa))) / ((R(1.00000) + (R(0.124500) * cfg_exp(((((-R(0.100000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))))) + (R(0.0353000) * cfg_exp((((-y_V) * K(C_F)) / (K(C_R) * K(C_T)))))));
    R a_E_Na = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_Na_o) / y_Na_i)));
    R a_i_Na = ((((K(C_g_Na) * cfg_ipow<3>(y_m)) * y_h) * y_j) * (y_V - a_E_Na));
    R a_i_b_Na = (K(C_g_bNa) * (y_V - a_E_Na));
    R a_i_NaCa = ((K(C_K_NaCa) * (((cfg_exp((((K(C_gamma_NCX) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))) * cfg_ipow<3>(y_Na_i)) * K(C_Ca_o)) - (((cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))) * cfg_ipow<3>(K(C_Na_o))) * y_Ca_i) * K(C_alpha_NCX)))) / (((cfg_ipow<3>(K(C_Km_Nai)) + cfg_ipow<3>(K(C_Na_o))) * (K(C_Km_Ca) + K(C_Ca_o))) * (R(1.00000) + (K(C_K_sat) * cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T))))))));
    R a_E_K = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_K_o) / y_K_i)));
    R a_alpha_K1 = (R(0.100000) / (R(1.00000) + cfg_exp((R(0.0600000) * ((y_V - a_E_K) - R(200.000))))));
    R a_beta_K1 = (((R(3.00000) * cfg_exp((R(0.000200000) * ((y_V - a_E_K) + R(100.000))))) + (R(1.00000) * cfg_exp((R(0.100000) * ((y_V - a_E_K) - R(10.0000)))))) / (R(1.00000) + cfg_exp(((-R(0.500000)) * (y_V - a_E_K)))));
    R a_xK1_inf = (a_alpha_K1 / (a_alpha_K1 + a_beta_K1));
    R a_i_K1 = (((K(C_g_K1) * a_xK1_inf) * cfg_sqrt((K(C_K_o) / R(5.40000)))) * (y_V - a_E_K));
    R a_i_to = (((K(C_g_to) * y_r) * y_s) * (y_V - a_E_K));
    R a_i_Kr = ((((K(C_g_Kr) * cfg_sqrt((K(C_K_o) / R(5.40000)))) * y_Xr1) * y_Xr2) * (y_V - a_E_K));
    R a_E_Ks = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log(((K(C_K_o) + (K(C_P_kna) * K(C_Na_o))) / (y_K_i + (K(C_P_kna) * y_Na_i)))));
    R a_i_Ks = ((K(C_g_Ks) * cfg_ipow<2>(y_Xs)) * (y_V - a_E_Ks));
    R a_i_CaL = (((((((((K(C_g_CaL) * y_d) * y_f) * y_fCa) * R(4.00000)) * y_V) * cfg_ipow<2>(K(C_F))) / (K(C_R) * K(C_T))) * ((y_Ca_i * cfg_exp((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T))))) - (R(0.341000) * K(C_Ca_o)))) / cfg_expm1((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))));
    R a_E_Ca = ((((R(0.500000) * K(C_R)) * K(C_T)) / K(C_F)) * cfg_log((K(C_Ca_o) / y_Ca_i)));
    R a_i_b_Ca = (K(C_g_bCa) * (y_V - a_E_Ca));
    R a_i_p_K = ((K(C_g_pK) * (y_V - a_E_K)) / (R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(5.98000)))));
    R a_i_p_Ca = ((K(C_g_pCa) * y_Ca_i) / (y_Ca_i + K(C_K_pCa)));
    R a_i_rel = (((((K(C_a_rel) * cfg_ipow<2>(y_Ca_SR)) / (cfg_ipow<2>(K(C_b_rel)) + cfg_ipow<2>(y_Ca_SR))) + K(C_c_rel)) * y_d) * y_g);
    R a_i_up = (K(C_Vmax_up) / (R(1.00000) + (cfg_ipow<2>(K(C_K_up)) / cfg_ipow<2>(y_Ca_i))));
    R a_i_leak = (K(C_V_leak) * (y_Ca_SR - y_Ca_i));
    R a_ddt_Ca_i_total = ((((((-(((a_i_CaL + a_i_b_Ca) + a_i_p_Ca) - (R(2.00000) * a_i_NaCa))) / ((R(2.00000) * K(C_V_c)) * K(C_F))) * K(C_Cm)) + a_i_leak) - a_i_up) + a_i_rel);
    R a_f_JCa_i_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_c) * K(C_K_buf_c)) / cfg_ipow<2>((y_Ca_i + K(C_K_buf_c))))));
    R a_ddt_Ca_sr_total = ((K(C_V_c) / K(C_V_sr)) * (a_i_up - (a_i_rel + a_i_leak)));
    R a_f_JCa_sr_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_sr) * K(C_K_buf_sr)) / cfg_ipow<2>((y_Ca_SR + K(C_K_buf_sr))))));
    R a_Iion_cm = (((((((((((a_i_K1 + a_i_to) + a_i_Kr) + a_i_Ks) + a_i_CaL) + a_i_NaK) + a_i_Na) + a_i_b_Na) + a_i_NaCa) + a_i_b_Ca) + a_i_p_K) + a_i_p_Ca);
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    a_m_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp((((-R(56.8600)) - y_V) / R(9.03000))))));
    a_alpha_m = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(5.00000)))));
    a_beta_m = ((R(0.100000) / (R(1.00000) + cfg_exp(((y_V + R(35.0000)) / R(5.00000))))) + (R(0.100000) / (R(1.00000) + cfg_exp(((y_V - R(50.0000)) / R(200.000))))));
    a_tau_m = ((R(1.00000) * a_alpha_m) * a_beta_m);
    dydt[S_m] = ((a_m_inf - y_m) / a_tau_m);
    a_h_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    a_alpha_h = ((y_V < (-R(40.0000))) ? (R(0.0570000) * cfg_exp(((-(y_V + R(80.0000))) / R(6.80000)))) : R(0.00000));
    a_beta_h = ((y_V < (-R(40.0000))) ? ((R(2.70000) * cfg_exp((R(0.0790000) * y_V))) + (R(310000.) * cfg_exp((R(0.348500) * y_V)))) : (R(0.770000) / (R(0.130000) * (R(1.00000) + cfg_exp(((y_V + R(10.6600)) / (-R(11.1000))))))));
    a_tau_h = (R(1.00000) / (a_alpha_h + a_beta_h));
    dydt[S_h] = ((a_h_inf - y_h) / a_tau_h);
    a_j_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    a_alpha_j = ((y_V < (-R(40.0000))) ? ((((((-R(25428.0)) * cfg_exp((R(0.244400) * y_V))) - (R(6.94800e-06) * cfg_exp(((-R(0.0439100)) * y_V)))) * (y_V + R(37.7800))) / R(1.00000)) / (R(1.00000) + cfg_exp((R(0.311000) * (y_V + R(79.2300)))))) : R(0.00000));
    a_beta_j = ((y_V < (-R(40.0000))) ? ((R(0.0242400) * cfg_exp(((-R(0.0105200)) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.137800)) * (y_V + R(40.1400)))))) : ((R(0.600000) * cfg_exp((R(0.0570000) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.100000)) * (y_V + R(32.0000)))))));
    a_tau_j = (R(1.00000) / (a_alpha_j + a_beta_j));
    dydt[S_j] = ((a_j_inf - y_j) / a_tau_j);
    a_d_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(7.50000)))));
    a_alpha_d = ((R(1.40000) / (R(1.00000) + cfg_exp((((-R(35.0000)) - y_V) / R(13.0000))))) + R(0.250000));
    a_gama_fCa = (R(1.40000) / (R(1.00000) + cfg_exp(((y_V + R(5.00000)) / R(5.00000)))));
    a_gamma_d = (R(1.00000) / (R(1.00000) + cfg_exp(((R(50.0000) - y_V) / R(20.0000)))));
    a_tau_d = (((R(1.00000) * a_alpha_d) * a_gama_fCa) + a_gamma_d);
    dydt[S_d] = ((a_d_inf - y_d) / a_tau_d);
    a_f_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(7.00000)))));
    a_tau_f = (((R(1125.00) * cfg_exp(((-cfg_ipow<2>((y_V + R(27.0000)))) / R(240.000)))) + R(80.0000)) + (R(165.000) / (R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(10.0000))))));
    dydt[S_f] = ((a_f_inf - y_f) / a_tau_f);
    a_alpha_fCa = (R(1.00000) / (R(1.00000) + cfg_ipow<8>((y_Ca_i / R(0.000325000)))));
    a_beta_fCa = (R(0.100000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000500000)) / R(0.000100000)))));
    a_beta_d = (R(0.200000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000750000)) / R(0.000800000)))));
    a_fCa_inf = ((((a_alpha_fCa + a_beta_fCa) + a_beta_d) + R(0.230000)) / R(1.46000));
    a_d_fCa = ((a_fCa_inf - y_fCa) / K(C_tau_fCa));
    dydt[S_fCa] = (((a_fCa_inf > y_fCa) && (y_V > (-R(60.0000)))) ? R(0.00000) : a_d_fCa);
    a_s_inf = ((tissue == 1) ? (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(5.00000))))) : (R(1.10000) / (R(1.00000) + cfg_exp(((y_V + R(28.0000)) / R(6.00000))))));
    a_tau_s = ((tissue == 1) ? (((R(85.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(45.0000)))) / R(320.000)))) + (R(5.00000) / (R(1.00000) + cfg_exp(((y_V - R(20.0000)) / R(5.00000)))))) + R(3.00000)) : ((R(1000.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(67.0000)))) / R(1000.000)))) + R(8.00000)));
    dydt[S_s] = ((a_s_inf - y_s) / a_tau_s);
    a_r_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((R(20.0000) - y_V) / R(6.00000)))));
    a_tau_r = ((R(9.50000) * cfg_exp(((-cfg_ipow<2>((y_V + R(40.0000)))) / R(1800.00)))) + R(0.800000));
    dydt[S_r] = ((a_r_inf - y_r) / a_tau_r);
    a_xr1_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(26.0000)) - y_V) / R(7.00000)))));
    a_alpha_xr1 = (R(450.000) / (R(1.00000) + cfg_exp((((-R(45.0000)) - y_V) / R(10.0000)))));
    a_beta_xr1 = (R(6.00000) / (R(1.00000) + cfg_exp(((y_V + R(30.0000)) / R(11.5000)))));
    a_tau_xr1 = ((R(1.00000) * a_alpha_xr1) * a_beta_xr1);
    dydt[S_Xr1] = ((a_xr1_inf - y_Xr1) / a_tau_xr1);
    a_xr2_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(88.0000)) / R(24.0000)))));
    a_alpha_xr2 = (R(3.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(20.0000)))));
    a_beta_xr2 = (R(1.12000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    a_tau_xr2 = ((R(1.00000) * a_alpha_xr2) * a_beta_xr2);
    dydt[S_Xr2] = ((a_xr2_inf - y_Xr2) / a_tau_xr2);
    a_xs_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(14.0000)))));
    a_alpha_xs = (R(1100.00) / cfg_sqrt((R(1.00000) + cfg_exp((((-R(10.0000)) - y_V) / R(6.00000))))));
    a_beta_xs = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    a_tau_xs = ((R(1.00000) * a_alpha_xs) * a_beta_xs);
    dydt[S_Xs] = ((a_xs_inf - y_Xs) / a_tau_xs);
    a_g_inf = ((y_Ca_i < R(0.000350000)) ? (R(1.00000) / (R(1.00000) + cfg_ipow<6>((y_Ca_i / R(0.000350000))))) : (R(1.00000) / (R(1.00000) + cfg_ipow<16>((y_Ca_i / R(0.000350000))))));
    a_d_g = ((a_g_inf - y_g) / K(C_tau_g));
    dydt[S_g] = (((a_g_inf > y_g) && (y_V > (-R(60.0000)))) ? R(0.00000) : a_d_g);
    a_i_NaK = (((((K(C_P_NaK) * K(C_K_o)) / (K(C_K_o) + K(C_K_mk))) * y_Na_i) / (y_Na_i + K(C_K_mNa))) / ((R(1.00000) + (R(0.124500) * cfg_exp(((((-R(0.100000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))))) + (R(0.0353000) * cfg_exp((((-y_V) * K(C_F)) / (K(C_R) * K(C_T)))))));
    a_E_Na = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_Na_o) / y_Na_i)));
    a_i_Na = ((((K(C_g_Na) * cfg_ipow<3>(y_m)) * y_h) * y_j) * (y_V - a_E_Na));
    a_i_b_Na = (K(C_g_bNa) * (y_V - a_E_Na));
    a_i_NaCa = ((K(C_K_NaCa) * (((cfg_exp((((K(C_gamma_NCX) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))) * cfg_ipow<3>(y_Na_i)) * K(C_Ca_o)) - (((cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))) * cfg_ipow<3>(K(C_Na_o))) * y_Ca_i) * K(C_alpha_NCX)))) / (((cfg_ipow<3>(K(C_Km_Nai)) + cfg_ipow<3>(K(C_Na_o))) * (K(C_Km_Ca) + K(C_Ca_o))) * (R(1.00000) + (K(C_K_sat) * cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T))))))));
    dydt[S_Na_i] = (((-(((a_i_Na + a_i_b_Na) + (R(3.00000) * a_i_NaK)) + (R(3.00000) * a_i_NaCa))) * K(C_Cm)) / (K(C_V_c) * K(C_F)));
    a_E_K = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_K_o) / y_K_i)));
    a_alpha_K1 = (R(0.100000) / (R(1.00000) + cfg_exp((R(0.0600000) * ((y_V - a_E_K) - R(200.000))))));
    a_beta_K1 = (((R(3.00000) * cfg_exp((R(0.000200000) * ((y_V - a_E_K) + R(100.000))))) + (R(1.00000) * cfg_exp((R(0.100000) * ((y_V - a_E_K) - R(10.0000)))))) / (R(1.00000) + cfg_exp(((-R(0.500000)) * (y_V - a_E_K)))));
    a_xK1_inf = (a_alpha_K1 / (a_alpha_K1 + a_beta_K1));
    a_i_K1 = (((K(C_g_K1) * a_xK1_inf) * cfg_sqrt((K(C_K_o) / R(5.40000)))) * (y_V - a_E_K));
    a_i_to = (((K(C_g_to) * y_r) * y_s) * (y_V - a_E_K));
    a_i_Kr = ((((K(C_g_Kr) * cfg_sqrt((K(C_K_o) / R(5.40000)))) * y_Xr1) * y_Xr2) * (y_V - a_E_K));
    a_E_Ks = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log(((K(C_K_o) + (K(C_P_kna) * K(C_Na_o))) / (y_K_i + (K(C_P_kna) * y_Na_i)))));
    a_i_Ks = ((K(C_g_Ks) * cfg_ipow<2>(y_Xs)) * (y_V - a_E_Ks));
    a_i_CaL = (((((((((K(C_g_CaL) * y_d) * y_f) * y_fCa) * R(4.00000)) * y_V) * cfg_ipow<2>(K(C_F))) / (K(C_R) * K(C_T))) * ((y_Ca_i * cfg_exp((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T))))) - (R(0.341000) * K(C_Ca_o)))) / cfg_expm1((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))));
    a_E_Ca = ((((R(0.500000) * K(C_R)) * K(C_T)) / K(C_F)) * cfg_log((K(C_Ca_o) / y_Ca_i)));
    a_i_b_Ca = (K(C_g_bCa) * (y_V - a_E_Ca));
    a_i_p_K = ((K(C_g_pK) * (y_V - a_E_K)) / (R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(5.98000)))));
    a_i_p_Ca = ((K(C_g_pCa) * y_Ca_i) / (y_Ca_i + K(C_K_pCa)));
    a_Iion_cm = (((((((((((a_i_K1 + a_i_to) + a_i_Kr) + a_i_Ks) + a_i_CaL) + a_i_NaK) + a_i_Na) + a_i_b_Na) + a_i_NaCa) + a_i_b_Ca) + a_i_p_K) + a_i_p_Ca);
    a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    dydt[S_V] = R(0.0);
    if (SOLVE_VM) {
        dydt[S_V] = ((-a_Iion_cm) - a_Istim);
    }
    dydt[S_K_i] = (((-((((((a_i_K1 + a_i_to) + a_i_Kr) + a_i_Ks) + a_i_p_K) + a_Istim) - (R(2.00000) * a_i_NaK))) * K(C_Cm)) / (K(C_V_c) * K(C_F)));
    a_i_rel = (((((K(C_a_rel) * cfg_ipow<2>(y_Ca_SR)) / (cfg_ipow<2>(K(C_b_rel)) + cfg_ipow<2>(y_Ca_SR))) + K(C_c_rel)) * y_d) * y_g);
    a_i_up = (K(C_Vmax_up) / (R(1.00000) + (cfg_ipow<2>(K(C_K_up)) / cfg_ipow<2>(y_Ca_i))));
    a_i_leak = (K(C_V_leak) * (y_Ca_SR - y_Ca_i));
    a_ddt_Ca_i_total = ((((((-(((a_i_CaL + a_i_b_Ca) + a_i_p_Ca) - (R(2.00000) * a_i_NaCa))) / ((R(2.00000) * K(C_V_c)) * K(C_F))) * K(C_Cm)) + a_i_leak) - a_i_up) + a_i_rel);
    a_f_JCa_i_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_c) * K(C_K_buf_c)) / cfg_ipow<2>((y_Ca_i + K(C_K_buf_c))))));
    dydt[S_Ca_i] = (a_ddt_Ca_i_total * a_f_JCa_i_free);
    a_ddt_Ca_sr_total = ((K(C_V_c) / K(C_V_sr)) * (a_i_up - (a_i_rel + a_i_leak)));
    a_f_JCa_sr_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_sr) * K(C_K_buf_sr)) / cfg_ipow<2>((y_Ca_SR + K(C_K_buf_sr))))));
    dydt[S_Ca_SR] = (a_ddt_Ca_sr_total * a_f_JCa_sr_free);
    (void)dydt;
    return a_Iion_cm;
}

// computeVariables with every algebraic stored: A[k] is ALGEBRAIC[k] (0 for
// the ones the body does not assign), dydt the RATES it assigns.
template <class R, bool SOLVE_VM, class YS, class KS>
__device__ __forceinline__ void variables_all(double t, const YS& Y, const KS& K, R* A, R* dydt, int tissue, const CfgStimulus& stim)
{
    (void)tissue; (void)stim; (void)t;
    const R y_V = Y(S_V);
    const R y_K_i = Y(S_K_i);
    const R y_Na_i = Y(S_Na_i);
    const R y_Ca_i = Y(S_Ca_i);
    const R y_Xr1 = Y(S_Xr1);
    const R y_Xr2 = Y(S_Xr2);
    const R y_Xs = Y(S_Xs);
    const R y_m = Y(S_m);
    const R y_h = Y(S_h);
    const R y_j = Y(S_j);
    const R y_d = Y(S_d);
    const R y_f = Y(S_f);
    const R y_fCa = Y(S_fCa);
    const R y_s = Y(S_s);
    const R y_r = Y(S_r);
    const R y_Ca_SR = Y(S_Ca_SR);
    const R y_g = Y(S_g);
    R a_f_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(7.00000)))));
    R a_tau_f = (((R(1125.00) * cfg_exp(((-cfg_ipow<2>((y_V + R(27.0000)))) / R(240.000)))) + R(80.0000)) + (R(165.000) / (R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(10.0000))))));
    R a_s_inf = ((tissue == 1) ? (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(20.0000)) / R(5.00000))))) : (R(1.10000) / (R(1.00000) + cfg_exp(((y_V + R(28.0000)) / R(6.00000))))));
    R a_tau_s = ((tissue == 1) ? (((R(85.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(45.0000)))) / R(320.000)))) + (R(5.00000) / (R(1.00000) + cfg_exp(((y_V - R(20.0000)) / R(5.00000)))))) + R(3.00000)) : ((R(1000.0000) * cfg_exp(((-cfg_ipow<2>((y_V + R(67.0000)))) / R(1000.000)))) + R(8.00000)));
    R a_r_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((R(20.0000) - y_V) / R(6.00000)))));
    R a_tau_r = ((R(9.50000) * cfg_exp(((-cfg_ipow<2>((y_V + R(40.0000)))) / R(1800.00)))) + R(0.800000));
    R a_g_inf = ((y_Ca_i < R(0.000350000)) ? (R(1.00000) / (R(1.00000) + cfg_ipow<6>((y_Ca_i / R(0.000350000))))) : (R(1.00000) / (R(1.00000) + cfg_ipow<16>((y_Ca_i / R(0.000350000))))));
    R a_d_g = ((a_g_inf - y_g) / K(C_tau_g));
    R a_xr1_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(26.0000)) - y_V) / R(7.00000)))));
    R a_alpha_xr1 = (R(450.000) / (R(1.00000) + cfg_exp((((-R(45.0000)) - y_V) / R(10.0000)))));
    R a_beta_xr1 = (R(6.00000) / (R(1.00000) + cfg_exp(((y_V + R(30.0000)) / R(11.5000)))));
    R a_tau_xr1 = ((R(1.00000) * a_alpha_xr1) * a_beta_xr1);
    R a_xr2_inf = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V + R(88.0000)) / R(24.0000)))));
    R a_alpha_xr2 = (R(3.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(20.0000)))));
    R a_beta_xr2 = (R(1.12000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    R a_tau_xr2 = ((R(1.00000) * a_alpha_xr2) * a_beta_xr2);
    R a_xs_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(14.0000)))));
    R a_alpha_xs = (R(1100.00) / cfg_sqrt((R(1.00000) + cfg_exp((((-R(10.0000)) - y_V) / R(6.00000))))));
    R a_beta_xs = (R(1.00000) / (R(1.00000) + cfg_exp(((y_V - R(60.0000)) / R(20.0000)))));
    R a_tau_xs = ((R(1.00000) * a_alpha_xs) * a_beta_xs);
    R a_m_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp((((-R(56.8600)) - y_V) / R(9.03000))))));
    R a_alpha_m = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(60.0000)) - y_V) / R(5.00000)))));
    R a_beta_m = ((R(0.100000) / (R(1.00000) + cfg_exp(((y_V + R(35.0000)) / R(5.00000))))) + (R(0.100000) / (R(1.00000) + cfg_exp(((y_V - R(50.0000)) / R(200.000))))));
    R a_tau_m = ((R(1.00000) * a_alpha_m) * a_beta_m);
    R a_h_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    R a_alpha_h = ((y_V < (-R(40.0000))) ? (R(0.0570000) * cfg_exp(((-(y_V + R(80.0000))) / R(6.80000)))) : R(0.00000));
    R a_beta_h = ((y_V < (-R(40.0000))) ? ((R(2.70000) * cfg_exp((R(0.0790000) * y_V))) + (R(310000.) * cfg_exp((R(0.348500) * y_V)))) : (R(0.770000) / (R(0.130000) * (R(1.00000) + cfg_exp(((y_V + R(10.6600)) / (-R(11.1000))))))));
    R a_tau_h = (R(1.00000) / (a_alpha_h + a_beta_h));
    R a_j_inf = (R(1.00000) / cfg_ipow<2>((R(1.00000) + cfg_exp(((y_V + R(71.5500)) / R(7.43000))))));
    R a_alpha_j = ((y_V < (-R(40.0000))) ? ((((((-R(25428.0)) * cfg_exp((R(0.244400) * y_V))) - (R(6.94800e-06) * cfg_exp(((-R(0.0439100)) * y_V)))) * (y_V + R(37.7800))) / R(1.00000)) / (R(1.00000) + cfg_exp((R(0.311000) * (y_V + R(79.2300)))))) : R(0.00000));
    R a_beta_j = ((y_V < (-R(40.0000))) ? ((R(0.0242400) * cfg_exp(((-R(0.0105200)) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.137800)) * (y_V + R(40.1400)))))) : ((R(0.600000) * cfg_exp((R(0.0570000) * y_V))) / (R(1.00000) + cfg_exp(((-R(0.100000)) * (y_V + R(32.0000)))))));
    R a_tau_j = (R(1.00000) / (a_alpha_j + a_beta_j));
    R a_d_inf = (R(1.00000) / (R(1.00000) + cfg_exp((((-R(5.00000)) - y_V) / R(7.50000)))));
    R a_alpha_d = ((R(1.40000) / (R(1.00000) + cfg_exp((((-R(35.0000)) - y_V) / R(13.0000))))) + R(0.250000));
    R a_gama_fCa = (R(1.40000) / (R(1.00000) + cfg_exp(((y_V + R(5.00000)) / R(5.00000)))));
    R a_gamma_d = (R(1.00000) / (R(1.00000) + cfg_exp(((R(50.0000) - y_V) / R(20.0000)))));
    R a_tau_d = (((R(1.00000) * a_alpha_d) * a_gama_fCa) + a_gamma_d);
    R a_alpha_fCa = (R(1.00000) / (R(1.00000) + cfg_ipow<8>((y_Ca_i / R(0.000325000)))));
    R a_beta_fCa = (R(0.100000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000500000)) / R(0.000100000)))));
    R a_beta_d = (R(0.200000) / (R(1.00000) + cfg_exp(((y_Ca_i - R(0.000750000)) / R(0.000800000)))));
    R a_fCa_inf = ((((a_alpha_fCa + a_beta_fCa) + a_beta_d) + R(0.230000)) / R(1.46000));
    R a_d_fCa = ((a_fCa_inf - y_fCa) / K(C_tau_fCa));
    R a_i_NaK = (((((K(C_P_NaK) * K(C_K_o)) / (K(C_K_o) + K(C_K_mk))) * y_Na_i) / (y_Na_i + K(C_K_mNa))) / ((R(1.00000) + (R(0.124500) * cfg_exp(((((-R(0.100000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))))) + (R(0.0353000) * cfg_exp((((-y_V) * K(C_F)) / (K(C_R) * K(C_T)))))));
    R a_E_Na = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_Na_o) / y_Na_i)));
    R a_i_Na = ((((K(C_g_Na) * cfg_ipow<3>(y_m)) * y_h) * y_j) * (y_V - a_E_Na));
    R a_i_b_Na = (K(C_g_bNa) * (y_V - a_E_Na));
    R a_i_NaCa = ((K(C_K_NaCa) * (((cfg_exp((((K(C_gamma_NCX) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))) * cfg_ipow<3>(y_Na_i)) * K(C_Ca_o)) - (((cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))) * cfg_ipow<3>(K(C_Na_o))) * y_Ca_i) * K(C_alpha_NCX)))) / (((cfg_ipow<3>(K(C_Km_Nai)) + cfg_ipow<3>(K(C_Na_o))) * (K(C_Km_Ca) + K(C_Ca_o))) * (R(1.00000) + (K(C_K_sat) * cfg_exp(((((K(C_gamma_NCX) - R(1.00000)) * y_V) * K(C_F)) / (K(C_R) * K(C_T))))))));
    R a_E_K = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log((K(C_K_o) / y_K_i)));
    R a_alpha_K1 = (R(0.100000) / (R(1.00000) + cfg_exp((R(0.0600000) * ((y_V - a_E_K) - R(200.000))))));
    R a_beta_K1 = (((R(3.00000) * cfg_exp((R(0.000200000) * ((y_V - a_E_K) + R(100.000))))) + (R(1.00000) * cfg_exp((R(0.100000) * ((y_V - a_E_K) - R(10.0000)))))) / (R(1.00000) + cfg_exp(((-R(0.500000)) * (y_V - a_E_K)))));
    R a_xK1_inf = (a_alpha_K1 / (a_alpha_K1 + a_beta_K1));
    R a_i_K1 = (((K(C_g_K1) * a_xK1_inf) * cfg_sqrt((K(C_K_o) / R(5.40000)))) * (y_V - a_E_K));
    R a_i_to = (((K(C_g_to) * y_r) * y_s) * (y_V - a_E_K));
    R a_i_Kr = ((((K(C_g_Kr) * cfg_sqrt((K(C_K_o) / R(5.40000)))) * y_Xr1) * y_Xr2) * (y_V - a_E_K));
    R a_E_Ks = (((K(C_R) * K(C_T)) / K(C_F)) * cfg_log(((K(C_K_o) + (K(C_P_kna) * K(C_Na_o))) / (y_K_i + (K(C_P_kna) * y_Na_i)))));
    R a_i_Ks = ((K(C_g_Ks) * cfg_ipow<2>(y_Xs)) * (y_V - a_E_Ks));
    R a_i_CaL = (((((((((K(C_g_CaL) * y_d) * y_f) * y_fCa) * R(4.00000)) * y_V) * cfg_ipow<2>(K(C_F))) / (K(C_R) * K(C_T))) * ((y_Ca_i * cfg_exp((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T))))) - (R(0.341000) * K(C_Ca_o)))) / cfg_expm1((((R(2.00000) * y_V) * K(C_F)) / (K(C_R) * K(C_T)))));
    R a_E_Ca = ((((R(0.500000) * K(C_R)) * K(C_T)) / K(C_F)) * cfg_log((K(C_Ca_o) / y_Ca_i)));
    R a_i_b_Ca = (K(C_g_bCa) * (y_V - a_E_Ca));
    R a_i_p_K = ((K(C_g_pK) * (y_V - a_E_K)) / (R(1.00000) + cfg_exp(((R(25.0000) - y_V) / R(5.98000)))));
    R a_i_p_Ca = ((K(C_g_pCa) * y_Ca_i) / (y_Ca_i + K(C_K_pCa)));
    R a_i_rel = (((((K(C_a_rel) * cfg_ipow<2>(y_Ca_SR)) / (cfg_ipow<2>(K(C_b_rel)) + cfg_ipow<2>(y_Ca_SR))) + K(C_c_rel)) * y_d) * y_g);
    R a_i_up = (K(C_Vmax_up) / (R(1.00000) + (cfg_ipow<2>(K(C_K_up)) / cfg_ipow<2>(y_Ca_i))));
    R a_i_leak = (K(C_V_leak) * (y_Ca_SR - y_Ca_i));
    R a_ddt_Ca_i_total = ((((((-(((a_i_CaL + a_i_b_Ca) + a_i_p_Ca) - (R(2.00000) * a_i_NaCa))) / ((R(2.00000) * K(C_V_c)) * K(C_F))) * K(C_Cm)) + a_i_leak) - a_i_up) + a_i_rel);
    R a_f_JCa_i_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_c) * K(C_K_buf_c)) / cfg_ipow<2>((y_Ca_i + K(C_K_buf_c))))));
    R a_ddt_Ca_sr_total = ((K(C_V_c) / K(C_V_sr)) * (a_i_up - (a_i_rel + a_i_leak)));
    R a_f_JCa_sr_free = (R(1.00000) / (R(1.00000) + ((K(C_Buf_sr) * K(C_K_buf_sr)) / cfg_ipow<2>((y_Ca_SR + K(C_K_buf_sr))))));
    R a_Iion_cm = (((((((((((a_i_K1 + a_i_to) + a_i_Kr) + a_i_Ks) + a_i_CaL) + a_i_NaK) + a_i_Na) + a_i_b_Na) + a_i_NaCa) + a_i_b_Ca) + a_i_p_K) + a_i_p_Ca);
    R a_Istim = (SOLVE_VM ? R(cfg_stimulus_current<double>(t, stim)) : R(0));
    A[0] = a_Istim;
    A[1] = a_xr1_inf;
    A[2] = a_xr2_inf;
    A[3] = a_xs_inf;
    A[4] = a_m_inf;
    A[5] = a_h_inf;
    A[6] = a_j_inf;
    A[7] = a_d_inf;
    A[8] = a_f_inf;
    A[9] = a_alpha_fCa;
    A[10] = a_s_inf;
    A[11] = a_r_inf;
    A[12] = a_g_inf;
    A[13] = a_E_Na;
    A[14] = a_alpha_xr1;
    A[15] = a_alpha_xr2;
    A[16] = a_alpha_xs;
    A[17] = a_alpha_m;
    A[18] = a_alpha_h;
    A[19] = a_alpha_j;
    A[20] = a_alpha_d;
    A[21] = a_tau_f;
    A[22] = a_beta_fCa;
    A[23] = a_tau_s;
    A[24] = a_tau_r;
    A[25] = a_d_g;
    A[26] = a_E_K;
    A[27] = a_beta_xr1;
    A[28] = a_beta_xr2;
    A[29] = a_beta_xs;
    A[30] = a_beta_m;
    A[31] = a_beta_h;
    A[32] = a_beta_j;
    A[33] = a_gama_fCa;
    A[34] = a_beta_d;
    A[35] = a_E_Ks;
    A[36] = a_tau_xr1;
    A[37] = a_tau_xr2;
    A[38] = a_tau_xs;
    A[39] = a_tau_m;
    A[40] = a_tau_h;
    A[41] = a_tau_j;
    A[42] = a_gamma_d;
    A[43] = a_fCa_inf;
    A[44] = a_E_Ca;
    A[45] = a_tau_d;
    A[46] = a_d_fCa;
    A[47] = a_alpha_K1;
    A[48] = a_beta_K1;
    A[49] = a_xK1_inf;
    A[50] = a_i_K1;
    A[51] = a_i_Kr;
    A[52] = a_i_Ks;
    A[53] = a_i_Na;
    A[54] = a_i_b_Na;
    A[55] = a_i_CaL;
    A[56] = a_i_b_Ca;
    A[57] = a_i_to;
    A[58] = a_i_NaK;
    A[59] = a_i_NaCa;
    A[60] = a_i_p_Ca;
    A[61] = a_i_p_K;
    A[62] = a_i_rel;
    A[63] = a_i_up;
    A[64] = a_i_leak;
    A[65] = a_ddt_Ca_i_total;
    A[66] = a_ddt_Ca_sr_total;
    A[67] = a_f_JCa_i_free;
    A[68] = a_f_JCa_sr_free;
    A[69] = a_Iion_cm;
}

// STATES_NAMES / ALGEBRAIC_NAMES as the header spells them; matched by
// position, entries the header leaves out are empty
static const char* const STATE_STRINGS[17] = {"V", "K_i", "Na_i", "Ca_i", "Xr1", "Xr2", "Xs", "m", "h", "j", "d", "f", "fCa", "s", "r", "Ca_SR", "g"};
static const char* const ALG_STRINGS[70] = {"Istim", "xr1_inf", "xr2_inf", "xs_inf", "m_inf", "h_inf", "j_inf", "d_inf", "f_inf", "alpha_fCa", "s_inf", "r_inf", "g_inf", "E_Na", "alpha_xr1", "alpha_xr2", "alpha_xs", "alpha_m", "alpha_h", "alpha_j", "alpha_d", "tau_f", "beta_fCa", "tau_s", "tau_r", "d_g", "E_K", "beta_xr1", "beta_xr2", "beta_xs", "beta_m", "beta_h", "beta_j", "gama_fCa", "beta_d", "E_Ks", "tau_xr1", "tau_xr2", "tau_xs", "tau_m", "tau_h", "tau_j", "gamma_d", "fCa_inf", "E_Ca", "tau_d", "d_fCa", "alpha_K1", "beta_K1", "xK1_inf", "i_K1", "i_Kr", "i_Ks", "i_Na", "i_b_Na", "i_CaL", "i_b_Ca", "i_to", "i_NaK", "i_NaCa", "i_p_Ca", "i_p_K", "i_rel", "i_up", "i_leak", "ddt_Ca_i_total", "ddt_Ca_sr_total", "f_JCa_i_free", "f_JCa_sr_free", "Iion_cm"};
// <Model>DependencyMap(): current -> comma-separated variables, null-ended
static const char* const SWEEP_CURRENTS[] = {"INa", "I_Na", "ICaL", "I_CaL", "Ito", "I_to", "IKr", "I_Kr", "IKs", "I_Ks", "IK1", "I_K1", "INaK", "I_NaK", "INaCa", "I_NaCa", "IbNa", "IbCa", "I_bNa", "I_bCa", "IpCa", "IpK", "I_pCa", "I_pK", "RyR_g", "Iion", "Iion_cm", "I_ion", nullptr};
static const char* const SWEEP_DEPS[] = {"i_Na,m_inf,h_inf,j_inf,tau_m,tau_h,tau_j", "i_Na,m_inf,h_inf,j_inf,tau_m,tau_h,tau_j", "i_CaL,d_inf,f_inf,fCa_inf,tau_d,tau_f", "i_CaL,d_inf,f_inf,fCa_inf,tau_d,tau_f", "i_to,r_inf,s_inf,tau_r,tau_s", "i_to,r_inf,s_inf,tau_r,tau_s", "i_Kr,xr1_inf,xr2_inf,tau_xr1,tau_xr2", "i_Kr,xr1_inf,xr2_inf,tau_xr1,tau_xr2", "i_Ks,xs_inf,tau_xs", "i_Ks,xs_inf,tau_xs", "i_K1,xK1_inf", "i_K1,xK1_inf", "i_NaK", "i_NaK", "i_NaCa", "i_NaCa", "i_b_Na", "i_b_Ca", "i_b_Na", "i_b_Ca", "i_p_Ca", "i_p_K", "i_p_Ca", "i_p_K", "g_inf", "i_K1,i_to,i_Kr,i_Ks,i_CaL,i_Na,i_b_Na,i_NaK,i_NaCa,i_b_Ca,i_p_K,i_p_Ca,Iion_cm", "i_K1,i_to,i_Kr,i_Ks,i_CaL,i_Na,i_b_Na,i_NaK,i_NaCa,i_b_Ca,i_p_K,i_p_Ca,Iion_cm", "i_K1,i_to,i_Kr,i_Ks,i_CaL,i_Na,i_b_Na,i_NaK,i_NaCa,i_b_Ca,i_p_K,i_p_Ca,Iion_cm", nullptr};

// traits bundle used by the kernel templates
struct Model {
    static constexpr int NS = tnnp::NS, NC = tnnp::NC;
    static constexpr unsigned long long WIDE_MASK = tnnp::WIDE_MASK;
    static constexpr double IION_SCALE = tnnp::IION_SCALE;
    static constexpr double TIME_SCALE = tnnp::TIME_SCALE;
    static constexpr int VM_MAP = tnnp::VM_MAP;
    CFG_HD static __forceinline__ void init(double* C, double* y, int tissue, const double* scale) { init_consts(C, y, tissue, scale); }
    template <int T> CFG_HD static constexpr double constant(int i) { return cval<T>(i); }
    static constexpr int NSD = tnnp::NSD, CA_STATE = tnnp::CA_STATE;
    static constexpr int NH = tnnp::NH;
    template <class R, class KS>
    __device__ static __forceinline__ void hoist_vm(R v, const KS& K, int tissue, R* H) { hoist<R>(v, K, tissue, H); }
    template <class R, class YS, class KS, class HS>
    __device__ static __forceinline__ R rates_tissue(double t, const YS& Y, const KS& K, const HS& H, R* dydt, int tissue, const CfgStimulus& st) { return rhs_tissue<R>(t, Y, K, H, dydt, tissue, st); }
    CFG_HD static constexpr int sd_slot(int i) { return tnnp::sd_slot(i); }
    static constexpr int NA = tnnp::NA;
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ void all_variables(double t, const YS& Y, const KS& K, R* A, R* dydt, int tissue, const CfgStimulus& st) { variables_all<R, SV>(t, Y, K, A, dydt, tissue, st); }
    CFG_HD static constexpr int sd_const(int k) { return tnnp::sd_const(k); }
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ R rates(double t, const YS& Y, const KS& K, R* dydt, int tissue, const CfgStimulus& st) { return rhs<R, SV>(t, Y, K, dydt, tissue, st); }
    template <class R, bool SV, class YS, class KS>
    __device__ static __forceinline__ R current(double t, const YS& Y, const KS& K, int tissue, const CfgStimulus& st) { return iion<R, SV>(t, Y, K, tissue, st); }
};

} }  // namespace cfg::tnnp
