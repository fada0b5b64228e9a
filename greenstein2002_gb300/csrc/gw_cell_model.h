/*
 * Global (whole-cell) model of the Greenstein-Winslow myocyte: the 37-state
 * right-hand side that the Dormand-Prince integrator advances between FRU
 * stages.  Plain C99 that also compiles as CUDA device code (GW_HD), so the
 * host driver and a device-resident integrator share one definition.
 *
 * Reference: fcn.c:29-1072 (equations, in the same operand order, so that
 * compiled without FP contraction the derivatives agree with the reference
 * bit for bit wherever the math library agrees), indices.h (state layout),
 * initialize_state.c:167-310 (rest state, CaTOT, error weights),
 * parameters.h:92-156 (protocol settings, here a runtime struct).
 */
#ifndef GW_CELL_MODEL_H
#define GW_CELL_MODEL_H

#include <math.h>

#include "gw_fru.h"

#ifdef __CUDACC__
#define GW_HD __host__ __device__ static inline
#else
#define GW_HD static inline
#endif

/* state indices (indices.h:5-41) */
enum {
  GW_V = 0, GW_mNa, GW_hNa, GW_jNa, GW_Nai, GW_Ki, GW_Cai, GW_CaNSR, GW_xKs, GW_LTRPNCa, GW_HTRPNCa,
  GW_C0Kv43, GW_C1Kv43, GW_C2Kv43, GW_C3Kv43, GW_OKv43, GW_CI0Kv43, GW_CI1Kv43, GW_CI2Kv43, GW_CI3Kv43,
  GW_OIKv43, GW_C0Kv14, GW_C1Kv14, GW_C2Kv14, GW_C3Kv14, GW_OKv14, GW_CI0Kv14, GW_CI1Kv14, GW_CI2Kv14,
  GW_CI3Kv14, GW_OIKv14, GW_CaTOT, GW_C1Herg, GW_C2Herg, GW_C3Herg, GW_OHerg, GW_IHerg, GW_NSTATE
};
/* current indices (indices.h:56-79) */
enum {
  GW_I_INa = 0, GW_I_IKr, GW_I_IKs, GW_I_Ito1, GW_I_IK1, GW_I_IKp, GW_I_INaCa, GW_I_INaK, GW_I_IpCa,
  GW_I_ICab, GW_I_INab, GW_I_ICa, GW_I_JDHPR, GW_I_Jup, GW_I_Jtrpn, GW_I_Jtr, GW_I_Jxfer, GW_I_IKv43,
  GW_I_IKv14, GW_I_IKv14_K, GW_I_IKv14_Na, GW_I_Ito2, GW_I_Istim, GW_I_Itot, GW_NCUR
};
/* other-state indices (indices.h:43-54) */
enum {
  GW_O_CaSSavg = 0, GW_O_CaJSRavg, GW_O_JRyRtot, GW_O_PRyR_Open, GW_O_PRyR_ready, GW_O_PNorm_Mode,
  GW_O_PnotVinact, GW_O_PLType_Open, GW_O_CaTOT2, GW_O_PIto2_Open, GW_O_CaJSRtot, GW_O_CaSStot, GW_NOTHER
};

/* Run settings (parameters.h:92-156 as runtime fields of the same names) are
 * the public gw_settings struct of gw_fru.h. */
typedef gw_settings gw_protocol;

/* ---- constants: parameters_fcn_fru.c:21-90 ---------------------------------- */
#define GWC_Ko 4.0
#define GWC_Nao 138.0
#define GWC_Cao 2.0
#define GWC_Faraday 96.5
#define GWC_RT_over_F (8.314 * 310.0 / 96.5)
#define GWC_Acap 1.534e-4
#define GWC_VNSR (0.53 * 2.10e-6)
#define GWC_Vmyo 25.84e-6
#define GWC_VJSR (((double)4) * 0.53 * 0.5 * 0.2 * 1.05e-10)
#define GWC_VSS (0.5 * 0.2 * 2.03e-12)
#define GWC_LTRPNtot 70.0e-3
#define GWC_HTRPNtot 140.0e-3
#define GWC_khtrpn_plus 20.0
#define GWC_khtrpn_minus 0.066e-3
#define GWC_kltrpn_plus 40.0
#define GWC_kltrpn_minus 40.0e-3
#define GWC_CMDNtot 50.0e-3
#define GWC_EGTAtot 0.0
#define GWC_KmCMDN 2.38e-3
#define GWC_KmEGTA 1.5e-4
#define GWC_CSQNtot 13.5
#define GWC_KmCSQN 0.63
#define GWC_BSRtot 0.047
#define GWC_KBSR 0.00087
#define GWC_BSLtot 1.124
#define GWC_KBSL 0.0087
/* FRU flux constants used by the per-FRU property output
 * (parameters_fcn_fru.c:24-25, :48-50, :83-87) */
#define GWC_Clo 150.0
#define GWC_Cli 20.0
#define GWC_PCa (1.5 / 2.8 * 0.2 * 0.9 * 0.9468e-11)
#define GWC_PCl 2.65e-15
#define GWC_JRyRmax (0.6 * 1.5 * 1.1 * 3.96)
#define GWC_tautr 3.0
#define GWC_tauxfer 0.005

GW_HD void gw_protocol_defaults(gw_protocol* p) {
  /* parameters.h:92-156 */
  p->time_start = 0.0; p->time_end = 12000.0; p->time_step = 1.0;
  p->step_min = 1.e-6; p->step_max = 0.1; p->tolrk = 1.e-6;
  p->pulse_duration = 1; p->pulse_amplitude = -100; p->period = 1000; p->shift = 10;
  p->vclamp_flag = 0; p->vclamp_duration = 200.0; p->vclamp_set = 0.0; p->vclamp_shift = 300.0;
  p->vclamp_hold = -80.0; p->vclamp_period = 500.0;
  p->vppclamp_flag = 0; p->vppclamp_ppset = -40.0; p->vppclamp_ppduration = 100.0; p->vppclamp_shift = 10000.0;
  p->vppclamp_set = 0.0; p->vppclamp_duration = 300.0; p->vppclamp_hold = -80.0; p->vppclamp_period = 500.0;
  p->iv_flag = 0; p->iv_clamp_duration = 50.0; p->iv_clamp_period = 200.0; p->iv_shift = 10.0;
  p->iv_clamp_set = -40.0; p->iv_clamp_hold = -100.0; p->iv_clamp_step = 10.0; p->iv_n = 0;
  p->chf_flag = 0; p->chfsc_IK1 = 0.68; p->chfsc_Jup = 0.38; p->chfsc_INaCa = 1.75; p->chfsc_IKv43 = 0.143;
  p->scale_PCa = 1.0; p->scale_GKr = 1.0;
}

/* Error weights of the DP error norm, initialize_state.c:274-310. */
GW_HD double gw_errweight(int i) {
  switch (i) {
    case GW_V: case GW_OIKv43: case GW_OIKv14: case GW_IHerg: return 0.0;
    case GW_Nai: return 0.1;
    case GW_Ki: return 1 / 140.0;
    case GW_Cai: return 1.e3;
    case GW_CaNSR: return 2.5;
    case GW_CaTOT: return 0.1;
    default: return 1.0;
  }
}

/* ---- transcendental terms of the right-hand side ------------------------------
 * Every exp, log and pow of fcn.c:549-998 depends only on the (clamped)
 * membrane potential and on concentrations, except K1_inf's exp, which
 * depends on EK (a log).  gw_tx holds them all, so that a GPU warp can
 * evaluate them side by side -- one per lane, the same function on every
 * lane -- before the arithmetic that combines them (gw_fcn_tx); each entry
 * is the value fcn.c computes, from the same operands by the same
 * operations.  The 34 exponents share one form, ((V or 0) + d) op c [* e]
 * with op a multiplication or a division: fcn.c's expressions rewritten by
 * commutation and sign symmetry only (a - b = -(b - a), -x / c = x / -c,
 * x - d = x + (-d)), which round identically. */
enum {
  GW_X_VFRT = 0, GW_X_KPV, GW_X_SIGMA, GW_X_NAK, GW_X_ETA, GW_X_AM, GW_X_BM, GW_X_AH, GW_X_BH1, GW_X_BH2, GW_X_BH3,
  GW_X_AJ1, GW_X_AJ2, GW_X_AJ3, GW_X_BJ1, GW_X_BJ2, GW_X_BJ3, GW_X_BJ4, GW_X_H0, GW_X_H1, GW_X_H2, GW_X_H3, GW_X_H4,
  GW_X_H5, GW_X_H6, GW_X_XKS, GW_X_KS1, GW_X_KS2, GW_X_43A, GW_X_43B, GW_X_43C, GW_X_43D, GW_X_14A, GW_X_14B, GW_NX
};
enum { GW_XF_V = 1, GW_XF_ADD = 2, GW_XF_DIV = 4, GW_XF_MUL2 = 8 };
typedef struct gw_tx {
  double x[GW_NX]; /* exp of the exponents above */
  double lg[4];    /* log(Nao/Nai), log(Ko/Ki), log(a1/a2) of EKs, log(Cao/Cai) */
  double pw[6];    /* pow(Ko/4, 0.5), pow(KmNai/Nai, 1.5), fb, rb, (Cai+KmCMDN)^2, (Cai+KmEGTA)^2 */
  double k1;       /* exp(1.76/RT_over_F (V - EK)) of K1_inf */
} gw_tx;

/* exponent k: flags, d, c, e (fcn.c:565-998) */
GW_HD int gw_x_form(int k, double* d, double* c, double* e) {
  const double RT = GWC_RT_over_F;
  *d = 0.0;
  *e = 1.0;
  switch (k) {
    case GW_X_VFRT: *c = RT; return GW_XF_V | GW_XF_DIV;                                  /* V/RT */
    case GW_X_KPV: *d = -7.488; *c = -5.98; return GW_XF_V | GW_XF_ADD | GW_XF_DIV;       /* (7.488 - V)/5.98 */
    case GW_X_SIGMA: *d = GWC_Nao; *c = 67.3; return GW_XF_ADD | GW_XF_DIV;               /* Nao/67.3 */
    case GW_X_NAK: *c = RT; *e = -0.1; return GW_XF_V | GW_XF_DIV | GW_XF_MUL2;           /* -0.1 VF/RT */
    case GW_X_ETA: *c = RT; *e = 0.35; return GW_XF_V | GW_XF_DIV | GW_XF_MUL2;           /* eta VF/RT */
    case GW_X_AM: *d = 47.13; *c = -0.1; return GW_XF_V | GW_XF_ADD;                      /* -0.1 (V + 47.13) */
    case GW_X_BM: *c = -11.0; return GW_XF_V | GW_XF_DIV;                                 /* -V/11 */
    case GW_X_AH: *d = 80.0; *c = -6.8; return GW_XF_V | GW_XF_ADD | GW_XF_DIV;           /* (80 + V)/-6.8 */
    case GW_X_BH1: *c = 0.079; return GW_XF_V;
    case GW_X_BH2: *c = 0.35; return GW_XF_V;
    case GW_X_BH3: *d = 10.66; *c = -11.1; return GW_XF_V | GW_XF_ADD | GW_XF_DIV;
    case GW_X_AJ1: *c = 0.2444; return GW_XF_V;
    case GW_X_AJ2: *c = -0.04391; return GW_XF_V;
    case GW_X_AJ3: *d = 79.23; *c = 0.311; return GW_XF_V | GW_XF_ADD;
    case GW_X_BJ1: *c = -0.01052; return GW_XF_V;
    case GW_X_BJ2: *d = 40.14; *c = -0.1378; return GW_XF_V | GW_XF_ADD;
    case GW_X_BJ3: *c = -2.535E-7; return GW_XF_V;
    case GW_X_BJ4: *d = 32.0; *c = -0.1; return GW_XF_V | GW_XF_ADD;
    case GW_X_H0: *c = 0.03304608038835; return GW_XF_V;   /* B0_HERG .. B6_HERG */
    case GW_X_H1: *c = -0.04306054163980; return GW_XF_V;
    case GW_X_H2: *c = 0.02617412715118; return GW_XF_V;
    case GW_X_H3: *c = -0.02691385498399; return GW_XF_V;
    case GW_X_H4: *c = 0.00568908859717; return GW_XF_V;
    case GW_X_H5: *c = -0.04536642959543; return GW_XF_V;
    case GW_X_H6: *c = 0.00000069808924; return GW_XF_V;
    case GW_X_XKS: *d = -24.7; *c = -13.6; return GW_XF_V | GW_XF_ADD | GW_XF_DIV;        /* -(V - 24.7)/13.6 */
    case GW_X_KS1: *d = -10.0; *c = -0.148; return GW_XF_V | GW_XF_ADD;
    case GW_X_KS2: *d = -10.0; *c = 0.0687; return GW_XF_V | GW_XF_ADD;
    case GW_X_43A: *c = 0.028983; return GW_XF_V;           /* aaKv43, -baKv43, -aiKv43, biKv43 */
    case GW_X_43B: *c = -0.0468437; return GW_XF_V;
    case GW_X_43C: *c = -0.000373016; return GW_XF_V;
    case GW_X_43D: *c = 0.00000005374; return GW_XF_V;
    case GW_X_14A: *c = 0.00695; return GW_XF_V;            /* aaKv14, -baKv14 */
    default: *c = -0.08527; return GW_XF_V;                 /* GW_X_14B */
  }
}

GW_HD double gw_x_arg(int k, double V) {
  double d, c, e;
  const int f = gw_x_form(k, &d, &c, &e);
  double t = (f & GW_XF_V) ? V : 0.0;
  if (f & GW_XF_ADD) t = t + d;
  t = (f & GW_XF_DIV) ? t / c : t * c;
  if (f & GW_XF_MUL2) t = t * e;
  return t;
}

/* Cai as fcn.c:558 uses it from there on */
GW_HD double gw_cai_clamped(const double* state) { return state[GW_Cai] <= 0.0 ? 1.e-15 : state[GW_Cai]; }

/* argument of log k and base / exponent of pow k */
GW_HD double gw_lg_arg(int k, const double* state) {
  const double Nai = state[GW_Nai], Ki = state[GW_Ki];
  switch (k) {
    case 0: return GWC_Nao / Nai;
    case 1: return GWC_Ko / Ki;
    case 2: return (GWC_Ko + 0.01833 * GWC_Nao) / (Ki + 0.01833 * Nai);
    default: return GWC_Cao / gw_cai_clamped(state);
  }
}
GW_HD double gw_pw_arg(int k, const double* state, double* y) {
  const double Cai = gw_cai_clamped(state);
  switch (k) {
    case 0: *y = 0.5; return GWC_Ko / 4.0;
    case 1: *y = 1.5; return 10.0 / state[GW_Nai];            /* KmNai / Nai */
    case 2: *y = 0.75; return Cai / 0.26e-3;                   /* Cai / Kfb, Nfb */
    case 3: *y = 0.75; return state[GW_CaNSR] / 1.8;           /* CaNSR / Krb, Nrb */
    case 4: *y = 2.0; return Cai + GWC_KmCMDN;
    default: *y = 2.0; return Cai + GWC_KmEGTA;
  }
}
/* exponent of K1_inf's exp: 1.76/RT_over_F (V - EK) */
GW_HD double gw_k1_arg(double V, const double* tx_lg) {
  const double EK = GWC_RT_over_F * tx_lg[1];
  return 1.76 / GWC_RT_over_F * (V - EK);
}

/* Membrane potential of fcn.c:434-535: the state's V, or the clamp level of
 * an active clamp protocol; *Istim receives the applied stimulus. */
GW_HD double gw_fcn_voltage(const double time, const double* state, const gw_protocol* P, double* Istim_out) {
  double V = state[GW_V], Istim;
  /* ---- applied stimulus, fcn.c:434-443 ---- */
  {
    const double on = floor((time - P->shift) / P->period) * P->period;
    const double off = on + P->pulse_duration;
    Istim = 0.0;
    if ((time - P->shift) >= on && (time - P->shift) <= off) Istim = Istim + P->pulse_amplitude;
  }
  /* ---- voltage clamp, fcn.c:448-483 ---- */
  if (P->vclamp_flag) {
    const double on = floor((time - P->vclamp_shift) / P->vclamp_period) * P->vclamp_period;
    const double off = on + P->vclamp_duration;
    if (((time - P->vclamp_shift) >= on) && (on >= 0.0) && ((time - P->vclamp_shift) < off)) V = P->vclamp_set;
    else V = P->vclamp_hold;
  }
  /* ---- clamp with a prepulse, fcn.c:485-516 ---- */
  if (P->vppclamp_flag) {
    const double on = floor((time - P->vppclamp_shift) / P->vppclamp_period) * P->vppclamp_period;
    const double ppoff = on + P->vppclamp_ppduration;
    const double off = on + P->vppclamp_duration + P->vppclamp_ppduration;
    if (((time - P->vppclamp_shift) >= on) && (on >= 0.0) && ((time - P->vppclamp_shift) < ppoff)) {
      V = P->vppclamp_ppset;
    } else if (((time - P->vppclamp_shift) >= ppoff) && (on >= 0.0) && ((time - P->vppclamp_shift) < off)) {
      V = P->vppclamp_set;
    } else if (((time - P->vppclamp_shift) < on) || (on < 0.0) || ((time - P->vppclamp_shift) >= off)) {
      V = P->vppclamp_hold;
    }
  }
  /* ---- I-V protocol clamp, fcn.c:521-535 ---- */
  if (P->iv_flag) {
    const double ps = (floor((time + 1.e-20) / P->iv_clamp_period)) * P->iv_clamp_period;
    const double pe = (1.0 + floor((time + 1.e-20) / P->iv_clamp_period)) * P->iv_clamp_period;
    const double on = P->iv_shift + ps;
    double off = on + P->iv_clamp_duration;
    off = (pe < off) ? pe : off;
    if ((time >= on) && (time < off)) V = P->iv_clamp_set + P->iv_n * P->iv_clamp_step;
    else V = P->iv_clamp_hold;
  }

  *Istim_out = Istim;
  return V;
}

/* Global right-hand side (fcn.c:29-1072) given its transcendental terms
 * (gw_tx, filled for this state and time).  May overwrite state[GW_mNa]
 * (V < -90 mV steady state) and state[GW_V] (clamp modes) in place, as the
 * reference does.  current[] is filled when keepc != 0. */
GW_HD void gw_fcn_tx(const double time, double* state, double* F, double* current, const int keepc,
                     const double Jxfer, const double Jtr, const double ICa, const double Ito2, const gw_protocol* P,
                     const gw_tx* tx) {
  /* membrane current parameters, fcn.c:169-264 */
  const double GKr = 0.029 * P->scale_GKr, GKs = 0.035, GK1 = 3.0, GKp = 1.2 * 0.002216, GNa = 12.8;
  /* eta, KmNai, Kfb, Krb, Nfb, Nrb and the exponents' rate constants enter
   * only the transcendental terms (gw_x_form, gw_pw_arg) */
  const double kNaCa = 0.9 * 0.30, KmNa = 87.5, KmCa = 1.38, KmK1 = 13.0, ksat = 0.2;
  const double INaKmax = 1.3 * 0.693, KmKo = 1.5, IpCamax = 0.6 * 0.05, KmpCa = 0.0005;
  const double GCab = 3.3 * 7.684e-5, GNab = 0.001;
  const double KSR = 1.0;
  const double vmaxf = 1.53 * 137.0e-6, vmaxr = 1.53 * 137.0e-6;
  const double KvScale = 1.13 * 1.03 * 1.55, Kv43Frac = 0.77;
  const double GKv43 = Kv43Frac * KvScale * 0.1;
  const double PKv14 = (1.0 - Kv43Frac) * KvScale * 4.792933e-7;
  const double alphaa0Kv43 = 0.543708, betaa0Kv43 = 0.080185;
  const double alphai0Kv43 = 0.0498424, betai0Kv43 = 0.000819482;
  const double alphaa0Kv14 = 6.0 * 0.31551, betaa0Kv14 = 6.0 * 0.001966;
  const double alphai0Kv14 = 6.0 * 0.0004938, betai0Kv14 = 6.0 * 0.0000176;
  const double f1Kv43 = 1.8936, f2Kv43 = 14.224647456, f3Kv43 = 158.574378389, f4Kv43 = 142.936645351;
  const double b1Kv43 = 6.77348, b2Kv43 = 15.6212705152, b3Kv43 = 28.7532603313, b4Kv43 = 524.576206679;
  const double f1Kv14 = 0.20005, f2Kv14 = 0.320280, f3Kv14 = 13.50909223, f4Kv14 = 1151.7651385;
  const double b1Kv14 = 2.2300, b2Kv14 = 12.000299, b3Kv14 = 5.3701338025, b4Kv14 = 5.2396395511;
  const double T_Const_HERG = 5.320000001;
  const double A0_HERG = 0.017147641733086, A1_HERG = 0.03969328381141, A2_HERG = 0.02057448605977;
  const double A3_HERG = 0.00134366604423, A4_HERG = 0.10666316491288, A5_HERG = 0.00646393910049;
  const double A6_HERG = 0.00008039374403;
  const double C2H_to_C3H = T_Const_HERG * 0.02608362043337;
  const double C3H_to_C2H = T_Const_HERG * 0.14832978132145;
  const double RT_over_F = GWC_RT_over_F, Faraday = GWC_Faraday, Ko = GWC_Ko, Nao = GWC_Nao, Cao = GWC_Cao;
  const double Acap = GWC_Acap, Vmyo = GWC_Vmyo, VNSR = GWC_VNSR, VJSR = GWC_VJSR, VSS = GWC_VSS;

  double V, mNa = state[GW_mNa], hNa = state[GW_hNa], jNa = state[GW_jNa], Nai = state[GW_Nai];
  double Ki = state[GW_Ki], Cai = state[GW_Cai], xKs = state[GW_xKs];
  double LTRPNCa = state[GW_LTRPNCa], HTRPNCa = state[GW_HTRPNCa];
  const double C0Kv43 = state[GW_C0Kv43], C1Kv43 = state[GW_C1Kv43], C2Kv43 = state[GW_C2Kv43];
  const double C3Kv43 = state[GW_C3Kv43], OKv43 = state[GW_OKv43], CI0Kv43 = state[GW_CI0Kv43];
  const double CI1Kv43 = state[GW_CI1Kv43], CI2Kv43 = state[GW_CI2Kv43], CI3Kv43 = state[GW_CI3Kv43];
  const double OIKv43 = 1.0 - CI0Kv43 - CI1Kv43 - CI2Kv43 - CI3Kv43 - OKv43 - C0Kv43 - C1Kv43 - C2Kv43 - C3Kv43;
  const double C0Kv14 = state[GW_C0Kv14], C1Kv14 = state[GW_C1Kv14], C2Kv14 = state[GW_C2Kv14];
  const double C3Kv14 = state[GW_C3Kv14], OKv14 = state[GW_OKv14], CI0Kv14 = state[GW_CI0Kv14];
  const double CI1Kv14 = state[GW_CI1Kv14], CI2Kv14 = state[GW_CI2Kv14], CI3Kv14 = state[GW_CI3Kv14];
  const double OIKv14 = 1.0 - CI0Kv14 - CI1Kv14 - CI2Kv14 - CI3Kv14 - OKv14 - C0Kv14 - C1Kv14 - C2Kv14 - C3Kv14;
  const double C1Herg = state[GW_C1Herg], C2Herg = state[GW_C2Herg], C3Herg = state[GW_C3Herg];
  const double OHerg = state[GW_OHerg];
  const double IHerg = 1.0 - OHerg - C1Herg - C2Herg - C3Herg;
  double Istim, a1, a2, a3, a4, a5;
  V = gw_fcn_voltage(time, state, P, &Istim);

  /* ---- reversal potentials, fcn.c:549-559 ---- */
  const double ENa = RT_over_F * tx->lg[0];
  const double EK = RT_over_F * tx->lg[1];
  a1 = Ko + 0.01833 * Nao;
  a2 = Ki + 0.01833 * Nai;
  const double EKs = RT_over_F * tx->lg[2];
  if (Cai <= 0.0) Cai = 1.e-15;
  const double ECa = 0.5 * RT_over_F * tx->lg[3];

  /* ---- INa, IKr, IKs, Ito1, IK1, INab, IKp, fcn.c:565-619 ---- */
  if (mNa <= 0.0) mNa = 1.e-15;
  const double INa = GNa * (mNa * mNa * mNa) * hNa * jNa * (V - ENa);
  const double fKo = tx->pw[0];
  const double IKr = GKr * fKo * OHerg * (V - EK);
  const double IKs = GKs * (xKs * xKs) * (V - EKs);
  double IKv43 = GKv43 * OKv43 * (V - EK);
  double VF_over_RT = V / RT_over_F;
  const double VFsq_over_RT = (1000.0 * Faraday) * VF_over_RT;
  const double exp_VFRT = tx->x[GW_X_VFRT];
  double IKv14_K, IKv14_Na;
  a1 = Ki * exp_VFRT - Ko;
  a2 = exp_VFRT - 1.0;
  if (fabs(V) < 1.e-6) IKv14_K = PKv14 * OKv14 * 1000.0 * Faraday * (Ki - Ko);
  else IKv14_K = PKv14 * OKv14 * VFsq_over_RT * (a1 / a2);
  a1 = Nai * exp_VFRT - Nao;
  if (fabs(V) < 1.e-6) IKv14_Na = 0.02 * PKv14 * OKv14 * 1000.0 * Faraday * (Nai - Nao);
  else IKv14_Na = 0.02 * PKv14 * OKv14 * VFsq_over_RT * (a1 / a2);
  const double IKv14 = IKv14_K + IKv14_Na;
  double Ito1 = IKv43 + IKv14;
  const double K1_inf = 1.0 / (0.94 + tx->k1);
  double IK1 = GK1 * Ko / (Ko + KmK1) * K1_inf * (V - EK);
  const double INab = GNab * (V - ENa);
  const double KpV = 1.0 / (1.0 + tx->x[GW_X_KPV]);
  const double IKp = GKp * KpV * (V - EK);

  /* ---- INaK, INaCa, ICab, IpCa, fcn.c:623-649 ---- */
  VF_over_RT = V / RT_over_F;
  const double sigma = (tx->x[GW_X_SIGMA] - 1.0) / 7.0;
  a1 = 1.0 + 0.1245 * tx->x[GW_X_NAK];
  a2 = 0.0365 * sigma / exp_VFRT;
  const double fNaK = 1.0 / (a1 + a2);
  a1 = Ko / (Ko + KmKo);
  a2 = 1.0 + tx->pw[1];
  const double INaK = INaKmax * fNaK * (a1 / a2);
  const double exp_etaVFRT = tx->x[GW_X_ETA];
  a1 = exp_etaVFRT * (Nai * Nai * Nai) * Cao;
  a2 = exp_etaVFRT / exp_VFRT * (Nao * Nao * Nao) * Cai;
  a3 = 1.0 + ksat * exp_etaVFRT / exp_VFRT;
  a4 = KmCa + Cao;
  a5 = 5000.0 / (KmNa * KmNa * KmNa + Nao * Nao * Nao);
  double INaCa = kNaCa * a5 * (a1 - a2) / (a4 * a3);
  const double ICab = GCab * (V - ECa);
  const double IpCa = IpCamax * Cai / (KmpCa + Cai);

  /* ---- gating derivatives, fcn.c:654-755 ---- */
  double alpha_m, dmNa;
  if (fabs(V + 47.13) <= 1.e-4) {
    alpha_m = 0.32 / (0.1 - 0.005 * (V + 47.13));
  } else {
    a1 = 0.32 * (V + 47.13);
    alpha_m = a1 / (1.0 - tx->x[GW_X_AM]);
  }
  const double beta_m = 0.08 * tx->x[GW_X_BM];
  if (V >= -90.0) {
    dmNa = alpha_m * (1.0 - mNa) - beta_m * mNa;
  } else {
    dmNa = 0.0;
    mNa = alpha_m / (alpha_m + beta_m);
    state[GW_mNa] = mNa;
  }
  const double alpha_h = 0.135 * tx->x[GW_X_AH];
  double beta_h, alpha_j, beta_j;
  if (V < -38.73809636838782) beta_h = 3.56 * tx->x[GW_X_BH1] + 310000 * tx->x[GW_X_BH2];
  else beta_h = 1 / (0.13 * (1 + tx->x[GW_X_BH3]));
  if (V < -37.78) {
    a1 = -127140 * tx->x[GW_X_AJ1];
    a2 = 3.474E-5 * tx->x[GW_X_AJ2];
    a3 = 1.0 + tx->x[GW_X_AJ3];
    alpha_j = (a1 - a2) * (V + 37.78) / a3;
  } else {
    alpha_j = 0;
  }
  if (V < -39.82600037702883) beta_j = 0.1212 * tx->x[GW_X_BJ1] / (1.0 + tx->x[GW_X_BJ2]);
  else beta_j = 0.3 * tx->x[GW_X_BJ3] / (1 + tx->x[GW_X_BJ4]);
  const double dhNa = alpha_h * (1.0 - hNa) - beta_h * hNa;
  const double djNa = alpha_j * (1.0 - jNa) - beta_j * jNa;

  /* HERG Markov model (IKr) */
  const double C1H_to_C2H = T_Const_HERG * A0_HERG * tx->x[GW_X_H0];
  const double C2H_to_C1H = T_Const_HERG * A1_HERG * tx->x[GW_X_H1];
  const double C3H_to_OH = T_Const_HERG * A2_HERG * tx->x[GW_X_H2];
  const double OH_to_C3H = T_Const_HERG * A3_HERG * tx->x[GW_X_H3];
  const double OH_to_IH = T_Const_HERG * A4_HERG * tx->x[GW_X_H4];
  const double IH_to_OH = T_Const_HERG * A5_HERG * tx->x[GW_X_H5];
  const double C3H_to_IH = T_Const_HERG * A6_HERG * tx->x[GW_X_H6];
  const double IH_to_C3H = (OH_to_C3H * IH_to_OH * C3H_to_IH) / (C3H_to_OH * OH_to_IH);
  const double dC1Herg = C2H_to_C1H * C2Herg - C1H_to_C2H * C1Herg;
  a1 = C1H_to_C2H * C1Herg + C3H_to_C2H * C3Herg;
  a2 = (C2H_to_C1H + C2H_to_C3H) * C2Herg;
  const double dC2Herg = a1 - a2;
  a1 = C2H_to_C3H * C2Herg + OH_to_C3H * OHerg + IH_to_C3H * IHerg;
  a2 = (C3H_to_IH + C3H_to_OH + C3H_to_C2H) * C3Herg;
  const double dC3Herg = a1 - a2;
  a1 = C3H_to_OH * C3Herg + IH_to_OH * IHerg;
  a2 = (OH_to_C3H + OH_to_IH) * OHerg;
  const double dOHerg = a1 - a2;

  /* IKs */
  const double xKs_inf = 1.0 / (1.0 + tx->x[GW_X_XKS]);
  if (fabs(V - 10) < 1.e-6) {
    a1 = (7.19e-5) / 0.148;
    a2 = (1.31e-4) / 0.0687;
  } else {
    a1 = 7.19e-5 * (V - 10.0) / (1.0 - tx->x[GW_X_KS1]);
    a2 = 1.31e-4 * (V - 10.0) / (tx->x[GW_X_KS2] - 1.0);
  }
  const double tau_xKs = 1.0 / (a1 + a2);
  const double dxKs = (xKs_inf - xKs) / tau_xKs;

  /* ---- SR uptake and troponin, fcn.c:759-776 ---- */
  const double fb = tx->pw[2];
  const double rb = tx->pw[3];
  double Jup = KSR * (vmaxf * fb - vmaxr * rb) / (1.0 + fb + rb);
  a1 = GWC_kltrpn_minus * LTRPNCa;
  const double dLTRPNCa = GWC_kltrpn_plus * Cai * (1.0 - LTRPNCa) - a1;
  a1 = GWC_khtrpn_minus * HTRPNCa;
  const double dHTRPNCa = GWC_khtrpn_plus * Cai * (1.0 - HTRPNCa) - a1;
  const double Jtrpn = GWC_LTRPNtot * dLTRPNCa + GWC_HTRPNtot * dHTRPNCa;
  a1 = GWC_CMDNtot * GWC_KmCMDN / (tx->pw[4]);
  a2 = GWC_EGTAtot * GWC_KmEGTA / (tx->pw[5]);
  const double beta_i = 1.0 / (1.0 + a1 + a2);

  /* ---- heart-failure scalings, fcn.c:780-786 ---- */
  if (P->chf_flag) {
    IK1 = P->chfsc_IK1 * IK1;
    Jup = P->chfsc_Jup * Jup;
    INaCa = P->chfsc_INaCa * INaCa;
    IKv43 = P->chfsc_IKv43 * IKv43;
    Ito1 = IKv43 + IKv14;
  }

  /* ---- concentrations and V, fcn.c:791-841 ---- */
  a1 = Acap / (Vmyo * Faraday * 1000.0);
  const double dNai = -(INa + INab + 3.0 * (INaCa + INaK) + IKv14_Na) * a1;
  a3 = IKr + IKs + IK1 + IKp;
  const double dKi = -(a3 - 2.0 * INaK + (Ito1 - IKv14_Na) + Istim) * a1;
  a3 = ICab - 2.0 * INaCa + IpCa;
  const double dCai = beta_i * (Jxfer * VSS / Vmyo - Jup - Jtrpn - a3 * 0.5 * a1);
  const double dCaNSR = Jup * Vmyo / VNSR - Jtr * VJSR / VNSR;
  const double dCaTOT = -(a3 + ICa) * 0.5 * a1 * Vmyo * 1.0e6;
  a1 = INa + ICa + IKr + IKs;
  a2 = IK1 + IKp + INaCa + INaK + Ito1 + Ito2;
  a3 = IpCa + ICab + INab;
  double dV, Itot;
  if (P->vclamp_flag || P->iv_flag) {
    dV = 0.0;
    state[GW_V] = V;
    Itot = a1 + a2 + a3;
  } else {
    Itot = a1 + a2 + a3 + Istim;
    dV = -Itot;
  }
  if (P->vppclamp_flag) {
    dV = 0.0;
    state[GW_V] = V;
    Itot = a1 + a2 + a3;
  }

  /* ---- Kv4.3, fcn.c:846-917 ---- */
  {
    const double al = alphaa0Kv43 * tx->x[GW_X_43A], be = betaa0Kv43 * tx->x[GW_X_43B];
    const double ali = alphai0Kv43 * tx->x[GW_X_43C], bei = betai0Kv43 * tx->x[GW_X_43D];
    const double C0C1 = 4.0 * al, C1C2 = 3.0 * al, C2C3 = 2.0 * al, C3O = al;
    const double CI0CI1 = 4.0 * b1Kv43 * al, CI1CI2 = 3.0 * b2Kv43 * al / b1Kv43;
    const double CI2CI3 = 2.0 * b3Kv43 * al / b2Kv43, CI3OI = b4Kv43 * al / b3Kv43;
    const double C1C0 = be, C2C1 = 2.0 * be, C3C2 = 3.0 * be, OC3 = 4.0 * be;
    const double CI1CI0 = be / f1Kv43, CI2CI1 = 2.0 * f1Kv43 * be / f2Kv43;
    const double CI3CI2 = 3.0 * f2Kv43 * be / f3Kv43, OICI3 = 4.0 * f3Kv43 * be / f4Kv43;
    const double C0CI0 = bei, C1CI1 = f1Kv43 * bei, C2CI2 = f2Kv43 * bei, C3CI3 = f3Kv43 * bei, OOI = f4Kv43 * bei;
    const double CI0C0 = ali, CI1C1 = ali / b1Kv43, CI2C2 = ali / b2Kv43, CI3C3 = ali / b3Kv43, OIO = ali / b4Kv43;
    double d[9];
    a1 = (C0C1 + C0CI0) * C0Kv43; a2 = C1C0 * C1Kv43 + CI0C0 * CI0Kv43; d[0] = a2 - a1;
    a1 = (C1C2 + C1C0 + C1CI1) * C1Kv43; a2 = C2C1 * C2Kv43 + CI1C1 * CI1Kv43 + C0C1 * C0Kv43; d[1] = a2 - a1;
    a1 = (C2C3 + C2C1 + C2CI2) * C2Kv43; a2 = C3C2 * C3Kv43 + CI2C2 * CI2Kv43 + C1C2 * C1Kv43; d[2] = a2 - a1;
    a1 = (C3O + C3C2 + C3CI3) * C3Kv43; a2 = OC3 * OKv43 + CI3C3 * CI3Kv43 + C2C3 * C2Kv43; d[3] = a2 - a1;
    a1 = (OC3 + OOI) * OKv43; a2 = C3O * C3Kv43 + OIO * OIKv43; d[4] = a2 - a1;
    a1 = (CI0C0 + CI0CI1) * CI0Kv43; a2 = C0CI0 * C0Kv43 + CI1CI0 * CI1Kv43; d[5] = a2 - a1;
    a1 = (CI1CI2 + CI1C1 + CI1CI0) * CI1Kv43; a2 = CI2CI1 * CI2Kv43 + C1CI1 * C1Kv43 + CI0CI1 * CI0Kv43;
    d[6] = a2 - a1;
    a1 = (CI2CI3 + CI2C2 + CI2CI1) * CI2Kv43; a2 = CI3CI2 * CI3Kv43 + C2CI2 * C2Kv43 + CI1CI2 * CI1Kv43;
    d[7] = a2 - a1;
    a1 = (CI3OI + CI3C3 + CI3CI2) * CI3Kv43; a2 = OICI3 * OIKv43 + C3CI3 * C3Kv43 + CI2CI3 * CI2Kv43;
    d[8] = a2 - a1;
    F[GW_C0Kv43] = d[0]; F[GW_C1Kv43] = d[1]; F[GW_C2Kv43] = d[2]; F[GW_C3Kv43] = d[3]; F[GW_OKv43] = d[4];
    F[GW_CI0Kv43] = d[5]; F[GW_CI1Kv43] = d[6]; F[GW_CI2Kv43] = d[7]; F[GW_CI3Kv43] = d[8];
    F[GW_OIKv43] = -d[5] - d[6] - d[7] - d[8] - d[4] - d[0] - d[1] - d[2] - d[3];
  }
  /* ---- Kv1.4, fcn.c:927-998 ---- */
  {
    const double al = alphaa0Kv14 * tx->x[GW_X_14A], be = betaa0Kv14 * tx->x[GW_X_14B];
    const double ali = alphai0Kv14, bei = betai0Kv14;
    const double C0C1 = 4.0 * al, C1C2 = 3.0 * al, C2C3 = 2.0 * al, C3O = al;
    const double CI0CI1 = 4.0 * b1Kv14 * al, CI1CI2 = 3.0 * b2Kv14 * al / b1Kv14;
    const double CI2CI3 = 2.0 * b3Kv14 * al / b2Kv14, CI3OI = b4Kv14 * al / b3Kv14;
    const double C1C0 = be, C2C1 = 2.0 * be, C3C2 = 3.0 * be, OC3 = 4.0 * be;
    const double CI1CI0 = be / f1Kv14, CI2CI1 = 2.0 * f1Kv14 * be / f2Kv14;
    const double CI3CI2 = 3.0 * f2Kv14 * be / f3Kv14, OICI3 = 4.0 * f3Kv14 * be / f4Kv14;
    const double C0CI0 = bei, C1CI1 = f1Kv14 * bei, C2CI2 = f2Kv14 * bei, C3CI3 = f3Kv14 * bei, OOI = f4Kv14 * bei;
    const double CI0C0 = ali, CI1C1 = ali / b1Kv14, CI2C2 = ali / b2Kv14, CI3C3 = ali / b3Kv14, OIO = ali / b4Kv14;
    double d[9];
    a1 = (C0C1 + C0CI0) * C0Kv14; a2 = C1C0 * C1Kv14 + CI0C0 * CI0Kv14; d[0] = a2 - a1;
    a1 = (C1C2 + C1C0 + C1CI1) * C1Kv14; a2 = C2C1 * C2Kv14 + CI1C1 * CI1Kv14 + C0C1 * C0Kv14; d[1] = a2 - a1;
    a1 = (C2C3 + C2C1 + C2CI2) * C2Kv14; a2 = C3C2 * C3Kv14 + CI2C2 * CI2Kv14 + C1C2 * C1Kv14; d[2] = a2 - a1;
    a1 = (C3O + C3C2 + C3CI3) * C3Kv14; a2 = OC3 * OKv14 + CI3C3 * CI3Kv14 + C2C3 * C2Kv14; d[3] = a2 - a1;
    a1 = (OC3 + OOI) * OKv14; a2 = C3O * C3Kv14 + OIO * OIKv14; d[4] = a2 - a1;
    a1 = (CI0C0 + CI0CI1) * CI0Kv14; a2 = C0CI0 * C0Kv14 + CI1CI0 * CI1Kv14; d[5] = a2 - a1;
    a1 = (CI1CI2 + CI1C1 + CI1CI0) * CI1Kv14; a2 = CI2CI1 * CI2Kv14 + C1CI1 * C1Kv14 + CI0CI1 * CI0Kv14;
    d[6] = a2 - a1;
    a1 = (CI2CI3 + CI2C2 + CI2CI1) * CI2Kv14; a2 = CI3CI2 * CI3Kv14 + C2CI2 * C2Kv14 + CI1CI2 * CI1Kv14;
    d[7] = a2 - a1;
    a1 = (CI3OI + CI3C3 + CI3CI2) * CI3Kv14; a2 = OICI3 * OIKv14 + C3CI3 * C3Kv14 + CI2CI3 * CI2Kv14;
    d[8] = a2 - a1;
    F[GW_C0Kv14] = d[0]; F[GW_C1Kv14] = d[1]; F[GW_C2Kv14] = d[2]; F[GW_C3Kv14] = d[3]; F[GW_OKv14] = d[4];
    F[GW_CI0Kv14] = d[5]; F[GW_CI1Kv14] = d[6]; F[GW_CI2Kv14] = d[7]; F[GW_CI3Kv14] = d[8];
    F[GW_OIKv14] = -d[5] - d[6] - d[7] - d[8] - d[4] - d[0] - d[1] - d[2] - d[3];
  }

  F[GW_V] = dV; F[GW_mNa] = dmNa; F[GW_hNa] = dhNa; F[GW_jNa] = djNa; F[GW_Nai] = dNai; F[GW_Ki] = dKi;
  F[GW_Cai] = dCai; F[GW_CaNSR] = dCaNSR; F[GW_xKs] = dxKs; F[GW_LTRPNCa] = dLTRPNCa; F[GW_HTRPNCa] = dHTRPNCa;
  F[GW_CaTOT] = dCaTOT; F[GW_C1Herg] = dC1Herg; F[GW_C2Herg] = dC2Herg; F[GW_C3Herg] = dC3Herg;
  F[GW_OHerg] = dOHerg;
  F[GW_IHerg] = -dC1Herg - dC2Herg - dC3Herg - dOHerg;

  if (keepc) {
    current[GW_I_INa] = INa; current[GW_I_IKr] = IKr; current[GW_I_IKs] = IKs; current[GW_I_Ito1] = Ito1;
    current[GW_I_IK1] = IK1; current[GW_I_IKp] = IKp; current[GW_I_INaCa] = INaCa; current[GW_I_INaK] = INaK;
    current[GW_I_IpCa] = IpCa; current[GW_I_ICab] = ICab; current[GW_I_INab] = INab; current[GW_I_ICa] = ICa;
    current[GW_I_JDHPR] = ICa * Acap / (-2.0 * Vmyo * Faraday * 1000.0);
    current[GW_I_Jup] = Jup; current[GW_I_Jtrpn] = Jtrpn;
    current[GW_I_Jtr] = Jtr * VJSR / Vmyo; current[GW_I_Jxfer] = Jxfer * VSS / Vmyo;
    current[GW_I_IKv43] = IKv43; current[GW_I_IKv14] = IKv14; current[GW_I_IKv14_K] = IKv14_K;
    current[GW_I_IKv14_Na] = IKv14_Na; current[GW_I_Ito2] = Ito2; current[GW_I_Istim] = Istim;
    current[GW_I_Itot] = Itot;
  }
}

/* The transcendental terms for the state at `time`, one after another. */
GW_HD void gw_tx_fill(const double time, const double* state, const gw_protocol* P, gw_tx* tx) {
  double Istim;
  const double V = gw_fcn_voltage(time, state, P, &Istim);
  int k;
  for (k = 0; k < GW_NX; k++) tx->x[k] = exp(gw_x_arg(k, V));
  for (k = 0; k < 4; k++) tx->lg[k] = log(gw_lg_arg(k, state));
  for (k = 0; k < 6; k++) {
    double y;
    const double b = gw_pw_arg(k, state, &y);
    tx->pw[k] = pow(b, y);
  }
  tx->k1 = exp(gw_k1_arg(V, tx->lg));
}

/* Global right-hand side (fcn.c:29-1072): gw_fcn_tx with the terms
 * evaluated in turn. */
GW_HD void gw_fcn(const double time, double* state, double* F, double* current, const int keepc,
                  const double Jxfer, const double Jtr, const double ICa, const double Ito2, const gw_protocol* P) {
  gw_tx tx;
  gw_tx_fill(time, state, P, &tx);
  gw_fcn_tx(time, state, F, current, keepc, Jxfer, Jtr, ICa, Ito2, P, &tx);
}

/* Rest state of initialize_state.c:167-203 (37 globals). */
GW_HD void gw_rest_state(double* s) {
  s[GW_V] = -0.9543106E+02; s[GW_mNa] = 0.2654309E-03; s[GW_hNa] = 0.9985519E+00; s[GW_jNa] = 0.9987711E+00;
  s[GW_Nai] = 0.1000000E+02; s[GW_Ki] = 0.1554636E+03; s[GW_Cai] = 0.7954739E-04; s[GW_CaNSR] = 0.176e0;
  s[GW_xKs] = 0.1501720E-03; s[GW_LTRPNCa] = 0.7485195E-01; s[GW_HTRPNCa] = 0.9748885E+00;
  s[GW_C0Kv43] = 0.590958E+00; s[GW_C1Kv43] = 0.155217E+00; s[GW_C2Kv43] = 0.152881E-01;
  s[GW_C3Kv43] = 0.669242E-03; s[GW_OKv43] = 0.109861E-04; s[GW_CI0Kv43] = 0.220999E-00;
  s[GW_CI1Kv43] = 0.143513E-01; s[GW_CI2Kv43] = 0.596808E-03; s[GW_CI3Kv43] = 0.642013E-04;
  s[GW_OIKv43] = 0.184528E-02; s[GW_C0Kv14] = 0.7646312E+00; s[GW_C1Kv14] = 0.7393727E-01;
  s[GW_C2Kv14] = 0.2681076E-02; s[GW_C3Kv14] = 0.4321218E-04; s[GW_OKv14] = 0.2620394E-06;
  s[GW_CI0Kv14] = 0.1493312E+00; s[GW_CI1Kv14] = 0.6441895E-02; s[GW_CI2Kv14] = 0.2012634E-02;
  s[GW_CI3Kv14] = 0.6128624E-03; s[GW_OIKv14] = 0.3084292E-03; s[GW_CaTOT] = 0.7417606475E+01;
  s[GW_C1Herg] = 0.99e+00; s[GW_C2Herg] = 0.8e-02; s[GW_C3Herg] = 0.2e-02; s[GW_OHerg] = 0.0e+00;
  s[GW_IHerg] = 0.0e+00;
}

/* Total cell Ca (femtomoles) from compartment sums, initialize_state.c:233-246
 * (the same expression is CaTOT2 of mpi_master.c:180-184).  sum_jsr and
 * sum_ss are the buffered-Ca sums over FRUs. */
GW_HD double gw_catot(double sum_jsr_tot, double sum_ss_tot, double nfru_scale, const double* s) {
  return 1.e6 * ((sum_jsr_tot * GWC_VJSR + sum_ss_tot * GWC_VSS) * nfru_scale + s[GW_CaNSR] * GWC_VNSR +
                 s[GW_Cai] * GWC_Vmyo *
                     (1.0 + GWC_CMDNtot / (GWC_KmCMDN + s[GW_Cai]) + GWC_EGTAtot / (GWC_KmEGTA + s[GW_Cai])) +
                 (s[GW_LTRPNCa] * GWC_LTRPNtot + s[GW_HTRPNCa] * GWC_HTRPNtot) * GWC_Vmyo);
}

/* Output quantities from the 11 FRU sums (mpi_master.c:175-190).  The
 * CaJSRtot / CaSStot slots keep the reference's swapped assignment. */
GW_HD void gw_otherstates(const double num[11], int nfru, double nfru_scale, const double* s, double* o) {
  const double n4 = (double)(nfru * 4);
  o[GW_O_CaSSavg] = num[0] / n4;
  o[GW_O_CaJSRavg] = num[1] / (double)(nfru);
  o[GW_O_JRyRtot] = num[2] * nfru_scale * GWC_VSS / GWC_Vmyo;
  o[GW_O_PRyR_Open] = num[3] / (double)(5 * 4 * nfru);
  o[GW_O_PRyR_ready] = (double)(num[4]) / (double)(5 * 4 * nfru);
  o[GW_O_CaTOT2] = 1.e6 * ((num[5] * GWC_VSS + num[6] * GWC_VJSR) * nfru_scale + s[GW_CaNSR] * GWC_VNSR +
                           s[GW_Cai] * GWC_Vmyo *
                               (1.0 + GWC_CMDNtot / (GWC_KmCMDN + s[GW_Cai]) +
                                GWC_EGTAtot / (GWC_KmEGTA + s[GW_Cai])) +
                           (s[GW_LTRPNCa] * GWC_LTRPNtot + s[GW_HTRPNCa] * GWC_HTRPNtot) * GWC_Vmyo);
  o[GW_O_PNorm_Mode] = num[7] / n4;
  o[GW_O_PnotVinact] = num[8] / n4;
  o[GW_O_PLType_Open] = num[9] / n4;
  o[GW_O_PIto2_Open] = num[10] / n4;
  o[GW_O_CaJSRtot] = 1.e6 * num[5] * GWC_VSS * nfru_scale;
  o[GW_O_CaSStot] = 1.e6 * num[6] * GWC_VJSR * nfru_scale;
}

#endif /* GW_CELL_MODEL_H */
