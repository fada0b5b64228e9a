// Device model of one Ca2+ release unit (FRU): constants, MT19937 stream,
// channel exit rates, local Ca ODE and the channel-state packing.
//
// FP64 arithmetic keeps the operand order of the reference so that, compiled
// with -fmad=false, results agree with the reference bit for bit wherever
// CUDA's exp() agrees with the host libm's.
//
// Reference: simfru_local.c, fru_rates_local.c, fcn_fru.c, mt19937_local.c,
// parameters_fcn_fru.c (citations at each function).
#pragma once
#include <stdint.h>

namespace gw {

constexpr int kClefts = 4;          // parameters.h:30
constexpr int kRyR = 5;             // parameters.h:37
constexpr int kMtN = 624;           // parameters.h:64
constexpr int kMtM = 397;           // mt19937_local.c:60
constexpr int kMtStride = 640;      // words per FRU row (2560 B, 128-B aligned rows)

// ---- physical constants: parameters_fcn_fru.c:21-90 --------------------------
constexpr double Cao = 2.0, Clo = 150.0, Cli = 20.0;
constexpr double Faraday = 96.5;
constexpr double RT_over_F = 8.314 * 310.0 / 96.5;
constexpr double Acap = 1.534e-4;
constexpr double VJSR = (((double)kClefts) * 0.53 * 0.5 * 0.2 * 1.05e-10);
constexpr double VSS = (0.5 * 0.2 * 2.03e-12);
constexpr double PCa = (1.5 / 2.8 * 0.2 * 0.9 * 0.9468e-11);
constexpr double PCl = 2.65e-15;
constexpr double BSLtot = 1.124, CSQNtot = 13.5, BSRtot = 0.047;
constexpr double KBSL = 0.0087, KmCSQN = 0.63, KBSR = 0.00087;
constexpr double JRyRmax = (0.6 * 1.5 * 1.1 * 3.96);
constexpr double tautr = 3.0, tauxfer = 0.005, tauss2ss = (10.0 * 0.005);

// ---- LCC modal gating: fru_rates_local.c:50-86 --------------------------------
constexpr double fL = 0.85, gL = 2.0, fLprime = 0.005, gLprime = 7.0;
constexpr double bL = 1.9356, aL = 2.0, kappa = 1.0;
constexpr double omega = 0.83 * 2.0 * 1.3 * 0.01;
constexpr double alphacf = 4.0 * 1.2 * 0.416;
constexpr double betacf = 4.0 * 0.45 * 0.049;
constexpr double gammacf = 0.83 * 1.9 * 1.3 * 0.31 * 7.5 * 0.09233;
constexpr double CCa0_to_C0 = kappa * kappa * kappa * kappa * omega;
constexpr double CCa1_to_C1 = kappa * kappa * kappa * omega / bL;
constexpr double CCa2_to_C2 = kappa * kappa * omega / (bL * bL);
constexpr double CCa3_to_C3 = kappa * omega / (bL * bL * bL);
constexpr double CCa4_to_C4 = omega / (bL * bL * bL * bL);
// ---- Ca-activated Cl channel: :94-96 ------------------------------------------
constexpr double kbIto2 = 2.0;
constexpr double kfIto2 = 2.0 / 0.1502;
// ---- RyR: :100-121 --------------------------------------------------------------
constexpr double k21 = 250.0, k32 = 9.6, k43 = 0.07 / 0.06667 * 13.0, k45 = 0.07;
constexpr double k52 = 0.001235, k65 = 30.0;
constexpr double k12cf = 3000.0, k23cf = 10.0 * 30000.0, k34cf = 0.6 * 3000.0;
constexpr double k54cf = 0.6 * 0.198, k25cf = 10.0 * 300.0, k56cf = 2.0 * 4.0 * 3000.0;
constexpr double k_rate = 0.00127215, k_rate2 = 3.4188;
constexpr double threshCa34to7 = 0.0368369379834969;
constexpr double threshCa56to8 = 0.00011447933531005;
constexpr double threshMAX = 2.0, threshMAXCa = 0.0504410547074504;

// a / b for the rate rows (correctly rounded in FP64 and in FP32)
__device__ __forceinline__ double fdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float fdiv(float a, float b) { return a / b; }

__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }

// ---- channel-state packing: one 32-bit word per cleft, eight 4-bit fields ----
//   bits 0-3 LCC state (1..12), 4-7 VDI gate (1..2), 8-27 RyR 0..4 (1..8),
//   28-31 Cl channel (1..2)
__device__ __forceinline__ int lcc_of(uint32_t w) { return w & 15u; }
__device__ __forceinline__ int vdi_of(uint32_t w) { return (w >> 4) & 15u; }
__device__ __forceinline__ int ryr_of(uint32_t w, int i) { return (w >> (8 + 4 * i)) & 15u; }
__device__ __forceinline__ int cl_of(uint32_t w) { return w >> 28; }
__device__ __forceinline__ uint32_t set_field(uint32_t w, int shift, int v) {
  return (w & ~(15u << shift)) | ((uint32_t)v << shift);
}
__device__ __forceinline__ bool lcc_open(uint32_t w) {
  int s = lcc_of(w);
  return (s == 6 || s == 12) && vdi_of(w) == 2;  // simfru_local.c:103-104
}
__device__ __forceinline__ bool ryr_open(int s) { return s == 3 || s == 4 || s == 7; }
__device__ __forceinline__ int ryr_open_count(uint32_t w) {
  int n = 0;
#pragma unroll
  for (int i = 0; i < kRyR; i++) n += ryr_open(ryr_of(w, i));
  return n;
}

// ---- MT19937 stream of one FRU: mt19937_local.c:76-240 ----------------------
// Words live in a per-FRU row of global memory; mti is held by the caller.
__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

// In-place regeneration of all 624 words (the "twist").
__device__ __forceinline__ void mt_regenerate(uint32_t* m) {
  uint32_t cur = m[0];
  for (int k = 0; k < kMtN - kMtM; k++) {
    uint32_t nxt = m[k + 1];
    uint32_t y = (cur & 0x80000000u) | (nxt & 0x7fffffffu);
    m[k] = m[k + kMtM] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    cur = nxt;
  }
  for (int k = kMtN - kMtM; k < kMtN - 1; k++) {
    uint32_t nxt = m[k + 1];
    uint32_t y = (cur & 0x80000000u) | (nxt & 0x7fffffffu);
    m[k] = m[k + kMtM - kMtN] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    cur = nxt;
  }
  uint32_t y = (cur & 0x80000000u) | (m[0] & 0x7fffffffu);
  m[kMtN - 1] = m[kMtM - 1] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

// Per-FRU MT context with copy-on-twist protection of the saved generation:
// the first regeneration after a save copies the words to `hold` and stamps
// `hold_epoch`, so a rejected Dormand-Prince step can restore them.
struct MtRef {
  uint32_t* m;
  uint32_t* hold;
  uint32_t* hold_epoch;
  uint32_t epoch;
  int mti;
  __device__ __forceinline__ uint32_t next_word() {
    if (mti >= kMtN) {
      if (*hold_epoch != epoch) {
        for (int k = 0; k < kMtN; k++) hold[k] = m[k];
        *hold_epoch = epoch;
      }
      mt_regenerate(m);
      mti = 0;
    }
    return mt_temper(m[mti++]);
  }
  // reals in [0,1): y / 2^32 (mt19937_local.c:113)
  __device__ __forceinline__ double next() { return (double)next_word() / 4294967296.0; }
};

// ---- LCC: total exit rate and exit row (fru_rates_local.c:131-341) ----------
// Rows are templates on the arithmetic type: double for the plain method,
// float for the mixed-precision one (same expressions, rounded in T).
template <typename T>
struct LccBasisT { T alpha, beta, bp; };
using LccBasis = LccBasisT<double>;

__device__ __forceinline__ LccBasis lcc_basis(double V) {
  LccBasis b;
  b.alpha = alphacf * exp(0.012 * (V - 35.0));
  b.beta = betacf * exp(-0.05 * (V - 35.0));
  b.bp = b.beta / (bL * kappa);
  return b;
}

// Exit row of state s: r[0] = total in the reference's summation order,
// r[1..len-1] with destinations d[1..len-1].
template <typename T>
__device__ __forceinline__ int lcc_row(int s, const LccBasisT<T>& b, T gam, T r[4], int d[4]) {
  const T ap = T(aL) * b.alpha;
  switch (s) {
    case 1: r[1] = T(4.0) * b.alpha; d[1] = 2; r[2] = gam; d[2] = 7; r[0] = r[1] + r[2]; return 3;
    case 2: r[1] = b.beta; d[1] = 1; r[2] = T(3.0) * b.alpha; d[2] = 3; r[3] = T(aL) * gam; d[3] = 8;
      r[0] = r[1] + r[2] + r[3]; return 4;
    case 3: r[1] = T(2.0) * b.beta; d[1] = 2; r[2] = T(2.0) * b.alpha; d[2] = 4; r[3] = T(aL * aL) * gam; d[3] = 9;
      r[0] = r[1] + r[2] + r[3]; return 4;
    case 4: r[1] = T(3.0) * b.beta; d[1] = 3; r[2] = b.alpha; d[2] = 5; r[3] = T(aL * aL * aL) * gam; d[3] = 10;
      r[0] = r[1] + r[2] + r[3]; return 4;
    case 5: r[1] = T(4.0) * b.beta; d[1] = 4; r[2] = T(fL); d[2] = 6; r[3] = T(aL * aL * aL * aL) * gam; d[3] = 11;
      r[0] = r[1] + r[2] + r[3]; return 4;
    case 6: r[0] = T(gL); r[1] = T(gL); d[1] = 5; return 2;
    case 7: r[1] = T(CCa0_to_C0); d[1] = 1; r[2] = T(4.0) * ap; d[2] = 8; r[0] = r[2] + r[1]; return 3;
    case 8: r[1] = b.bp; d[1] = 7; r[2] = T(CCa1_to_C1); d[2] = 2; r[3] = T(3.0) * ap; d[3] = 9;
      r[0] = r[1] + r[3] + r[2]; return 4;
    case 9: r[1] = T(2.0) * b.bp; d[1] = 8; r[2] = T(CCa2_to_C2); d[2] = 3; r[3] = T(2.0) * ap; d[3] = 10;
      r[0] = r[1] + r[3] + r[2]; return 4;
    case 10: r[1] = T(3.0) * b.bp; d[1] = 9; r[2] = T(CCa3_to_C3); d[2] = 4; r[3] = ap; d[3] = 11;
      r[0] = r[1] + r[3] + r[2]; return 4;
    case 11: r[1] = T(4.0) * b.bp; d[1] = 10; r[2] = T(CCa4_to_C4); d[2] = 5; r[3] = T(fLprime); d[3] = 12;
      r[0] = r[1] + r[2] + r[3]; return 4;
    case 12: r[0] = T(gLprime); r[1] = T(gLprime); d[1] = 11; return 2;
    default: r[0] = T(0); return 1;
  }
}

__device__ __forceinline__ double lcc_total(int s, const LccBasis& b, double gam) {
  double r[4];
  int d[4];
  lcc_row(s, b, gam, r, d);
  return r[0];
}

// ---- RyR: per-cleft constants and rows (fru_rates_local.c:374-736) ----------
template <typename T>
struct RyrKT { T k12, k23, k34, k54, k25, k56; int regime; };
using RyrK = RyrKT<double>;

__device__ __forceinline__ RyrK ryr_constants(double cass) {
  RyrK k;
  const double sat = dmin(threshMAX, (cass * cass) / k_rate);
  const double sat2 = dmin(threshMAX, (cass * cass) / k_rate2);
  const double c = dmin(cass, threshMAXCa);
  k.k12 = k12cf * sat2;
  k.k23 = k23cf * sat;
  k.k34 = k34cf * sat;
  k.k54 = k54cf * sat;
  k.k25 = k25cf * sat;
  k.k56 = k56cf * sat;
  k.regime = (c < threshCa56to8) ? 0 : ((c < threshCa34to7) ? 1 : 2);
  return k;
}

// Merged pseudo-states of the three Ca regimes: state 7 = {3,4}, 8 = {5,6}.
// Rewrites s before the rates are formed; may draw one uniform.
__device__ __forceinline__ int ryr_resolve(int s, const RyrK& k, MtRef& rng) {
  if (k.regime == 0) {
    if (s == 7) s = (rng.next() < (k.k34 / (k.k34 + k43))) ? 4 : 3;
    else if (s == 8) s = (rng.next() < k.k56 / (k.k56 + k65)) ? 6 : 5;
  } else if (k.regime == 1) {
    if (s == 7) s = (rng.next() < k.k34 / (k.k34 + k43)) ? 4 : 3;
    if (s == 5 || s == 6) s = 8;
  } else {
    if (s == 3 || s == 4) s = 7;
    else if (s == 5 || s == 6) s = 8;
  }
  return s;
}

// Exit row of a resolved RyR state.
template <typename T>
__device__ __forceinline__ int ryr_row(int s, const RyrKT<T>& k, T r[4], int d[4]) {
  const int g = k.regime;
  switch (s) {
    case 1: r[0] = k.k12; r[1] = k.k12; d[1] = 2; return 2;
    case 2: r[1] = T(k21); d[1] = 1; r[2] = k.k23; d[2] = (g == 2) ? 7 : 3; r[3] = k.k25; d[3] = (g == 0) ? 5 : 8;
      r[0] = T(k21) + k.k23 + k.k25; return 4;
    case 3: r[1] = T(k32); d[1] = 2; r[2] = k.k34; d[2] = 4; r[0] = T(k32) + k.k34; return 3;
    case 4: r[1] = T(k43); d[1] = 3; r[2] = T(k45); d[2] = (g == 0) ? 5 : 8; r[0] = T(k43) + T(k45); return 3;
    case 5: r[1] = T(k52); d[1] = 2; r[2] = k.k54; d[2] = 4; r[3] = k.k56; d[3] = 6;
      r[0] = T(k52) + k.k54 + k.k56; return 4;
    case 6: r[0] = T(k65); r[1] = T(k65); d[1] = 5; return 2;
    case 7: {
      const T a1 = fdiv(k.k34, T(k43) + k.k34);
      r[1] = (T(1) - a1) * T(k32); d[1] = 2; r[2] = a1 * T(k45); d[2] = 8; r[0] = r[1] + r[2]; return 3;
    }
    case 8: {
      const T a1 = fdiv(T(k65), k.k56 + T(k65));
      r[1] = a1 * T(k52); d[1] = 2; r[2] = a1 * k.k54; d[2] = (g == 2) ? 7 : 4; r[0] = r[1] + r[2]; return 3;
    }
    default: r[0] = T(0); return 1;
  }
}

__device__ __forceinline__ double ryr_total(int s, const RyrK& k) {
  double r[4];
  int d[4];
  ryr_row(s, k, r, d);
  return r[0];
}

// ---- local Ca ODE: fcn_fru.c:23-137 -----------------------------------------
// y = (CaJSR, CaSS1..4), dep = (V, Cai, CaNSR); lopen = LCC open flags (0/1),
// nopen = open RyRs per cleft.
__device__ __forceinline__ void fcn_fru(const double y[5], const double dep[3], const double lopen[kClefts],
                                        const int nopen[kClefts], double dy[5]) {
  const double JDHconstant = 1.0 / (2.0 * VSS * Faraday * 1000.0);
  const double V = dep[0], Cai = dep[1], CaNSR = dep[2], CaJSR = y[0];
  double JRyR[kClefts], Jss[kClefts];
  const double Jtr = (CaNSR - CaJSR) / tautr;
#pragma unroll
  for (int c = 0; c < kClefts; c++) JRyR[c] = JRyRmax * ((double)nopen[c]) * (CaJSR - y[c + 1]);
  const double JRyRtot = JRyR[0] + JRyR[1] + JRyR[2] + JRyR[3];
#pragma unroll
  for (int c = 0; c < kClefts; c++) Jss[c] = (y[c + 1] - y[(c + 1) % kClefts + 1]) / tauss2ss;
  const double VFRT = V / RT_over_F;
  const double VFsqRT = (1000.0 * Faraday) * VFRT;
  const double e2 = exp(2.0 * VFRT);
  const bool small = fabs(V) < 1.e-6;
  const double a2j = small ? 0.0 : PCa * 4.0 * VFsqRT / (e2 - 1.0) * JDHconstant;
  {
    const double a1 = CSQNtot * KmCSQN / ((CaJSR + KmCSQN) * (CaJSR + KmCSQN));
    const double bJSR = 1.0 / (1.0 + a1);
    dy[0] = bJSR * (Jtr - VSS / VJSR * JRyRtot);
  }
#pragma unroll
  for (int c = 0; c < kClefts; c++) {
    const double cs = y[c + 1];
    const double JDH = small ? -PCa * 2.0 * 1000.0 * Faraday * (cs - Cao * 0.341) * lopen[c] * JDHconstant
                             : -(cs * e2 - Cao * 0.341) * a2j * lopen[c];
    const double Jxfer = (cs - Cai) / tauxfer;
    const double a1 = BSRtot * KBSR / ((cs + KBSR) * (cs + KBSR));
    const double a2 = BSLtot * KBSL / ((cs + KBSL) * (cs + KBSL));
    const double bSS = 1.0 / (1.0 + a1 + a2);
    dy[c + 1] = bSS * (JDH + JRyR[c] - Jxfer - Jss[c] + Jss[(c + kClefts - 1) % kClefts]);
  }
}

}  // namespace gw
