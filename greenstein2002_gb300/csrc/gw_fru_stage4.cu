// Cleft-parallel FP64 FRU stage kernel: each FRU is advanced by a group of
// four lanes, one per dyadic cleft (8 FRUs per warp).
//
// Why: on GB300 every SM sub-partition issues one FP64 warp instruction per
// 64 cycles whatever the active-lane mask, so a stage lasts as long as the
// FP64 instruction chain of its slowest FRU.  Spreading an FRU over its four
// clefts divides that chain by about four at the same total FP64 work, and
// the arithmetic below is arranged to issue as few FP64 instructions as
// possible while staying bit-identical to the reference's operations:
//   - divisions by constants use Markstein's correction (q = x*r;
//     q += fma(-q, d, x)*r), which returns the correctly rounded quotient;
//   - max/min of non-negative doubles compare their bit patterns as integers;
//   - channel exit totals come from per-state coefficient tables instead of
//     divergent switches;
//   - uniforms are compared with thresholds in the integer domain
//     (u = y/2^32 > P  <=>  y > floor(P*2^32));
//   - the four voltage exponentials of a substep are computed one per lane,
//     and exp(2VF/RT) at the end of a substep is reused at the start of the
//     next.
//
// Reference: simfru_local.c:32-278, fru_rates_local.c:30-798, fcn_fru.c:23-137,
// mt19937_local.c:97-240, calc_fru_flux_local.c:28-77, mpi_master.c:447-468,
// mpi_slave.c:150-226.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gw_fru_core.cuh"
#include "gw_fru_model.cuh"
#include "gw_kernels.h"

namespace gw {
namespace c4 {

constexpr unsigned kFull = 0xffffffffu;

// correctly rounded x/d for a constant d, with r = RN(1/d)
__device__ __forceinline__ double divc(double x, double d, double r) {
  const double q = x * r;
  return fma(fma(-q, d, x), r, q);
}
// max/min of doubles known to be >= 0 (or of a negative value against a
// positive constant): IEEE order equals signed integer order of the bits;
// ties return the first argument like the reference's macros
__device__ __forceinline__ double imax(double a, double b) {
  return __double_as_longlong(a) < __double_as_longlong(b) ? b : a;
}
__device__ __forceinline__ double imin(double a, double b) {
  return __double_as_longlong(a) < __double_as_longlong(b) ? a : b;
}
__device__ __forceinline__ bool ilt(double a, double b) { return __double_as_longlong(a) < __double_as_longlong(b); }

// u = y/2^32 compared with P in [0, 1]:  u > P  and  u >= P, in integers.
__device__ __forceinline__ void thresh(double P, uint64_t& fl, bool& exact) {
  const uint64_t b = (uint64_t)__double_as_longlong(P);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  const uint64_t M = (b & 0xfffffffffffffull) | (1ull << 52);
  const int sh = 20 - e;  // floor(P * 2^32) = M >> (52 - 32 - e)
  if (P <= 0.0) {         // never on valid input (dt*rate <= 0.1); keeps u > P true
    fl = 0;
    exact = false;
    return;
  }
  if (sh >= 64) {
    fl = 0;
    exact = (M == 0);
  } else {
    fl = M >> sh;
    exact = (M & ((1ull << sh) - 1ull)) == 0ull;
  }
}
__device__ __forceinline__ bool u_gt(uint32_t y, double P) {
  if (P <= 0.0) return true;
  uint64_t fl;
  bool ex;
  thresh(P, fl, ex);
  return (uint64_t)y > fl;
}
__device__ __forceinline__ bool u_ge(uint32_t y, double P) {
  if (P <= 0.0) return true;
  uint64_t fl;
  bool ex;
  thresh(P, fl, ex);
  return (uint64_t)y > fl || (ex && (uint64_t)y == fl);
}

// LCC exit total = (cX*bX + cY*bY) + cZ*bZ with bases {1, alpha, beta,
// gamma, alpha', beta'}: the sums of fru_rates_local.c:176-340 in their order.
__constant__ double c_lcc_coef[13][3] = {
    {0.0, 0.0, 0.0},
    {4.0, 1.0, 0.0},                     // 1: 4a + g
    {1.0, 3.0, aL},                      // 2: b + 3a + aL g
    {2.0, 2.0, aL * aL},                 // 3
    {3.0, 1.0, aL * aL * aL},            // 4
    {4.0, fL, aL * aL * aL * aL},        // 5
    {gL, 0.0, 0.0},                      // 6
    {4.0, CCa0_to_C0, 0.0},              // 7: 4a' + omega
    {1.0, 3.0, CCa1_to_C1},              // 8: b' + 3a' + omega/bL
    {2.0, 2.0, CCa2_to_C2},              // 9
    {3.0, 1.0, CCa3_to_C3},              // 10
    {4.0, CCa4_to_C4, fLprime},          // 11
    {gLprime, 0.0, 0.0},                 // 12
};
// basis index of each term, packed 3 x 4 bits per state:
// 0 = 1, 1 = alpha, 2 = beta, 3 = gamma, 4 = alpha', 5 = beta'
__constant__ uint16_t c_lcc_basis[13] = {
    0x000, 0x031, 0x312, 0x312, 0x312, 0x302, 0x000, 0x004, 0x045, 0x045, 0x045, 0x005, 0x000,
};

__device__ __forceinline__ double pick_basis(int i, double al, double be, double ga, double ap, double bp) {
  double v = 1.0;
  v = (i == 1) ? al : v;
  v = (i == 2) ? be : v;
  v = (i == 3) ? ga : v;
  v = (i == 4) ? ap : v;
  v = (i == 5) ? bp : v;
  return v;
}

struct Group {
  int c;           // cleft of this lane (0..3)
  int base;        // lane index of cleft 0 of this FRU within the warp
  unsigned mask;   // the four lanes of this FRU
};

// group-local shuffles (the four lanes of one FRU may run while other
// groups of the warp have finished their substeps)
template <typename T>
__device__ __forceinline__ T from(const Group& g, T v, int c) {
  return __shfl_sync(g.mask, v, g.base + c);
}
__device__ __forceinline__ double gmax(const Group& g, double v) {
  v = imax(v, __shfl_xor_sync(g.mask, v, 1));
  v = imax(v, __shfl_xor_sync(g.mask, v, 2));
  return v;
}

// Cooperative in-place regeneration of an FRU's 624 words by its 4 lanes, in
// chunks of 4 consecutive words.  Words k >= 227 depend on words the same
// regeneration produced 227 positions earlier (other lanes), so the group
// synchronises after every chunk.
__device__ __forceinline__ void regen4(uint32_t* m, const Group& g) {
  for (int k0 = 0; k0 < kMtN; k0 += 4) {
    const int k = k0 + g.c;
    const uint32_t cur = m[k];
    const uint32_t nxt = m[(k + 1 == kMtN) ? 0 : k + 1];
    const uint32_t far = m[(k + kMtM) % kMtN];
    __syncwarp(g.mask);
    const uint32_t y = (cur & 0x80000000u) | (nxt & 0x7fffffffu);
    m[k] = far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    __syncwarp(g.mask);
  }
}
__device__ __forceinline__ void copy4(uint32_t* dst, const uint32_t* src, const Group& g) {
  for (int k = g.c; k < kMtN; k += 4) dst[k] = src[k];
  __syncwarp(g.mask);
}

struct StageCtx {
  const StageParams* p;
  uint32_t* m;          // MT row of this FRU
  uint32_t* hold;       // copy-on-twist row
  uint32_t* hold_epoch;
};

// Fetch the words of one substep: E_tot extra draws (lane c owns positions
// pre .. pre+ne-1) followed by the 32 batch draws (lane c owns 8c .. 8c+7),
// regenerating the row in between when the stream crosses word 624.
__device__ __forceinline__ void fetch_words(const StageCtx& sc, const Group& g, int& mti, int pre, int ne, int etot,
                                            uint32_t ex[kRyR], uint32_t bw[8]) {
  const int W = etot + 32;
  const bool cross = (mti + W > kMtN);
  int pos;
  // old generation first
#pragma unroll
  for (int i = 0; i < kRyR; i++) {
    pos = mti + pre + i;
    if (i < ne && pos < kMtN) ex[i] = sc.m[pos];
  }
#pragma unroll
  for (int k = 0; k < 8; k++) {
    pos = mti + etot + 8 * g.c + k;
    if (pos < kMtN) bw[k] = sc.m[pos];
  }
  if (cross) {
    const bool need_copy = *sc.hold_epoch != sc.p->epoch;
    __syncwarp(g.mask);  // every lane has read its old words and the epoch
    if (need_copy) {
      copy4(sc.hold, sc.m, g);
      if (g.c == 0) *sc.hold_epoch = sc.p->epoch;
    }
    regen4(sc.m, g);
#pragma unroll
    for (int i = 0; i < kRyR; i++) {
      pos = mti + pre + i;
      if (i < ne && pos >= kMtN) ex[i] = sc.m[pos - kMtN];
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
      pos = mti + etot + 8 * g.c + k;
      if (pos >= kMtN) bw[k] = sc.m[pos - kMtN];
    }
    mti = mti + W - kMtN;
  } else {
    mti = mti + W;
  }
#pragma unroll
  for (int i = 0; i < kRyR; i++) ex[i] = mt_temper(ex[i]);
#pragma unroll
  for (int k = 0; k < 8; k++) bw[k] = mt_temper(bw[k]);
}

// Local Ca ODE of one cleft (fcn_fru.c:23-137) evaluated by the FRU's four
// lanes.  Each lane returns dCaSS of its cleft; every lane returns the same
// dCaJSR.  e2 = exp(2 V F/RT) and a2j are passed in (shared by all lanes).
__device__ __forceinline__ void fcn_fru4(const Group& g, double cajsr, double cass, const double dep[3], double e2,
                                         double a2j, bool small, double lopen, int nopen, double& dJSR, double& dSS) {
  constexpr double JDHconstant = 1.0 / (2.0 * VSS * Faraday * 1000.0);
  constexpr double rtautr = 1.0 / tautr, rtauxfer = 1.0 / tauxfer, rtauss = 1.0 / tauss2ss;
  const double Cai = dep[1], CaNSR = dep[2];
  // JRyR of every cleft, summed in cleft order
  const double jcoef = JRyRmax * (double)nopen;  // exact small-integer multiple
  const double JRyR = jcoef * (cajsr - cass);
  const double j0 = from(g, JRyR, 0), j1 = from(g, JRyR, 1), j2 = from(g, JRyR, 2), j3 = from(g, JRyR, 3);
  const double JRyRtot = j0 + j1 + j2 + j3;
  const double cnext = from(g, cass, (g.c + 1) & 3);
  const double Jss = divc(cass - cnext, tauss2ss, rtauss);
  const double Jss_prev = from(g, Jss, (g.c + 3) & 3);
  const double Jxfer = divc(cass - Cai, tauxfer, rtauxfer);
  const double JDH = small ? -PCa * 2.0 * 1000.0 * Faraday * (cass - Cao * 0.341) * lopen * JDHconstant
                           : -(cass * e2 - Cao * 0.341) * a2j * lopen;
  double a1 = BSRtot * KBSR / ((cass + KBSR) * (cass + KBSR));
  double a2 = BSLtot * KBSL / ((cass + KBSL) * (cass + KBSL));
  const double bSS = 1.0 / (1.0 + a1 + a2);
  dSS = bSS * (JDH + JRyR - Jxfer - Jss + Jss_prev);
  const double Jtr = divc(CaNSR - cajsr, tautr, rtautr);
  a1 = CSQNtot * KmCSQN / ((cajsr + KmCSQN) * (cajsr + KmCSQN));
  const double bJSR = 1.0 / (1.0 + a1);
  dJSR = bJSR * (Jtr - VSS / VJSR * JRyRtot);
}

// exp(2 V F / RT) and the GHK factor a2 of fcn_fru.c:78-101 for voltage V
__device__ __forceinline__ void ghk_terms(double V, double& e2, double& a2j, bool& small) {
  constexpr double JDHconstant = 1.0 / (2.0 * VSS * Faraday * 1000.0);
  constexpr double rRT = 1.0 / RT_over_F;
  const double VFRT = divc(V, RT_over_F, rRT);
  const double VFsqRT = (1000.0 * Faraday) * VFRT;
  e2 = exp(2.0 * VFRT);
  small = fabs(V) < 1.e-6;
  a2j = small ? 0.0 : PCa * 4.0 * VFsqRT / (e2 - 1.0) * JDHconstant;
}

// One FRU over [t0, tf] by its four lanes (simfru_local.c:83-277).
__device__ __forceinline__ void advance4(const StageCtx& sc, const Group& g, double& cajsr, double& cass, uint32_t& w,
                                         int& mti, uint32_t& nsub, bool& overflow) {
  const StageParams& p = *sc.p;
  double dep[3];
#pragma unroll
  for (int i = 0; i < 3; i++) dep[i] = p.dep0[i];
  double lopen = lcc_open(w) ? 1.0 : 0.0;
  int nopen = ryr_open_count(w);
  const double interval = p.tf - p.t0;
  double t = p.t0;
  double e2, a2j;
  bool small;
  ghk_terms(dep[0], e2, a2j, small);
  // per-lane voltage exponential of the rates: alpha, beta, yCa_inf, tau_yCa
  //   lane 0: alphacf*exp(0.012*(V-35))     lane 1: betacf*exp(-0.05*(V-35))
  //   lane 2: 0.4/(1+exp((V+12.5)/5)) + 0.6  lane 3: 60 + 340/(1+exp((V+30)/12))
  const bool isdiv = g.c >= 2;
  const double cA = isdiv ? (g.c == 2 ? 12.5 : 30.0) : -35.0;
  const double cR = isdiv ? (g.c == 2 ? 1.0 / 5.0 : 1.0 / 12.0) : (g.c == 0 ? 0.012 : -0.05);
  const double cD = isdiv ? (g.c == 2 ? 5.0 : 12.0) : 1.0;
  const double cCF = isdiv ? 0.0 : (g.c == 0 ? alphacf : betacf);
  const double cK = isdiv ? (g.c == 2 ? 0.4 : 340.0) : 1.0;
  const double cM = isdiv ? (g.c == 2 ? 1.0 - 0.4 : 60.0) : 0.0;
  while (true) {
    // the loop condition is uniform over the group (t is the same in all four lanes)
    if (!(t < p.tf)) break;
    if (nsub >= (1u << 22)) {
      overflow = true;
      break;
    }
    // ---- voltage terms at the substep start, one exponential per lane ----
    const double x = dep[0] + cA;
    double q = x * cR;
    if (isdiv) q = fma(fma(-q, cD, x), cR, q);
    const double ev = exp(q);
    const double r01 = cCF * ev;
    const double r23 = cK / (1.0 + ev) + cM;
    const double vterm = isdiv ? r23 : r01;
    const double alpha = from(g, vterm, 0), beta = from(g, vterm, 1);
    const double yinf = from(g, vterm, 2), tau = from(g, vterm, 3);
    constexpr double rbL = 1.0 / (bL * kappa);
    const double bp = divc(beta, bL * kappa, rbL);
    const double ap = aL * alpha;
    // ---- exit totals of this cleft's 8 channels ----
    const double cass0 = cass;
    const double gam = gammacf * cass;
    double R0[8];
    {
      const int s = lcc_of(w);
      const uint16_t bi = c_lcc_basis[s];
      const double X = c_lcc_coef[s][0] * pick_basis(bi & 15, alpha, beta, gam, ap, bp);
      const double Y = c_lcc_coef[s][1] * pick_basis((bi >> 4) & 15, alpha, beta, gam, ap, bp);
      const double Z = c_lcc_coef[s][2] * pick_basis((bi >> 8) & 15, alpha, beta, gam, ap, bp);
      R0[0] = X + Y + Z;
    }
    {
      const double num = (vdi_of(w) == 2) ? (1.0 - yinf) : yinf;
      R0[1] = num / tau;
    }
    // RyR constants of the cleft and the pseudo-state draws
    constexpr double rk_rate = 1.0 / k_rate, rk_rate2 = 1.0 / k_rate2;
    const double c2 = cass * cass;
    const double sat = imin(threshMAX, divc(c2, k_rate, rk_rate));
    const double sat2 = imin(threshMAX, divc(c2, k_rate2, rk_rate2));
    RyrK k;
    k.k12 = k12cf * sat2;
    k.k23 = k23cf * sat;
    k.k34 = k34cf * sat;
    k.k54 = k54cf * sat;
    k.k25 = k25cf * sat;
    k.k56 = k56cf * sat;
    {
      const double cc = imin(cass, threshMAXCa);
      k.regime = ilt(cc, threshCa56to8) ? 0 : (ilt(cc, threshCa34to7) ? 1 : 2);
    }
    // extra draws: regime 0 resolves 7 and 8, regime 1 resolves 7 (in cleft, then RyR order)
    int ne = 0;
#pragma unroll
    for (int i = 0; i < kRyR; i++) {
      const int s = ryr_of(w, i);
      ne += (k.regime == 0 && (s == 7 || s == 8)) || (k.regime == 1 && s == 7);
    }
    const int n0 = from(g, ne, 0), n1 = from(g, ne, 1), n2 = from(g, ne, 2), n3 = from(g, ne, 3);
    const int pre = (g.c > 0 ? n0 : 0) + (g.c > 1 ? n1 : 0) + (g.c > 2 ? n2 : 0);
    const int etot = n0 + n1 + n2 + n3;
    uint32_t exw[kRyR] = {0u, 0u, 0u, 0u, 0u}, bw[8];
    fetch_words(sc, g, mti, pre, ne, etot, exw, bw);
    {
      int used = 0;
#pragma unroll
      for (int i = 0; i < kRyR; i++) {
        int s = ryr_of(w, i);
        if (k.regime == 0) {
          if (s == 7 || s == 8) {
            const double u = (double)exw[used++] / 4294967296.0;
            if (s == 7) s = (u < (k.k34 / (k.k34 + k43))) ? 4 : 3;
            else s = (u < k.k56 / (k.k56 + k65)) ? 6 : 5;
          }
        } else if (k.regime == 1) {
          if (s == 7) {
            const double u = (double)exw[used++] / 4294967296.0;
            s = (u < k.k34 / (k.k34 + k43)) ? 4 : 3;
          }
          if (s == 5 || s == 6) s = 8;
        } else {
          if (s == 3 || s == 4) s = 7;
          else if (s == 5 || s == 6) s = 8;
        }
        w = set_field(w, 8 + 4 * i, s);
      }
    }
    {
      bool need7 = false, need8 = false;
#pragma unroll
      for (int i = 0; i < kRyR; i++) {
        const int s = ryr_of(w, i);
        need7 |= (s == 7);
        need8 |= (s == 8);
      }
      const double T2 = k21 + k.k23 + k.k25, T3 = k32 + k.k34, T5 = k52 + k.k54 + k.k56;
      constexpr double T4 = k43 + k45;
      double T7 = 0.0, T8 = 0.0;
      if (need7) {
        const double a1 = k.k34 / (k43 + k.k34);
        T7 = (1.0 - a1) * k32 + a1 * k45;
      }
      if (need8) {
        const double a1 = k65 / (k.k56 + k65);
        T8 = a1 * k52 + a1 * k.k54;
      }
#pragma unroll
      for (int i = 0; i < kRyR; i++) {
        const int s = ryr_of(w, i);
        double r = k.k12;
        r = (s == 2) ? T2 : r;
        r = (s == 3) ? T3 : r;
        r = (s == 4) ? T4 : r;
        r = (s == 5) ? T5 : r;
        r = (s == 6) ? k65 : r;
        r = (s == 7) ? T7 : r;
        r = (s == 8) ? T8 : r;
        R0[2 + i] = r;
      }
    }
    R0[7] = (cl_of(w) == 1) ? kfIto2 * cass : kbIto2;
    double mx = 0.0;
#pragma unroll
    for (int j = 0; j < 8; j++) mx = imax(mx, R0[j]);
    mx = gmax(g, mx);
    // ---- substep size (simfru_local.c:135-146) ----
    double dt = imin(0.1 / mx, 10.001e-3);
    const double cmax = gmax(g, imax(0.e-3, cass));
    if (cmax > 1.5e-3) dt = imin(dt, 5.001e-3);
    dt = imin(dt, p.tf - t);
    // ---- Heun step (simfru_local.c:149-173) ----
    double dJ, dS;
    fcn_fru4(g, cajsr, cass, dep, e2, a2j, small, lopen, nopen, dJ, dS);
    const double k1J = dt * dJ, k1S = dt * dS;
    const double y1J = cajsr + k1J, y1S = cass + k1S;
    t = t + dt;
    const double frac = (t - p.t0) / interval;
#pragma unroll
    for (int i = 0; i < 3; i++) dep[i] = p.dep0[i] + frac * p.span[i];
    ghk_terms(dep[0], e2, a2j, small);
    fcn_fru4(g, y1J, y1S, dep, e2, a2j, small, lopen, nopen, dJ, dS);
    cajsr = cajsr + (k1J + dt * dJ) / 2.0;
    cass = cass + (k1S + dt * dS) / 2.0;
    // ---- transitions of this cleft's 8 channels (:215-276) ----
    bool moved = false;
    if (u_gt(bw[0], 1.0 - dt * R0[0])) {
      const LccBasis lb{alpha, beta, bp};
      double r[4];
      int d[4];
      const int len = lcc_row(lcc_of(w), lb, gammacf * cass0, r, d);
      w = set_field(w, 0, pick_dest(r, d, len, dt, (double)bw[0] / 4294967296.0));
    }
    if (u_ge(bw[1], 1.0 - dt * R0[1])) w = set_field(w, 4, 3 - vdi_of(w));
#pragma unroll
    for (int i = 0; i < kRyR; i++) {
      if (u_gt(bw[2 + i], 1.0 - dt * R0[2 + i])) {
        double r[4];
        int d[4];
        const int len = ryr_row(ryr_of(w, i), k, r, d);
        w = set_field(w, 8 + 4 * i, pick_dest(r, d, len, dt, (double)bw[2 + i] / 4294967296.0));
        moved = true;
      }
    }
    if (u_ge(bw[7], 1.0 - dt * R0[7])) w = set_field(w, 28, 3 - cl_of(w));
    lopen = lcc_open(w) ? 1.0 : 0.0;
    if (moved) nopen = ryr_open_count(w);
    nsub++;
  }
}

__global__ void __launch_bounds__(32) fru_stage4_kernel(DevState s, StageParams p) {
  __shared__ double smem[32 * 5];
  const int lane = threadIdx.x & 31;
  Group g;
  g.c = lane & 3;
  g.base = lane & ~3;
  g.mask = 0xfu << g.base;
  const int f = blockIdx.x * 8 + (threadIdx.x >> 2);
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  uint32_t nsub = 0;
  bool overflow = false;
  const bool active = f < s.nfru;  // uniform over each 4-lane group
  if (active) {
    const size_t nf = (size_t)s.stride;
    double cajsr, cass;
    uint32_t w;
    int mti;
    StageCtx sc;
    sc.p = &p;
    sc.m = s.mt + (size_t)f * kMtStride;
    sc.hold = s.mt_hold + (size_t)f * kMtStride;
    sc.hold_epoch = s.hold_epoch + f;
    if (p.flags & kFlagResume) {
      cajsr = s.frus_s[f];
      cass = s.frus_s[(g.c + 1) * nf + f];
      w = s.chan_s[g.c * nf + f];
      mti = s.mti_s[f];
      if (*sc.hold_epoch == p.epoch) copy4(sc.m, sc.hold, g);
    } else {
      cajsr = s.frus[f];
      cass = s.frus[(g.c + 1) * nf + f];
      w = s.chan[g.c * nf + f];
      mti = s.mti[f];
    }
    if (p.flags & kFlagSave) {
      if (g.c == 0) {
        s.frus_s[f] = cajsr;
        s.mti_s[f] = mti;
      }
      s.frus_s[(g.c + 1) * nf + f] = cass;
      s.chan_s[g.c * nf + f] = w;
    }
    if (p.flags & kFlagAdvance) advance4(sc, g, cajsr, cass, w, mti, nsub, overflow);
    if (g.c == 0) {
      s.frus[f] = cajsr;
      s.mti[f] = mti;
    }
    s.frus[(g.c + 1) * nf + f] = cass;
    s.chan[g.c * nf + f] = w;
    v[0] = cass;
    v[1] = (g.c == 0) ? cajsr : 0.0;
    if (lcc_open(w)) {
      v[2] = cass;
      v[3] = 1.0;
    }
    if (cl_of(w) == 2) v[4] = 1.0;
  }
  __syncwarp();
  if (overflow) s.out[kOutError] = 1.0;
  if (s.substeps) {
    unsigned long long c = (g.c == 0) ? nsub : 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(kFull, c, o);
    if (lane == 0 && c) atomicAdd(s.substeps, c);
  }
  block_reduce<5>(v, smem);
  double tot[5];
  if (grid_finish<5>(v, s.partials, s.ticket, smem, tot)) {
    double cur[4];
    currents_from_sums(s.nfru, p.nfru_scale, p.depf, tot, cur);
#pragma unroll
    for (int k2 = 0; k2 < 5; k2++) s.out[k2] = tot[k2];
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) s.out[5 + k2] = cur[k2];
  }
}

}  // namespace c4

cudaError_t launch_stage4(const DevState& s, const StageParams& p, cudaStream_t st) {
  const int blocks = (s.nfru + 7) / 8;
  c4::fru_stage4_kernel<<<blocks, 32, 0, st>>>(s, p);
  return cudaGetLastError();
}

}  // namespace gw
