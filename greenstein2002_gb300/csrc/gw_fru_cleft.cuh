// Cleft-parallel FRU substep loop, shared by the FP64 and the mixed-precision
// stage kernels: each FRU is advanced by a group of four lanes, one per
// dyadic cleft (8 FRUs per warp).
//
// Why four lanes per FRU: on GB300 every SM sub-partition issues one FP64
// warp instruction per 64 cycles whatever the active-lane mask, so a stage
// lasts as long as the FP64 instruction chain of its slowest FRU.  Spreading an
// FRU over its clefts divides that chain by about four at the same total work.
//
// R = double: the plain FP64 method.  Every operation is the reference's, and
// the arithmetic is arranged to issue few FP64 instructions while staying
// bit-identical to it:
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
// R = float: the mixed-precision method.  Transition rates, the local Ca ODE
// and the FRU clock are evaluated in FP32, the Ca states and the clock
// accumulated as compensated FP32 pairs; FP64 is kept for the FRU arrays in
// memory and for the cross-FRU flux sums.  Channel transitions use the
// complement form 1 - u < dt*rate, which keeps full resolution near u = 1.
//
// MT19937 rows are drawn from and regenerated in place, in the FRU's own
// row in global memory (L1-cached; the kernels use no shared memory): on
// GB300 this ran as fast as staging the eight rows of a warp in shared
// memory for FP64 and 15% faster for mixed precision, whose warps the
// staging's 20 KB per warp had held to eleven per SM.
//
// Reference: simfru_local.c:32-278, fru_rates_local.c:30-798, fcn_fru.c:23-137,
// mt19937_local.c:97-240.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gw_fru_core.cuh"
#include "gw_fru_model.cuh"
#include "gw_kernels.h"

namespace gw {
namespace cleft {

// ---- type-specific operations ----------------------------------------------
__device__ __forceinline__ long long ord(double a) { return __double_as_longlong(a); }
__device__ __forceinline__ int ord(float a) { return __float_as_int(a); }
// max/min of values known to be >= 0 (or of a negative value against a
// positive constant): IEEE order equals the signed integer order of the bits;
// ties return the first argument like the reference's macros
template <typename R>
__device__ __forceinline__ R imax(R a, R b) { return ord(a) < ord(b) ? b : a; }
template <typename R>
__device__ __forceinline__ R imin(R a, R b) { return ord(a) < ord(b) ? a : b; }
template <typename R>
__device__ __forceinline__ bool ilt(R a, R b) { return ord(a) < ord(b); }
// |v| < c for a positive constant c, on the integer pipe
__device__ __forceinline__ bool abs_lt(double v, double c) {
  return (__double_as_longlong(v) & 0x7fffffffffffffffLL) < __double_as_longlong(c);
}
__device__ __forceinline__ bool abs_lt(float v, float c) { return (__float_as_int(v) & 0x7fffffff) < __float_as_int(c); }

// x / d for a compile-time constant d with r = 1/d: correctly rounded in FP64
__device__ __forceinline__ double divc(double x, double d, double r) {
  const double q = x * r;
  return fma(fma(-q, d, x), r, q);
}
__device__ __forceinline__ float divc(float x, float d, float r) { return x * r; }
// Divisions by variable divisors.  FP64: the hardware's correctly rounded
// quotient.  (The integer-pipe division of gw_intdiv.h gives the same bits
// with ~6 fewer FP64-pipe slots, but its longer dependent chain made the
// latency-bound stage kernels 25-30% slower on GB300, so it is not used
// here.)  FP32: rdiv is the fast approximate quotient, qdiv the correctly
// rounded one.
__device__ __forceinline__ double rdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double qdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float qdiv(float a, float b) { return a / b; }
__device__ __forceinline__ double rexp(double x) { return exp(x); }
__device__ __forceinline__ float rexp(float x) { return expf(x); }
// e = exp(x) and the GHK denominator e - 1.  FP64: the reference's e - 1.
// FP32: expm1f, because expf(x) - 1 keeps almost no relative precision for
// the |x| < 1e-5 of membrane potentials within a few tenths of a mV of zero,
// and is exactly 0 for potentials of a few uV (just above the 1e-6 mV of the
// reference's V = 0 branch), which made the GHK factor infinite.
__device__ __forceinline__ void exp_em1(double x, double& e, double& em1) {
  e = exp(x);
  em1 = e - 1.0;
}
__device__ __forceinline__ void exp_em1(float x, float& e, float& em1) {
  em1 = expm1f(x);
  e = 1.0f + em1;
}

// FP64: u = y/2^32 compared with P = 1 - dt*R in the integer domain.
__device__ __forceinline__ void thresh(double P, uint64_t& fl, bool& exact) {
  const uint64_t b = (uint64_t)__double_as_longlong(P);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  const uint64_t M = (b & 0xfffffffffffffull) | (1ull << 52);
  const int sh = 20 - e;  // floor(P * 2^32) = M >> (52 - 32 - e)
  if (sh >= 64) {
    fl = 0;
    exact = false;
  } else {
    fl = M >> sh;
    exact = (M & ((1ull << sh) - 1ull)) == 0ull;
  }
}
// leaves its state when u > 1 - dt*R (LCC, RyR) ...
__device__ __forceinline__ bool nonpos(double P) { return __double_as_longlong(P) <= 0LL; }  // P <= 0 (not NaN)
__device__ __forceinline__ bool leave_gt(uint32_t y, double dt, double R) {
  const double P = 1.0 - dt * R;
  if (nonpos(P)) return true;  // never on valid input (dt*rate <= 0.1)
  uint64_t fl;
  bool ex;
  thresh(P, fl, ex);
  return (uint64_t)y > fl;
}
// ... or when u >= 1 - dt*R (VDI gate, Cl channel)
__device__ __forceinline__ bool leave_ge(uint32_t y, double dt, double R) {
  const double P = 1.0 - dt * R;
  if (nonpos(P)) return true;
  uint64_t fl;
  bool ex;
  thresh(P, fl, ex);
  return (uint64_t)y > fl || (ex && (uint64_t)y == fl);
}
// 2^32 - y rounded to FP32, from a 32-bit conversion (0 - y wraps to it for
// y > 0): the same value as converting the 33-bit integer, without a 64-bit
// integer conversion, which runs on the FP64 pipe.
__device__ __forceinline__ float comp_u32(uint32_t y) { return y ? (float)(0u - y) : 4294967296.0f; }
// FP32: complement form, 1 - u = (2^32 - y)/2^32 against dt*R
__device__ __forceinline__ bool leave_gt(uint32_t y, float dt, float R) {
  return comp_u32(y) < dt * R * 4294967296.0f;
}
__device__ __forceinline__ bool leave_ge(uint32_t y, float dt, float R) {
  return comp_u32(y) <= dt * R * 4294967296.0f;
}

// Destination of a channel that leaves its state (simfru_local.c:215-253):
// FP64 walks the reference's cumulative probabilities with u = y/2^32; FP32
// walks the remaining exit mass against 1 - u = (2^32 - y)/2^32, which keeps
// full resolution near u = 1 where the walk happens.
__device__ __forceinline__ int choose_dest(const double r[4], const int d[4], int len, double dt, uint32_t y) {
  return pick_dest(r, d, len, dt, (double)y / 4294967296.0);
}
__device__ __forceinline__ int choose_dest(const float r[4], const int d[4], int len, float dt, uint32_t y) {
  const float c = comp_u32(y) * 2.3283064365386963e-10f;
  float rem = dt * r[0] - dt * r[1];
  int n = 1;
  while (c < rem && n + 1 < len) {
    n++;
    rem = rem - dt * r[n];
  }
  return d[n];
}

// u = y/2^32 < p for 0 < p < 1 (pseudo-state draws, fru_rates_local.c):
// FP64 in the integer domain (u < p <=> y < p*2^32); FP32 directly
__device__ __forceinline__ bool u_below(uint32_t y, double p) {
  if (nonpos(p)) return false;
  uint64_t fl;
  bool ex;
  thresh(p, fl, ex);
  return ex ? (uint64_t)y < fl : (uint64_t)y <= fl;
}
__device__ __forceinline__ bool u_below(uint32_t y, float p) { return (float)y * 2.3283064365386963e-10f < p; }

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

template <typename R>
__device__ __forceinline__ R pick_basis(int i, R al, R be, R ga, R ap, R bp) {
  R v = R(1);
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
template <typename R>
__device__ __forceinline__ R gmax(const Group& g, R v) {
  v = imax(v, __shfl_xor_sync(g.mask, v, 1));
  v = imax(v, __shfl_xor_sync(g.mask, v, 2));
  return v;
}

// In-place regeneration of one FRU's 624 words (mt19937_local.c:97-154) by
// all 32 lanes of the warp, 32 consecutive words per step.  Word k < 227
// reads the old word k + 397 (not reached yet), word k >= 227 the new word
// k - 227 (written at least seven steps earlier) and word 623 the new words 0
// and 396, as in the sequential loop; every lane reads before the barrier
// and writes after it.
__device__ __forceinline__ void regen32(uint32_t* m, int lane) {
  for (int k0 = 0; k0 < kMtN; k0 += 32) {
    const int k = k0 + lane;
    const bool in = k < kMtN;
    uint32_t nw = 0u;
    if (in) {
      const uint32_t cur = m[k];
      const uint32_t nxt = m[(k + 1 == kMtN) ? 0 : k + 1];
      const uint32_t far = m[(k + kMtM < kMtN) ? k + kMtM : k + kMtM - kMtN];
      const uint32_t y = (cur & 0x80000000u) | (nxt & 0x7fffffffu);
      nw = far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    __syncwarp();
    if (in) m[k] = nw;
    __syncwarp();
  }
}
__device__ __forceinline__ void copy4(uint32_t* dst, const uint32_t* src, const Group& g) {
  for (int k = g.c; k < kMtN; k += 4) dst[k] = src[k];
  __syncwarp(g.mask);
}
// 624 words in 16-byte pieces by the group's 4 lanes (rows 16-byte aligned)
__device__ __forceinline__ void copy_row16(uint32_t* dst, const uint32_t* src, const Group& g) {
  const uint4* s4 = reinterpret_cast<const uint4*>(src);
  uint4* d4 = reinterpret_cast<uint4*>(dst);
  for (int i = g.c; i < kMtN / 4; i += 4) d4[i] = s4[i];
  __syncwarp(g.mask);
}

// The launch's view of one warp's 8 FRUs: each lane's FRU row (in place,
// global memory) and the copy-on-twist rows of the cell.
struct StageCtx {
  const StageParams* p;
  uint32_t* m;               // this lane's FRU row
  uint32_t* hold_base;       // copy-on-twist rows of the cell, FRU-major
  uint32_t* hold_epoch_base; // their epochs
  uint32_t* my_hold_epoch;   // the epoch of this lane's FRU
  int f;                     // this lane's FRU (any value for a group without one)
};

// Point the group at its FRU's row; on a resume whose epoch's snapshot
// holds the row's words from before its last regeneration, put them back
// first (send_resume_state's MT restore, mpi_slave.c:150-184).
__device__ __forceinline__ void use_row(StageCtx& sc, uint32_t* row, const uint32_t* hold, bool restore,
                                        const Group& g) {
  if (restore) copy_row16(row, hold, g);
  sc.m = row;
}

// The words of one substep are E_tot extra draws (lane c owns positions
// pre .. pre+ne-1) followed by the 32 batch draws (lane c owns 8c .. 8c+7).
// fetch_old reads those below word 624; regen_crossing then regenerates, with
// the whole warp, the rows whose draws run past it; fetch_new reads the rest
// from the new generation, tempers, and advances mti.
__device__ __forceinline__ void fetch_old(const StageCtx& sc, const Group& g, int mti, int pre, int ne, int etot,
                                          uint32_t ex[kRyR], uint32_t bw[8]) {
#pragma unroll
  for (int i = 0; i < kRyR; i++) {
    const int pos = mti + pre + i;
    if (i < ne && pos < kMtN) ex[i] = sc.m[pos];
  }
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int pos = mti + etot + 8 * g.c + k;
    if (pos < kMtN) bw[k] = sc.m[pos];
  }
}

// cross / copy: bit 4*i set when group i regenerates / first copies its
// pre-regeneration words to its hold row in this epoch (lane 4*i's ballot).
__device__ __forceinline__ void regen_crossing(const StageCtx& sc, int lane, unsigned cross, unsigned copy) {
  while (cross) {
    const int l0 = __ffs(cross) - 1;
    cross &= cross - 1u;
    uint32_t* row = reinterpret_cast<uint32_t*>(__shfl_sync(0xffffffffu, (unsigned long long)sc.m, l0));
    const int fg = __shfl_sync(0xffffffffu, sc.f, l0);  // the FRU of group l0/4
    __syncwarp();  // the group has read its old words
    if (copy & (1u << l0)) {
      const uint4* s4 = reinterpret_cast<const uint4*>(row);
      uint4* d4 = reinterpret_cast<uint4*>(sc.hold_base + (size_t)fg * kMtStride);
      for (int i = lane; i < kMtN / 4; i += 32) d4[i] = s4[i];
      if (lane == 0) sc.hold_epoch_base[fg] = sc.p->epoch;
    }
    regen32(row, lane);
  }
}

__device__ __forceinline__ void fetch_new(const StageCtx& sc, const Group& g, int& mti, int pre, int ne, int etot,
                                          uint32_t ex[kRyR], uint32_t bw[8]) {
  const int W = etot + 32;
  if (mti + W > kMtN) {
#pragma unroll
    for (int i = 0; i < kRyR; i++) {
      const int pos = mti + pre + i;
      if (i < ne && pos >= kMtN) ex[i] = sc.m[pos - kMtN];
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int pos = mti + etot + 8 * g.c + k;
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

// JRyRmax * (R)n for n = 0..5 open RyRs, by selection instead of a
// conversion and a multiply (the products are the same rounded values)
template <typename R>
__device__ __forceinline__ R jryr_coef(int n) {
  R v = R(0);
  v = (n == 1) ? R(JRyRmax) * R(1) : v;
  v = (n == 2) ? R(JRyRmax) * R(2) : v;
  v = (n == 3) ? R(JRyRmax) * R(3) : v;
  v = (n == 4) ? R(JRyRmax) * R(4) : v;
  v = (n == 5) ? R(JRyRmax) * R(5) : v;
  return v;
}

// Local Ca ODE of one cleft (fcn_fru.c:23-137) evaluated by the FRU's four
// lanes.  Each lane returns dCaSS of its cleft; every lane returns the same
// dCaJSR.  e2 = exp(2 V F/RT) and a2j are passed in (shared by all lanes).
template <typename R>
__device__ __forceinline__ void fcn_fru4(const Group& g, R cajsr, R cass, const R dep[3], R e2, R a2j, bool small,
                                         R lopen, int nopen, R pca_scale, R& dJSR, R& dSS) {
  constexpr double JDHconstant = 1.0 / (2.0 * VSS * Faraday * 1000.0);
  constexpr double KJDHsmall = -PCa * 2.0 * 1000.0 * Faraday;
  const R Cai = dep[1], CaNSR = dep[2];
  // JRyR of every cleft, summed in cleft order
  const R jcoef = jryr_coef<R>(nopen);
  const R JRyR = jcoef * (cajsr - cass);
  const R j0 = from(g, JRyR, 0), j1 = from(g, JRyR, 1), j2 = from(g, JRyR, 2), j3 = from(g, JRyR, 3);
  const R JRyRtot = j0 + j1 + j2 + j3;
  const R cnext = from(g, cass, (g.c + 1) & 3);
  const R Jss = divc(cass - cnext, R(tauss2ss), R(1.0 / tauss2ss));
  const R Jss_prev = from(g, Jss, (g.c + 3) & 3);
  const R Jxfer = divc(cass - Cai, R(tauxfer), R(1.0 / tauxfer));
  R JDH;
  if (small) JDH = R(KJDHsmall) * pca_scale * (cass - R(Cao * 0.341)) * lopen * R(JDHconstant);
  else JDH = -(cass * e2 - R(Cao * 0.341)) * a2j * lopen;
  R a1 = rdiv(R(BSRtot * KBSR), (cass + R(KBSR)) * (cass + R(KBSR)));
  R a2 = rdiv(R(BSLtot * KBSL), (cass + R(KBSL)) * (cass + R(KBSL)));
  const R bSS = rdiv(R(1), R(1) + a1 + a2);
  dSS = bSS * (JDH + JRyR - Jxfer - Jss + Jss_prev);
  const R Jtr = divc(CaNSR - cajsr, R(tautr), R(1.0 / tautr));
  a1 = rdiv(R(CSQNtot * KmCSQN), (cajsr + R(KmCSQN)) * (cajsr + R(KmCSQN)));
  const R bJSR = rdiv(R(1), R(1) + a1);
  dJSR = bJSR * (Jtr - R(VSS / VJSR) * JRyRtot);
}

// exp(2 V F / RT) and the GHK factor a2 of fcn_fru.c:78-101 for voltage V
template <typename R>
__device__ __forceinline__ void ghk_terms(R V, R pca_scale, R& e2, R& a2j, bool& small) {
  constexpr double JDHconstant = 1.0 / (2.0 * VSS * Faraday * 1000.0);
  const R VFRT = divc(V, R(RT_over_F), R(1.0 / RT_over_F));
  const R VFsqRT = R(1000.0 * Faraday) * VFRT;
  R em1;
  exp_em1(R(2) * VFRT, e2, em1);
  small = abs_lt(V, R(1.e-6));
  if (small) a2j = R(0);
  else a2j = rdiv(R(PCa * 4.0) * pca_scale * VFsqRT, em1) * R(JDHconstant);
}

// (t - t0) / interval with r = 1/interval rounded once per stage: Markstein's
// correction of q = x*r returns the correctly rounded quotient
__device__ __forceinline__ double frac_of(double t, double t0, double interval, double r) {
  const double x = t - t0;
  const double q = x * r;
  return fma(fma(-q, interval, x), r, q);
}
__device__ __forceinline__ float frac_of(double t, double t0, double, float rinterval) {
  return (float)(t - t0) * rinterval;
}

// The constants of one lane for a stage (the same for every FRU of it).
template <typename R>
struct LaneStage {
  R dep0[3], span[3], pca_scale, rinterval;
  double t0, tf, interval;
  float ihi, ilo;  // the interval as a compensated FP32 pair (the mixed-precision clock)
  // per-lane voltage exponential of the rates: alpha, beta, yCa_inf, tau_yCa
  //   lane 0: alphacf*exp(0.012*(V-35))     lane 1: betacf*exp(-0.05*(V-35))
  //   lane 2: 0.4/(1+exp((V+12.5)/5)) + 0.6  lane 3: 60 + 340/(1+exp((V+30)/12))
  bool isdiv;
  R cA, cR, cD, cCF, cK, cM;
};

template <typename R>
__device__ __forceinline__ void lane_stage(const StageParams& p, const Group& g, LaneStage<R>& L) {
#pragma unroll
  for (int i = 0; i < 3; i++) {
    L.dep0[i] = (R)p.dep0[i];
    L.span[i] = (R)p.span[i];
  }
  L.pca_scale = (R)p.pca_scale;
  L.t0 = p.t0;
  L.tf = p.tf;
  L.interval = p.tf - p.t0;
  L.rinterval = (R)(1.0 / L.interval);
  L.ihi = (float)L.interval;
  L.ilo = (float)(L.interval - (double)L.ihi);
  L.isdiv = g.c >= 2;
  L.cA = L.isdiv ? (g.c == 2 ? R(12.5) : R(30.0)) : R(-35.0);
  L.cR = L.isdiv ? (g.c == 2 ? R(1.0 / 5.0) : R(1.0 / 12.0)) : (g.c == 0 ? R(0.012) : R(-0.05));
  L.cD = L.isdiv ? (g.c == 2 ? R(5.0) : R(12.0)) : R(1.0);
  L.cCF = L.isdiv ? R(0.0) : (g.c == 0 ? R(alphacf) : R(betacf));
  L.cK = L.isdiv ? (g.c == 2 ? R(0.4) : R(340.0)) : R(1.0);
  L.cM = L.isdiv ? (g.c == 2 ? R(1.0 - 0.4) : R(60.0)) : R(0.0);
}

// Accumulator of an FRU Ca concentration over the substeps.  FP64: a double,
// updated as the reference does.  Mixed precision: a compensated FP32 pair
// (Neumaier's summation: hi + lo carries about 48 bits), so the FP32
// increments accumulate without FP64 instructions or conversions in the
// substep loop; the FRU arrays stay FP64 (split on load, joined on store).
template <typename R>
struct CaAcc;
template <>
struct CaAcc<double> {
  double v;
  __device__ __forceinline__ void set(double x) { v = x; }
  __device__ __forceinline__ double get() const { return v; }
  __device__ __forceinline__ double r() const { return v; }
  __device__ __forceinline__ void add(double inc) { v = v + inc; }
};
template <>
struct CaAcc<float> {
  float hi, lo;
  __device__ __forceinline__ void set(double x) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
  }
  __device__ __forceinline__ double get() const { return (double)hi + (double)lo; }
  __device__ __forceinline__ float r() const { return hi + lo; }
  __device__ __forceinline__ void add(float inc) {
    const float t = hi + inc;
    lo = lo + ((fabsf(hi) >= fabsf(inc)) ? (hi - t) + inc : (inc - t) + hi);
    hi = t;
  }
};

// The FRU's clock over [t0, tf] (simfru_local.c:135-146, :161): the step of
// a substep is dt = min(dt_rate, tf - t), so the last substep lands on tf.
// FP64: the reference's time_FRU, an FP64 time (t + (tf - t) is exactly tf,
// as both are close).  Mixed precision: the time since t0 as a compensated
// FP32 pair (about 48 bits, far finer than any substep of a stage of at most
// 0.1 ms), the last substep taking exactly the time that remains -- no FP64
// instruction or conversion in the substep loop.
template <typename R>
struct FruClock;
template <>
struct FruClock<double> {
  double t;
  __device__ __forceinline__ void begin(const LaneStage<double>& L) { t = L.t0; }
  __device__ __forceinline__ bool running(const LaneStage<double>& L) const { return t < L.tf; }
  __device__ __forceinline__ double advance(double dtr, const LaneStage<double>& L) {
    const double dt64 = imin(dtr, L.tf - t);
    t = t + dt64;
    return dt64;
  }
  __device__ __forceinline__ double frac(const LaneStage<double>& L) const {
    return frac_of(t, L.t0, L.interval, L.rinterval);
  }
};
template <>
struct FruClock<float> {
  float hi, lo;  // time since t0
  bool fin;      // the FRU has reached tf
  __device__ __forceinline__ void begin(const LaneStage<float>& L) {
    hi = 0.0f;
    lo = 0.0f;
    fin = !(L.interval > 0.0);
  }
  __device__ __forceinline__ bool running(const LaneStage<float>&) const { return !fin; }
  __device__ __forceinline__ float advance(float dtr, const LaneStage<float>& L) {
    const float rem = (L.ihi - hi) + (L.ilo - lo);
    if (!(dtr < rem)) {
      fin = true;
      hi = L.ihi;
      lo = L.ilo;
      return rem;
    }
    const float s = hi + dtr;  // Knuth's two-sum of hi and dtr
    const float b = s - hi;
    lo = lo + ((hi - (s - b)) + (dtr - b));
    hi = s;
    return dtr;
  }
  __device__ __forceinline__ float frac(const LaneStage<float>& L) const { return (hi + lo) * L.rinterval; }
};

// One FRU's state in the substep loop, as seen by one lane (its cleft):
// the FRU Ca state and clock, channel word, MT position, and the values
// carried from one substep to the next.
template <typename R>
struct Fru4 {
  FruClock<R> clk;
  CaAcc<R> jsr, ss;  // CaJSR and this cleft's CaSS
  uint32_t w, nsub;
  int mti, nopen;
  R dep[3], e2, a2j, lopen;
  bool small;
};

// the FRU at the stage start (t0, voltages dep0)
template <typename R>
__device__ __forceinline__ void fru_begin(Fru4<R>& F, const LaneStage<R>& L) {
#pragma unroll
  for (int i = 0; i < 3; i++) F.dep[i] = L.dep0[i];
  F.lopen = lcc_open(F.w) ? R(1) : R(0);
  F.nopen = ryr_open_count(F.w);
  F.clk.begin(L);
  ghk_terms(F.dep[0], L.pca_scale, F.e2, F.a2j, F.small);
}

// Values of one substep carried from its first half (rates, extra-draw
// layout, words below 624) to its second (words past 624, Heun step,
// transitions), between which the warp regenerates MT rows.
template <typename R>
struct Sub4 {
  R cajsr, cass, alpha, beta, bp, gam, k12, k23, k34, k54, k25, k56, p34, R0[8];
  int regime, ne, pre, etot;
  uint32_t exw[kRyR], bw[8];
};

// First half of one substep of the FRU (simfru_local.c:83-146 up to the
// draws): voltage terms, exit totals, the RyR constants, the layout of the
// extra draws and the words that precede word 624.
template <typename R>
__device__ __forceinline__ void substep_a(Fru4<R>& F, Sub4<R>& S, const LaneStage<R>& L, const Group& g,
                                          const StageCtx& sc) {
  uint32_t& w = F.w;
  const int mti = F.mti;
  const R* dep = F.dep;
  R &cajsr = S.cajsr, &cass = S.cass, &alpha = S.alpha, &beta = S.beta, &bp = S.bp, &gam = S.gam;
  R &k12 = S.k12, &k23 = S.k23, &k34 = S.k34, &k54 = S.k54, &k25 = S.k25, &k56 = S.k56;
  R* R0 = S.R0;
  int &regime = S.regime, &ne = S.ne, &pre = S.pre, &etot = S.etot;
  const bool isdiv = L.isdiv;
  const R cA = L.cA, cR = L.cR, cD = L.cD, cCF = L.cCF, cK = L.cK, cM = L.cM;
  cajsr = F.jsr.r();
  cass = F.ss.r();
  // ---- voltage terms at the substep start, one exponential per lane ----
  const R x = dep[0] + cA;
  R q = x * cR;
  if (isdiv) q = divc(x, cD, cR);
  const R ev = rexp(q);
  const R r01 = cCF * ev;
  const R r23 = rdiv(cK, R(1) + ev) + cM;
  const R vterm = isdiv ? r23 : r01;
  alpha = from(g, vterm, 0);
  beta = from(g, vterm, 1);
  const R yinf = from(g, vterm, 2), tau = from(g, vterm, 3);
  bp = divc(beta, R(bL * kappa), R(1.0 / (bL * kappa)));
  const R ap = R(aL) * alpha;
  // ---- exit totals of this cleft's 8 channels ----
  gam = R(gammacf) * cass;
  {
    const int s = lcc_of(w);
    const uint16_t bi = c_lcc_basis[s];
    const R X = R(c_lcc_coef[s][0]) * pick_basis(bi & 15, alpha, beta, gam, ap, bp);
    const R Y = R(c_lcc_coef[s][1]) * pick_basis((bi >> 4) & 15, alpha, beta, gam, ap, bp);
    const R Z = R(c_lcc_coef[s][2]) * pick_basis((bi >> 8) & 15, alpha, beta, gam, ap, bp);
    R0[0] = X + Y + Z;
  }
  {
    const R num = (vdi_of(w) == 2) ? (R(1) - yinf) : yinf;
    R0[1] = rdiv(num, tau);
  }
  // RyR constants of the cleft and the pseudo-state draws
  const R c2 = cass * cass;
  const R sat = imin(R(threshMAX), divc(c2, R(k_rate), R(1.0 / k_rate)));
  const R sat2 = imin(R(threshMAX), divc(c2, R(k_rate2), R(1.0 / k_rate2)));
  k12 = R(k12cf) * sat2;
  k23 = R(k23cf) * sat;
  k34 = R(k34cf) * sat;
  k54 = R(k54cf) * sat;
  k25 = R(k25cf) * sat;
  k56 = R(k56cf) * sat;
  {
    const R cc = imin(cass, R(threshMAXCa));
    regime = ilt(cc, R(threshCa56to8)) ? 0 : (ilt(cc, R(threshCa34to7)) ? 1 : 2);
  }
  // extra draws: regime 0 resolves 7 and 8, regime 1 resolves 7 (in cleft, then RyR order)
  ne = 0;
  #pragma unroll
  for (int i = 0; i < kRyR; i++) {
    const int s = ryr_of(w, i);
    ne += (regime == 0 && (s == 7 || s == 8)) || (regime == 1 && s == 7);
  }
  const int n0 = from(g, ne, 0), n1 = from(g, ne, 1), n2 = from(g, ne, 2), n3 = from(g, ne, 3);
  pre = (g.c > 0 ? n0 : 0) + (g.c > 1 ? n1 : 0) + (g.c > 2 ? n2 : 0);
  etot = n0 + n1 + n2 + n3;
  fetch_old(sc, g, mti, pre, ne, etot, S.exw, S.bw);
}

// Second half: the remaining words, the RyR pseudo-states, the substep size,
// the Heun step of the local Ca ODE and the transitions (:135-277).
template <typename R>
__device__ __forceinline__ void substep_b(Fru4<R>& F, Sub4<R>& S, const LaneStage<R>& L, const Group& g,
                                          StageCtx& sc) {
  uint32_t& w = F.w;
  int& mti = F.mti;
  R* dep = F.dep;
  R &e2 = F.e2, &a2j = F.a2j, &lopen = F.lopen;
  bool& small = F.small;
  int& nopen = F.nopen;
  const R cajsr = S.cajsr, cass = S.cass, alpha = S.alpha, beta = S.beta, bp = S.bp, gam = S.gam;
  const R k12 = S.k12, k23 = S.k23, k34 = S.k34, k54 = S.k54, k25 = S.k25, k56 = S.k56;
  R& p34 = S.p34;
  R* R0 = S.R0;
  const int regime = S.regime, ne = S.ne, pre = S.pre, etot = S.etot;
  uint32_t* exw = S.exw;
  uint32_t* bw = S.bw;
  const R pca_scale = L.pca_scale;
  fetch_new(sc, g, mti, pre, ne, etot, exw, bw);
  {
    // the draws are taken in order from a shifting window (static
    // register indices); k34/(k34+k43) is formed once, for the draws of
    // regimes 0/1 or for the merged state 7 of regime 2 (never both)
    bool has7 = false, has34 = false;
  #pragma unroll
    for (int i = 0; i < kRyR; i++) {
      const int s = ryr_of(w, i);
      has7 |= (s == 7);
      has34 |= (s == 3 || s == 4);
    }
    if ((regime <= 1 && has7) || (regime == 2 && (has7 || has34))) p34 = qdiv(k34, k34 + R(k43));
  #pragma unroll
    for (int i = 0; i < kRyR; i++) {
      int s = ryr_of(w, i);
      if (regime == 0) {
        if (s == 7 || s == 8) {
          const uint32_t y = exw[0];
          exw[0] = exw[1];
          exw[1] = exw[2];
          exw[2] = exw[3];
          exw[3] = exw[4];
          if (s == 7) s = u_below(y, p34) ? 4 : 3;
          else s = u_below(y, qdiv(k56, k56 + R(k65))) ? 6 : 5;
        }
      } else if (regime == 1) {
        if (s == 7) {
          const uint32_t y = exw[0];
          exw[0] = exw[1];
          exw[1] = exw[2];
          exw[2] = exw[3];
          exw[3] = exw[4];
          s = u_below(y, p34) ? 4 : 3;
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
    const R T2 = R(k21) + k23 + k25, T3 = R(k32) + k34, T5 = R(k52) + k54 + k56;
    const R T4 = R(k43 + k45);
    R T7 = R(0), T8 = R(0);
    if (need7) {
      const R a1 = p34;  // k34 / (k43 + k34)
      T7 = (R(1) - a1) * R(k32) + a1 * R(k45);
    }
    if (need8) {
      const R a1 = qdiv(R(k65), k56 + R(k65));
      T8 = a1 * R(k52) + a1 * k54;
    }
  #pragma unroll
    for (int i = 0; i < kRyR; i++) {
      const int s = ryr_of(w, i);
      R r = k12;
      r = (s == 2) ? T2 : r;
      r = (s == 3) ? T3 : r;
      r = (s == 4) ? T4 : r;
      r = (s == 5) ? T5 : r;
      r = (s == 6) ? R(k65) : r;
      r = (s == 7) ? T7 : r;
      r = (s == 8) ? T8 : r;
      R0[2 + i] = r;
    }
  }
  R0[7] = (cl_of(w) == 1) ? R(kfIto2) * cass : R(kbIto2);
  R mx = R(0);
  #pragma unroll
  for (int j = 0; j < 8; j++) mx = imax(mx, R0[j]);
  mx = gmax(g, mx);
  // ---- substep size (simfru_local.c:135-146) ----
  R dtr = imin(rdiv(R(0.1), mx), R(10.001e-3));
  const R cmax = gmax(g, imax(R(0.e-3), cass));
  if (ilt(R(1.5e-3), cmax)) dtr = imin(dtr, R(5.001e-3));
  const R dt = F.clk.advance(dtr, L);
  // ---- Heun step (simfru_local.c:149-173) ----
  R dJ, dS;
  fcn_fru4(g, cajsr, cass, dep, e2, a2j, small, lopen, nopen, pca_scale, dJ, dS);
  const R k1J = dt * dJ, k1S = dt * dS;
  const R y1J = cajsr + k1J, y1S = cass + k1S;
  const R frac = F.clk.frac(L);
  #pragma unroll
  for (int i = 0; i < 3; i++) dep[i] = L.dep0[i] + frac * L.span[i];
  ghk_terms(dep[0], pca_scale, e2, a2j, small);
  fcn_fru4(g, y1J, y1S, dep, e2, a2j, small, lopen, nopen, pca_scale, dJ, dS);
  F.jsr.add((k1J + dt * dJ) / R(2));
  F.ss.add((k1S + dt * dS) / R(2));
  // ---- transitions of this cleft's 8 channels (:215-276) ----
  bool moved = false;
  if (leave_gt(bw[0], dt, R0[0])) {
    const LccBasisT<R> lb{alpha, beta, bp};
    R r[4];
    int d[4];
    const int len = lcc_row(lcc_of(w), lb, gam, r, d);
    w = set_field(w, 0, choose_dest(r, d, len, dt, bw[0]));
  }
  if (leave_ge(bw[1], dt, R0[1])) w = set_field(w, 4, 3 - vdi_of(w));
  // The RyRs that leave their state, then one pass per leaving RyR: the
  // lanes of a warp share the pass (one rate row and destination walk per
  // pass for every lane that has a RyR left), instead of one divergent body
  // per RyR index taken whenever any lane's RyR of that index leaves.  Each
  // RyR's row depends only on its own state and its cleft's constants, so
  // the order of the passes does not matter.
  unsigned pend = 0u;
  #pragma unroll
  for (int i = 0; i < kRyR; i++) pend |= leave_gt(bw[2 + i], dt, R0[2 + i]) ? (1u << i) : 0u;
  moved = pend != 0u;
  while (pend) {
    const int i = __ffs(pend) - 1;
    pend &= pend - 1u;
    uint32_t y = bw[2];  // the RyR's uniform, by selection (no dynamic register indexing)
    y = (i == 1) ? bw[3] : y;
    y = (i == 2) ? bw[4] : y;
    y = (i == 3) ? bw[5] : y;
    y = (i == 4) ? bw[6] : y;
    const RyrKT<R> k{k12, k23, k34, k54, k25, k56, regime};
    R r[4];
    int d[4];
    const int len = ryr_row(ryr_of(w, i), k, r, d);
    w = set_field(w, 8 + 4 * i, choose_dest(r, d, len, dt, y));
  }
  if (leave_ge(bw[7], dt, R0[7])) w = set_field(w, 28, 3 - cl_of(w));
  lopen = lcc_open(w) ? R(1) : R(0);
  if (moved) nopen = ryr_open_count(w);
  F.nsub++;
}

// Regenerate, with the whole warp, the MT rows whose draws in this substep
// run past word 624 (`go`: this lane's FRU takes a substep now).
template <typename R>
__device__ __forceinline__ void regen_step(const StageCtx& sc, int lane, const Group& g, bool go, const Fru4<R>& F,
                                           const Sub4<R>& S) {
  const bool cross = go && (F.mti + S.etot + 32 > kMtN);
  const unsigned cross_mask = __ballot_sync(0xffffffffu, cross && g.c == 0);
  const unsigned copy_mask = __ballot_sync(0xffffffffu, cross && g.c == 0 && *sc.my_hold_epoch != sc.p->epoch);
  if (cross_mask) regen_crossing(sc, lane, cross_mask, copy_mask);
}

// One FRU over [t0, tf] by its four lanes (simfru_local.c:83-277).  cajsr and
// cass are the FRU's FP64 state; arithmetic runs in R.  Every lane of the
// warp calls it together (live = false for a group without an FRU).
template <typename R>
__device__ __forceinline__ void advance4(StageCtx& sc, const Group& g, bool live, double& cajsr64, double& cass64,
                                         uint32_t& w, int& mti, uint32_t& nsub, bool& overflow) {
  LaneStage<R> L;
  lane_stage(*sc.p, g, L);
  Fru4<R> F;
  F.jsr.set(cajsr64);
  F.ss.set(cass64);
  F.w = w;
  F.mti = mti;
  F.nsub = nsub;
  fru_begin(F, L);
  const int lane = threadIdx.x & 31;
  while (true) {
    // all 32 lanes stay in the loop until every FRU of the warp is done, so
    // the warp can regenerate MT rows together; a group whose FRU has
    // reached tf (or never had one) idles
    bool go = live && F.clk.running(L);
    if (go && F.nsub >= (1u << 22)) {
      overflow = true;
      go = false;
    }
    if (!__any_sync(0xffffffffu, go)) break;
    Sub4<R> S;
    S.etot = 0;
#pragma unroll
    for (int i = 0; i < kRyR; i++) S.exw[i] = 0u;
    S.p34 = R(0);
    if (go) substep_a(F, S, L, g, sc);
    regen_step(sc, lane, g, go, F, S);
    if (go) substep_b(F, S, L, g, sc);
  }
  cajsr64 = F.jsr.get();
  cass64 = F.ss.get();
  w = F.w;
  mti = F.mti;
  nsub = F.nsub;
}

// Sum over the 32 lanes of a warp: one fixed shuffle tree.
template <int NV>
__device__ __forceinline__ void warp_sum(double v[NV]) {
#pragma unroll
  for (int k = 0; k < NV; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
}

// Cross-FRU sums of one cell, independent of the launch shape: every warp
// (8 FRUs, group grp of the cell's ngroups) stores its warp total, and the
// last warp to arrive adds the group totals in a fixed lane-strided order
// and one warp tree.  Whatever the warps per block, the sums are the same
// bits.  Returns true in lane 0 of that last warp, with the totals in tot[].
template <int NV>
__device__ __forceinline__ bool cell_finish(const double v[NV], double* partials, unsigned* ticket, double tot[NV],
                                            int grp, int ngroups) {
  const int lane = threadIdx.x & 31;
  unsigned last = 0u;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; k++) partials[grp * NV + k] = v[k];
    __threadfence();
    last = (atomicAdd(ticket, 1u) == (unsigned)ngroups - 1u) ? 1u : 0u;
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return false;
  __threadfence();
  double s[NV];
#pragma unroll
  for (int k = 0; k < NV; k++) s[k] = 0.0;
  for (int b = lane; b < ngroups; b += 32)
#pragma unroll
    for (int k = 0; k < NV; k++) s[k] += __ldcg(&partials[b * NV + k]);
  warp_sum<NV>(s);
  if (lane == 0) {
    *ticket = 0u;
#pragma unroll
    for (int k = 0; k < NV; k++) tot[k] = s[k];
  }
  return lane == 0;
}

// The stage of one cell, block bidx of the cell's blocks (blockDim.x / 32
// warps of 8 FRUs each): load, optional snapshot save/restore, advance,
// store, and the fused deterministic flux reduction
// (calc_fru_flux_local.c:28-77, mpi_master.c:447-468, mpi_slave.c:150-226);
// the cell's totals go to out[0..8] and its error flag to out[kOutError].
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Where a launch's cell totals go: OutFin writes them to the cell's out[]
// slots (the host reads them back); the device-resident integrator passes
// its own finisher.  Called by one lane, with the 5 flux numerators, the
// currents (Jxfer, Jtr, ICa, Ito2) and, when the launch carried
// kFlagAvg, the 11 output-average sums (else null).
struct OutFin {
  double* out;
  __device__ void operator()(const double tot[5], const double cur[4], const double*) const {
#pragma unroll
    for (int k = 0; k < 5; k++) out[k] = tot[k];
#pragma unroll
    for (int k = 0; k < 4; k++) out[5 + k] = cur[k];
  }
  __device__ void error() const { out[kOutError] = 1.0; }
};

// The 11 output-average terms of one cleft (calc_fru_avg_local.c:27-105):
// the FRU-level ones (CaJSR and its buffered total) on the cleft-0 lane.
__device__ __forceinline__ void avg_terms(int c, double jsr, double ss, uint32_t w, double a[11]) {
  int no = 0, ready = 0;
#pragma unroll
  for (int i = 0; i < kRyR; i++) {
    const int r = ryr_of(w, i);
    no += ryr_open(r);
    ready += (r == 1 || r == 2);
  }
  a[0] = ss;
  a[1] = (c == 0) ? jsr : 0.0;
  a[2] = JRyRmax * ((double)no) * (jsr - ss);
  a[3] = (double)no;
  a[4] = (double)ready;
  a[5] = ss * (1.0 + BSRtot / (KBSR + ss) + BSLtot / (KBSL + ss));
  a[6] = (c == 0) ? jsr * (1.0 + CSQNtot / (KmCSQN + jsr)) : 0.0;
  a[7] = (lcc_of(w) <= 6) ? 1.0 : 0.0;
  a[8] = (vdi_of(w) == 2) ? 1.0 : 0.0;
  a[9] = lcc_open(w) ? 1.0 : 0.0;
  a[10] = (cl_of(w) == 2) ? 1.0 : 0.0;
}

template <typename R, typename Fin>
__device__ __forceinline__ void stage_body_fin(const DevState& s, const StageParams& p, int bidx, const Fin& fin) {
  const int lane = threadIdx.x & 31;
  const int grp = bidx * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5);
  const int ngroups = (s.nfru + 7) >> 3;
  if ((p.flags & kFlagQueueReset) && bidx == 0 && threadIdx.x == 0) {
    // after a packed launch: ready the queue for the next one (the heavy-FRU
    // threshold becomes 3x this launch's mean substeps per FRU, at least 8)
    const uint32_t n = (uint32_t)s.nfru;
    const uint32_t thr = 3u * (s.qctl[3] / (n ? n : 1u));
    s.qctl[4] = thr > 8u ? thr : 8u;
    s.qctl[3] = 0u;
    s.qctl[0] = 0u;
    s.qctl[1 + ((p.launch + 1u) & 1u)] = 0u;
  }
  if (grp >= ngroups) return;  // whole warps past the cell's last FRU
  if (s.trace_ns && lane == 0) s.trace_ns[2 * grp] = global_ns();
  Group g;
  g.c = lane & 3;
  g.base = lane & ~3;
  g.mask = 0xfu << g.base;
  const int f = grp * 8 + (lane >> 2);
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  uint32_t nsub = 0;
  bool overflow = false;
  const bool active = f < s.nfru;  // uniform over each 4-lane group
  const size_t nf = (size_t)s.stride;
  double cajsr = 0.0, cass = 0.0;
  uint32_t w = 0u;
  int mti = 0;
  uint32_t* gm = s.mt + (size_t)f * kMtStride;
  StageCtx sc;
  sc.p = &p;
  sc.m = gm;
  sc.hold_base = s.mt_hold;
  sc.hold_epoch_base = s.hold_epoch;
  sc.f = f;
  sc.my_hold_epoch = s.hold_epoch + f;  // within the padded arrays even past the last FRU
  bool restore = false;
  if (active) {
    if (p.flags & kFlagResume) {
      cajsr = s.frus_s[f];
      cass = s.frus_s[(g.c + 1) * nf + f];
      w = s.chan_s[g.c * nf + f];
      mti = s.mti_s[f];
      restore = (*sc.my_hold_epoch == p.epoch);
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
  }
  const uint32_t* hold = sc.hold_base + (size_t)f * kMtStride;
  if (p.flags & kFlagAdvance) {
    if (active) use_row(sc, gm, hold, restore, g);
    __syncwarp();
    advance4<R>(sc, g, active, cajsr, cass, w, mti, nsub, overflow);
    __syncwarp();
  } else if (active && restore) {
    copy_row16(gm, hold, g);
  }
  if (active) {
    if (s.trace_sub && g.c == 0) s.trace_sub[f] = nsub;
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
  if (s.trace_ns && lane == 0) s.trace_ns[2 * grp + 1] = global_ns();
  if (overflow) fin.error();
  if (s.substeps) {
    unsigned long long c = (g.c == 0) ? nsub : 0;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0 && c) atomicAdd(s.substeps, c);
  }
  if (p.flags & kFlagAvg) {
    // flux numerators and output averages in one pass (16 partials per group)
    double u[16];
#pragma unroll
    for (int k = 0; k < 5; k++) u[k] = v[k];
    double a[11];
    avg_terms(g.c, cajsr, cass, w, a);
#pragma unroll
    for (int k = 0; k < 11; k++) u[5 + k] = active ? a[k] : 0.0;
    warp_sum<16>(u);
    double tot[16];
    if (cell_finish<16>(u, s.partials, s.ticket, tot, grp, ngroups)) {
      double cur[4];
      currents_from_sums(s.nfru, p.nfru_scale, p.depf, tot, cur);
      cur[2] = cur[2] * p.pca_scale;  // ICa is proportional to the LCC permeability
      fin(tot, cur, tot + 5);
    }
    return;
  }
  warp_sum<5>(v);
  double tot[5];
  if (cell_finish<5>(v, s.partials, s.ticket, tot, grp, ngroups)) {
    double cur[4];
    currents_from_sums(s.nfru, p.nfru_scale, p.depf, tot, cur);
    cur[2] = cur[2] * p.pca_scale;  // ICa is proportional to the LCC permeability
    fin(tot, cur, nullptr);
  }
}

template <typename R>
__device__ __forceinline__ void stage_body(const DevState& s, const StageParams& p, int bidx, double* out) {
  stage_body_fin<R>(s, p, bidx, OutFin{out});
}

// ---- packed stage: a queue of FRUs per 4-lane group -----------------------------
// A warp's eight 4-lane groups each advance one FRU at a time and, when it
// reaches tf, store it and take the next from the cell's queue, so a warp's
// lanes stay busy until the queue is empty instead of idling behind the
// slowest of eight fixed FRUs.  The queue hands out first the FRUs that were
// heavy (many substeps) in the cell's previous packed launch, then the others
// in order.  The per-FRU arithmetic is advance4's, so every FRU ends in the
// same state as with the fixed layout; the flux sums come from a following
// non-advancing launch over the stored states, in the usual fixed order.
template <typename R>
__device__ __forceinline__ void stage_body_packed(const DevState& s, const StageParams& p, double* out) {
  const int lane = threadIdx.x & 31;
  Group g;
  g.c = lane & 3;
  g.base = lane & ~3;
  g.mask = 0xfu << g.base;
  const size_t nf = (size_t)s.stride;
  const int n = s.nfru;
  const uint32_t L = p.launch;
  const int* heavy_prev = s.heavy_list + (size_t)((L + 1u) & 1u) * nf;
  int* heavy_next = s.heavy_list + (size_t)(L & 1u) * nf;
  // tags by launch parity too: this launch re-tags the FRUs it finds heavy
  // without changing what its own queue skips
  const uint32_t* tag_prev = s.heavy_tag + (size_t)((L + 1u) & 1u) * nf;
  uint32_t* tag_next = s.heavy_tag + (size_t)(L & 1u) * nf;
  const unsigned H = s.qctl[1 + ((L + 1u) & 1u)];
  const unsigned thr = s.qctl[4];
  LaneStage<R> LS;
  lane_stage(p, g, LS);
  StageCtx sc;
  sc.p = &p;
  sc.m = s.mt;
  sc.hold_base = s.mt_hold;
  sc.hold_epoch_base = s.hold_epoch;
  sc.f = 0;
  sc.my_hold_epoch = s.hold_epoch;
  Fru4<R> F;
  F.clk = {};
  F.jsr.set(0.0);
  F.ss.set(0.0);
  F.w = 0u;
  F.nsub = 0u;
  F.mti = 0;
  int f = -1;
  bool overflow = false;
  // the next FRU of the queue (every lane of the group gets it; -1: none left)
  auto take = [&]() -> int {
    int got = -1;
    if (g.c == 0) {
      for (int tries = 0; tries <= n + (int)H; tries++) {
        const unsigned i = atomicAdd(s.qctl, 1u);
        if (i < H) {
          got = heavy_prev[i];
          break;
        }
        const unsigned j = i - H;
        if (j >= (unsigned)n) break;
        if (H == 0u || tag_prev[j] != L) {  // tag L: in the previous launch's heavy list
          got = (int)j;
          break;
        }
      }
    }
    return __shfl_sync(g.mask, got, g.base);
  };
  auto load = [&](int ff) {
    f = ff;
    sc.f = ff;
    sc.my_hold_epoch = s.hold_epoch + ff;
    bool restore = false;
    if (p.flags & kFlagResume) {
      F.jsr.set(s.frus_s[ff]);
      F.ss.set(s.frus_s[(g.c + 1) * nf + ff]);
      F.w = s.chan_s[g.c * nf + ff];
      F.mti = s.mti_s[ff];
      restore = (*sc.my_hold_epoch == p.epoch);
    } else {
      F.jsr.set(s.frus[ff]);
      F.ss.set(s.frus[(g.c + 1) * nf + ff]);
      F.w = s.chan[g.c * nf + ff];
      F.mti = s.mti[ff];
    }
    if (p.flags & kFlagSave) {
      if (g.c == 0) {
        s.frus_s[ff] = F.jsr.get();
        s.mti_s[ff] = F.mti;
      }
      s.frus_s[(g.c + 1) * nf + ff] = F.ss.get();
      s.chan_s[g.c * nf + ff] = F.w;
    }
    use_row(sc, s.mt + (size_t)ff * kMtStride, s.mt_hold + (size_t)ff * kMtStride, restore, g);
    F.nsub = 0u;
    fru_begin(F, LS);
  };
  auto finish = [&]() {
    if (g.c == 0) {
      s.frus[f] = F.jsr.get();
      s.mti[f] = F.mti;
      if (s.trace_sub) s.trace_sub[f] = F.nsub;
      atomicAdd(&s.qctl[3], F.nsub);
      if (s.substeps) atomicAdd(s.substeps, (unsigned long long)F.nsub);
      if (F.nsub >= thr && thr > 0u) {
        tag_next[f] = L + 1u;
        heavy_next[atomicAdd(&s.qctl[1 + (L & 1u)], 1u)] = f;
      }
    }
    s.frus[(g.c + 1) * nf + f] = F.ss.get();
    s.chan[g.c * nf + f] = F.w;
  };
  {
    const int ff = take();
    if (ff >= 0) load(ff);
  }
  __syncwarp();
  while (true) {
    const bool has = f >= 0;
    bool go = has && F.clk.running(LS);
    if (go && F.nsub >= (1u << 22)) {
      overflow = true;
      go = false;
    }
    if (!__any_sync(0xffffffffu, has)) break;
    Sub4<R> S;
    S.etot = 0;
#pragma unroll
    for (int i = 0; i < kRyR; i++) S.exw[i] = 0u;
    S.p34 = R(0);
    if (go) substep_a(F, S, LS, g, sc);
    regen_step(sc, lane, g, go, F, S);
    if (go) substep_b(F, S, LS, g, sc);
    // a group whose FRU reached tf stores it and takes the next one
    if (has && !(go && F.clk.running(LS))) {
      finish();
      f = -1;
      const int ff = take();
      if (ff >= 0) load(ff);
    }
    __syncwarp();
  }
  if (overflow) out[kOutError] = 1.0;
}

// ---- many cells in one launch ------------------------------------------------
// Cell i owns blocks block0[i] .. block0[i+1]-1 of the grid (8 FRUs per
// warp); its parameters are params[i] and its totals go to outs[i*32 ..].
template <typename R>
__device__ __forceinline__ void batch_body(const BatchArgs& a) {
  // the cell of this block: binary search of the block prefix sums
  int lo = 0, hi = a.ncells - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&a.block0[mid]) <= b) lo = mid;
    else hi = mid - 1;
  }
  // the cell's arrays and parameters are read where used (through L1)
  // rather than copied into registers
  const DevState& s = a.cells[lo];
  const StageParams& p = a.params[lo];
  if (p.flags < 0) return;  // the cell posted no operation this round
  stage_body<R>(s, p, b - a.block0[lo], a.outs + kBatchOutStride * lo);
}

}  // namespace cleft
}  // namespace gw
