/*
 * Correctly rounded FP64 division on the integer pipe.
 *
 * GB300 issues one FP64 warp instruction per 64 cycles per SM sub-partition,
 * and a hardware-sequence double division takes about six of those slots,
 * while integer instructions issue every cycle.  The FRU stage kernels divide
 * about fifteen times per lane and substep, so moving division off the FP64
 * pipe frees it for the rest of the substep.  The quotient is the IEEE-754
 * round-to-nearest-even one, bit for bit, so results do not change.
 *
 * Method (for normal operands whose quotient is normal; anything else --
 * zeros, subnormals, infinities, NaNs, underflow, overflow -- takes the
 * ordinary division):
 *   1. a = ma 2^(ea-1075), b = mb 2^(eb-1075) with 53-bit integer mantissas;
 *      n = ma, or 2 ma when ma < mb, so that n / mb lies in [1, 2).
 *   2. W ~ 2^116 / mb, a 64-bit fixed-point reciprocal: a single-precision
 *      reciprocal of mb's leading 24 bits (about 22 correct bits), then two
 *      Newton-Raphson steps W += W (2^116 - mb W) / 2^116 in integer
 *      arithmetic (about 44, then about 62 bits).
 *   3. Q = floor(n W / 2^64) is floor(n 2^52 / mb) or one less; the exact
 *      remainder R = n 2^52 - Q mb (it fits in 64 bits) corrects it.
 *   4. Rounding from 2R against mb: above -> up, equal -> to even.
 * The same code runs on the host, where tests compare it with the C
 * division on random and boundary operands.
 */
#ifndef GW_INTDIV_H
#define GW_INTDIV_H

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define GW_ID_HD __host__ __device__ static inline
#else
#define GW_ID_HD static inline
#endif

GW_ID_HD uint64_t gw_id_bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

GW_ID_HD double gw_id_double(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

/* high 64 bits of a 64 x 64-bit product */
GW_ID_HD uint64_t gw_id_mulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

/* 1 / f for f in [1, 2), rounded to single precision (the seed) */
GW_ID_HD float gw_id_rcpf(float f) {
#ifdef __CUDA_ARCH__
  return __frcp_rn(f);
#else
  volatile float one = 1.0f;
  return one / f;
#endif
}

/* a / b, rounded to nearest even. */
GW_ID_HD double gw_div_rn(double a, double b) {
  const uint64_t M52 = 0x000fffffffffffffull, IMPL = 0x0010000000000000ull;
  const uint64_t ua = gw_id_bits(a), ub = gw_id_bits(b);
  const int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
  const uint64_t ma = (ua & M52) | IMPL, mb = (ub & M52) | IMPL;
  const int lt = ma < mb;
  const int e = ea - eb + 1023 - lt; /* biased exponent of the quotient */
  if (ea == 0 || ea == 0x7ff || eb == 0 || eb == 0x7ff || e <= 0 || e >= 0x7fe) return a / b;
  const uint64_t n = lt ? (ma << 1) : ma; /* n / mb in [1, 2) */
  /* seed: mb's leading 24 bits as a float in [1, 2) and its reciprocal */
  uint32_t fb = 0x3f800000u | (uint32_t)((mb >> 29) & 0x7fffffu);
  float f;
  memcpy(&f, &fb, sizeof f);
  const float r = gw_id_rcpf(f); /* (0.5, 1] */
  uint32_t rb;
  memcpy(&rb, &r, sizeof rb);
  /* W = r 2^64: r = m 2^-24 with m in [2^23, 2^24) for r < 1 */
  uint64_t W = (rb >= 0x3f800000u) ? 0xffffffffffffffffull : (((uint64_t)((rb & 0x7fffffu) | 0x800000u)) << 40);
  for (int it = 0; it < 2; it++) {
    /* P = mb W (117 bits) as hi:lo; E = 2^116 - P (signed, small) */
    const uint64_t plo = mb * W, phi = gw_id_mulhi(mb, W);
    /* 2^116 = (2^52) : 0 */
    const uint64_t elo = (uint64_t)0 - plo;
    const uint64_t ehi = ((uint64_t)1 << 52) - phi - (plo != 0);
    const int neg = (int64_t)ehi < 0;
    /* |E| >> 52, and W |E| / 2^116 = mulhi(W, |E| >> 52) */
    uint64_t mhi = ehi, mlo = elo;
    if (neg) {
      mlo = (uint64_t)0 - elo;
      mhi = ~ehi + (elo == 0);
    }
    const uint64_t e52 = (mhi << 12) | (mlo >> 52);
    const uint64_t corr = gw_id_mulhi(W, e52);
    W = neg ? W - corr : W + corr;
  }
  /* quotient estimate and exact remainder */
  uint64_t Q = gw_id_mulhi(n, W);
  int64_t R = (int64_t)((n << 52) - Q * mb);
  if (R < 0) {
    Q -= 1;
    R += (int64_t)mb;
  }
  if (R >= (int64_t)mb) {
    Q += 1;
    R -= (int64_t)mb;
  }
  if (R >= (int64_t)mb) {
    Q += 1;
    R -= (int64_t)mb;
  }
  /* round to nearest, ties to even */
  const uint64_t twice = (uint64_t)R << 1;
  const uint64_t up = (twice > mb) || (twice == mb && (Q & 1u));
  /* Q in [2^52, 2^53): a carry out of the mantissa bumps the exponent */
  const uint64_t bits = ((ua ^ ub) & 0x8000000000000000ull) + ((((uint64_t)e) << 52) + (Q - IMPL) + up);
  return gw_id_double(bits);
}

#endif /* GW_INTDIV_H */
