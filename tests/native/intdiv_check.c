/* Checks gw_div_rn (the integer-pipe division of the FRU kernels) against the
 * C division: n random operand pairs drawn from the bit patterns of normal
 * doubles (all exponents and, in a second pass, the operand ranges of the
 * FRU substep), plus boundary mantissas.  Prints the mismatches found. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gw_intdiv.h"

static uint64_t s_state = 0x9e3779b97f4a7c15ull;
static uint64_t next(void) { /* splitmix64 */
  uint64_t z = (s_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double from_bits(uint64_t u) {
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
}
static uint64_t to_bits(double x) {
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
}

static long bad = 0;
static void check(double a, double b) {
  volatile double q = a / b;
  const double g = gw_div_rn(a, b);
  if (to_bits(q) != to_bits(g) && !(q != q && g != g)) {
    if (bad < 10) printf("mismatch: %a / %a = %a, got %a\n", a, b, (double)q, g);
    bad++;
  }
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 10000000;
  if (argc > 2) s_state = strtoull(argv[2], NULL, 10);
  /* any normal or special bit patterns */
  for (long i = 0; i < n; i++) check(from_bits(next()), from_bits(next()));
  /* operands of the FRU substep's divisions: magnitudes 1e-8 .. 1e4 */
  for (long i = 0; i < n; i++) {
    const uint64_t ea = 1023 - 27 + next() % 41, eb = 1023 - 27 + next() % 41;
    const uint64_t a = (next() & 0x800fffffffffffffull) | (ea << 52);
    const uint64_t b = (next() & 0x800fffffffffffffull) | (eb << 52);
    check(from_bits(a), from_bits(b));
  }
  /* boundary mantissas: all ones, all zeros, one ulp either side, near-equal */
  const uint64_t mants[] = {0, 1, 2, 0x000fffffffffffffull, 0x000ffffffffffffeull, 0x0008000000000000ull,
                            0x0007ffffffffffffull, 0x0008000000000001ull, 0x0005555555555555ull,
                            0x000aaaaaaaaaaaaaull, 0x0001000000000000ull, 0x000f000000000000ull};
  const int nm = sizeof mants / sizeof mants[0];
  for (int i = 0; i < nm; i++)
    for (int j = 0; j < nm; j++)
      for (int ea = 1; ea < 2047; ea += 7)
        for (int s = 0; s < 4; s++) {
          const uint64_t eb = 1 + (uint64_t)((ea * 13 + s * 331) % 2046);
          check(from_bits(((uint64_t)(s & 1) << 63) | ((uint64_t)ea << 52) | mants[i]),
                from_bits(((uint64_t)(s >> 1) << 63) | (eb << 52) | mants[j]));
        }
  /* special values */
  const double sp[] = {0.0, -0.0, 1.0, -1.0, 1e-310, -1e-310, 1e308, 4.9e-324, 1.0 / 0.0, -1.0 / 0.0, 0.0 / 0.0};
  for (int i = 0; i < 11; i++)
    for (int j = 0; j < 11; j++) check(sp[i], sp[j]);
  printf("%ld mismatches in %ld divisions\n", bad, 2 * n + (long)nm * nm * 293 * 4 + 121);
  return bad != 0;
}
