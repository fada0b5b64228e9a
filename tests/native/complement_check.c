/* The identity the mixed-precision transition tests rely on
 * (greenstein2002_gb300/csrc/gw_fru_cleft.cuh, comp_u32): for every 32-bit
 * MT19937 output y, 2^32 - y rounded to FP32 equals the FP32 conversion of
 * the 32-bit integer 0 - y (which wraps to 2^32 - y for y > 0), with y = 0
 * giving 2^32.  Checked for all 2^32 values of y. */
#include <stdint.h>
#include <stdio.h>

int main(void) {
  unsigned long long bad = 0;
  for (uint64_t y = 0; y <= 0xffffffffull; y++) {
    const uint32_t v = (uint32_t)y;
    const float wide = (float)(4294967296ull - (uint64_t)v);
    const float narrow = v ? (float)(0u - v) : 4294967296.0f;
    if (wide != narrow) {
      if (bad < 5) printf("y = %u: %.9g vs %.9g\n", v, wide, narrow);
      bad++;
    }
  }
  printf("mismatches: %llu of 4294967296\n", bad);
  return bad != 0;
}
