/* Host check of vsr_tt_exact and vsr_int_scaled_bits (csrc/terrain_exact.h):
 * on random 3x3 float32 windows (DEM-like values, sea-level crossings,
 * negative and tiny values, spans of one to three binades) every window the
 * integer path accepts must give exactly the float64 bits of
 *   TRI = (|z0-z4| + ... + |z8-z4|) / 8   (float64, left to right)
 *   TPI = z4 - (z0 + ... + z8 without z4) / 8
 * the reference's formulas.  Prints "n accepted mismatches". */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "terrain_exact.h"

static uint64_t state = 0x2545F4914F6CDD1Dull;
static uint64_t next(void) {
  state ^= state << 13;
  state ^= state >> 7;
  state ^= state << 17;
  return state;
}
static double unit(void) { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }

int main(int argc, char** argv) {
  const long count = argc > 1 ? atol(argv[1]) : 1000000;
  long accepted = 0, bad = 0;
  for (long it = 0; it < count; ++it) {
    const int mode = (int)(next() % 5);
    double base = mode == 0 ? 3000.0 * unit() : (mode == 1 ? 2.0 * unit() - 1.0 : (mode == 2 ? -500.0 * unit() : 1e-3 * unit()));
    if (mode == 4) base = 1000.0 + 0.01 * unit();
    const double spread = mode == 4 ? 0.001 : (mode == 3 ? 1e-3 : 50.0);
    float z[9];
    uint32_t b[9];
    for (int k = 0; k < 9; ++k) {
      z[k] = (float)(base + spread * (unit() - 0.5));
      memcpy(&b[k], &z[k], 4);
    }
    int32_t t8, p8;
    int e2;
    if (!vsr_tt_exact(b, &t8, &p8, &e2)) continue;
    ++accepted;
    double tri = 0.0, sum = 0.0;
    for (int k = 0; k < 9; ++k) {
      if (k == 4) continue;
      tri += fabs((double)z[k] - (double)z[4]);
      sum += (double)z[k];
    }
    tri /= 8.0;
    const double tpi = (double)z[4] - sum / 8.0;
    uint64_t rt, rp;
    memcpy(&rt, &tri, 8);
    memcpy(&rp, &tpi, 8);
    const uint64_t gt = vsr_int_scaled_bits(t8, e2 - 3), gp = vsr_int_scaled_bits(p8, e2 - 3);
    if (gt != rt || gp != rp) {
      if (bad < 5) printf("mismatch tri %016llx/%016llx tpi %016llx/%016llx\n", (unsigned long long)gt,
                          (unsigned long long)rt, (unsigned long long)gp, (unsigned long long)rp);
      ++bad;
    }
  }
  printf("%ld %ld %ld\n", count, accepted, bad);
  return bad != 0;
}
