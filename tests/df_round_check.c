/* Host check of the integer float-to-double widening (csrc/df_round.h):
 * every float it accepts must give exactly the bits of the compiler's
 * (double) conversion, and it must accept every normal float and both
 * zeros.  Walks all 2^32 float bit patterns when given "all", else a
 * strided sample.  Prints "n accepted mismatches"; exits non-zero on a
 * mismatch or a wrongly declined value. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "df_round.h"

int main(int argc, char** argv) {
  const uint64_t step = (argc > 1 && strcmp(argv[1], "all") == 0) ? 1u : 977u;
  uint64_t n = 0, accepted = 0, bad = 0;
  for (uint64_t u = 0; u < (1ull << 32); u += step) {
    const uint32_t b = (uint32_t)u;
    float f;
    memcpy(&f, &b, 4);
    const uint32_t e = b & 0x7f800000u;
    const int normal_or_zero = e != 0x7f800000u && (e != 0u || (b << 1) == 0u);
    ++n;
    if (vsr_f32_widen_ok(b) != normal_or_zero) {
      ++bad;
      continue;
    }
    if (!normal_or_zero) continue;
    ++accepted;
    const double d = (double)f;
    uint64_t ref, got;
    uint32_t hw, lw;
    memcpy(&ref, &d, 8);
    vsr_f32_widen(b, &hw, &lw);
    got = ((uint64_t)hw << 32) | lw;
    if (got != ref) {
      if (bad < 5) printf("mismatch %08x: %016llx vs %016llx\n", b, (unsigned long long)got, (unsigned long long)ref);
      ++bad;
    }
  }
  printf("%llu %llu %llu\n", (unsigned long long)n, (unsigned long long)accepted, (unsigned long long)bad);
  return bad != 0;
}
