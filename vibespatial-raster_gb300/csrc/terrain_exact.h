// TRI and TPI of a 3x3 float32 window as exact integers, when the window
// allows it.
//
// If the nine values are finite, non-zero, of one sign and their exponents
// span at most 2, each is N_k 2^E with N_k an integer below 2^26 and E the
// smallest exponent's unit: the differences d_k = z_k - z_4 are exact
// integers N_k - N_4 in units of 2^E, and
//   TRI = sum |d_k| / 8,   TPI = z_4 - mean(z_k) = -sum d_k / 8
// are integers below 2^30 times 2^E / 8.  The reference forms both in
// float64, where every term and partial sum is such a multiple with at most
// 30 significant bits, so its results are these exact values: the integer
// forms give the same float64 bits without double-float arithmetic.
// Windows outside these bounds keep the double-float path.
//
// Plain C so that the host test compiles it with gcc and compares it with
// float64 arithmetic; CUDA includes it as host-device functions.
#ifndef VSR_TERRAIN_EXACT_H
#define VSR_TERRAIN_EXACT_H

#include <stdint.h>

#if defined(__CUDACC__)
#define VSR_TE_FN __host__ __device__ __forceinline__
#else
#define VSR_TE_FN static inline
#endif

// b: the nine values' bit patterns (row-major window, centre b[4]).  On
// success returns 1 with TRI = tri8 2^e2 / 8 and TPI = tpi8 2^e2 / 8 (tri8
// >= 0; tpi8 signed), e2 the unit exponent.
VSR_TE_FN int vsr_tt_exact(const uint32_t b[9], int32_t* tri8, int32_t* tpi8, int* e2) {
  uint32_t emin = 255u, emax = 0u, sor = 0u, sand = 0x80000000u;
  for (int k = 0; k < 9; ++k) {
    const uint32_t e = (b[k] >> 23) & 0xffu;
    emin = e < emin ? e : emin;
    emax = e > emax ? e : emax;
    sor |= b[k];
    sand &= b[k];
  }
  // finite and normal (no zero, subnormal, inf, NaN), one sign, span <= 2
  if (emin == 0u || emax == 255u || emax - emin > 2u) return 0;
  if ((sor & 0x80000000u) != (sand & 0x80000000u)) return 0;
  int32_t n[9];
  for (int k = 0; k < 9; ++k) {
    const uint32_t e = (b[k] >> 23) & 0xffu;
    n[k] = (int32_t)(((b[k] & 0x7fffffu) | 0x800000u) << (e - emin));  // < 2^26
  }
  int32_t ta = 0, ts = 0;
  for (int k = 0; k < 9; ++k) {
    if (k == 4) continue;
    const int32_t d = n[k] - n[4];
    ta += d < 0 ? -d : d;
    ts += d;
  }
  // negative values: z = -n 2^E, so every difference changes sign
  const int neg = (sand & 0x80000000u) != 0u;
  *tri8 = ta;
  *tpi8 = neg ? ts : -ts;  // TPI = -sum d / 8
  *e2 = (int)emin - 150;
  return 1;
}

// The float64 bits of s 2^e (|s| < 2^31, exact): +0.0 for s == 0.
VSR_TE_FN uint64_t vsr_int_scaled_bits(int32_t s, int e) {
  if (s == 0) return 0u;
  const uint64_t sign = s < 0 ? 1u : 0u;
  const uint32_t a = s < 0 ? (uint32_t)(-(int64_t)s) : (uint32_t)s;
#if defined(__CUDA_ARCH__)
  const int p = 31 - __clz(a);  // the leading bit of a
#else
  const int p = 31 - __builtin_clz(a);
#endif
  const uint64_t frac = ((uint64_t)a << (52 - p)) & ((1ull << 52) - 1ull);
  return (sign << 63) | ((uint64_t)(p + e + 1023) << 52) | frac;
}

#endif
