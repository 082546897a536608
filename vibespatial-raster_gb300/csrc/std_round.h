// sqrt(N) / n rounded to the nearest float32 (ties to even), for the exact
// integer variance numerators of the 8/16-bit focal std
// (N = n sum x^2 - (sum x)^2, so std = sqrt(N) / n), without FP64: a float32
// estimate (within two ulps) corrected by exact comparisons of sqrt(N) / n
// with the rounding midpoints next to it.  A midpoint a 2^b (a odd) is
// crossed when N 2^(-2b) >= (a n)^2; both sides are formed as 128-bit
// integers (two 64-bit words).
//
// Plain C so that the host test compiles it with gcc and checks it against
// a long-double reference; CUDA includes it as device functions.
#ifndef VSR_STD_ROUND_H
#define VSR_STD_ROUND_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define VSR_SR_FN __device__ __forceinline__
#define VSR_SR_MULHI(a, b) __umul64hi((a), (b))
#else
#define VSR_SR_FN static inline
#define VSR_SR_MULHI(a, b) ((uint64_t)(((unsigned __int128)(a) * (b)) >> 64))
#endif

VSR_SR_FN uint32_t vsr_sr_bits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}
VSR_SR_FN float vsr_sr_float(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

// sign of sqrt(N)/n - a 2^b for a >= 1 odd, b < 0 (-1, 0 or +1): compares
// N 2^(-2b) with (a n)^2.
VSR_SR_FN int vsr_sr_cmp(uint64_t N, uint32_t n, uint64_t a, int b) {
  const int s = -2 * b;  // > 0
  uint64_t nh, nl;
  if (s >= 64) {
    nh = N << (s - 64);
    nl = 0;
  } else {
    nh = N >> (64 - s);
    nl = N << s;
  }
  const uint64_t p = a * n;  // < 2^40
  const uint64_t ph = VSR_SR_MULHI(p, p), pl = p * p;
  if (nh != ph) return nh > ph ? 1 : -1;
  if (nl != pl) return nl > pl ? 1 : -1;
  return 0;
}

// N < 2^62, 1 <= n < 2^14, and sqrt(N)/n < 2^24 (so that every midpoint
// exponent b is negative).
VSR_SR_FN float vsr_std_f32(uint64_t N, uint32_t n) {
  if (N == 0) return 0.0f;
  float y = sqrtf((float)N) / (float)n;
  for (int it = 0; it < 6; ++it) {
    const uint32_t u = vsr_sr_bits(y);
    const int ex = (int)((u >> 23) & 0xffu) - 150;  // y = m 2^ex
    const uint64_t m = (u & 0x7fffffu) | 0x800000u;
    // above the upper midpoint (2m + 1) 2^(ex - 1): round up; exactly on it: to even
    const int up = vsr_sr_cmp(N, n, 2 * m + 1, ex - 1);
    if (up > 0 || (up == 0 && (m & 1u))) {
      y = vsr_sr_float(u + 1u);
      continue;
    }
    // below the lower midpoint (one ulp of the binade below when m = 2^23)
    const int lo = m > 0x800000u ? vsr_sr_cmp(N, n, 2 * m - 1, ex - 1) : vsr_sr_cmp(N, n, 4 * m - 1, ex - 2);
    if (lo < 0 || (lo == 0 && (m & 1u))) {
      y = vsr_sr_float(u - 1u);
      continue;
    }
    break;
  }
  return y;
}

// The same for windows of at most 127 taps (n < 2^7): every (a n) with
// a < 2^25 is below 2^32, so its square fits one 64-bit word and a midpoint
// test is a shift and a 64-bit compare.
VSR_SR_FN int vsr_sr_cmp_small(uint64_t N, uint32_t n, uint64_t a, int b) {
  const int s = -2 * b;  // > 0
  const uint64_t p = a * n, pp = p * p;
  if (s >= 64 || (N >> (64 - s)) != 0) return N ? 1 : -1;  // N 2^s >= 2^64 > pp (N > 0 here)
  const uint64_t ns = N << s;
  return ns > pp ? 1 : (ns < pp ? -1 : 0);
}

VSR_SR_FN float vsr_std_f32_small(uint64_t N, uint32_t n) {
  if (N == 0) return 0.0f;
  // estimate within two ulps: N through two 32-bit halves (no 64-bit
  // conversion), correctly rounded sqrt and division
  const float nf = (float)(uint32_t)(N >> 32) * 4294967296.0f + (float)(uint32_t)N;
  const uint32_t u = vsr_sr_bits(sqrtf(nf) / (float)n);
  // the result is u - 2 .. u + 2: count the midpoints between consecutive
  // candidates that lie below sqrt(N)/n (a tie goes to the even candidate);
  // the midpoint above float ud is (2 m + 1) 2^(ex - 1) for ud = m 2^ex,
  // across a binade boundary too.  No branch: every lane runs the same four
  // tests.
  int k = -2;
#pragma unroll
  for (int d = -2; d < 2; ++d) {
    const uint32_t ud = u + (uint32_t)d;
    const int ex = (int)((ud >> 23) & 0xffu) - 150;
    const uint64_t m = (ud & 0x7fffffu) | 0x800000u;
    const int c = vsr_sr_cmp_small(N, n, 2 * m + 1, ex - 1);
    k += (c > 0 || (c == 0 && (ud & 1u))) ? 1 : 0;
  }
  return vsr_sr_float(u + (uint32_t)k);
}

#endif
