// Widening a float to a double with 32-bit integer operations.
//
// The FP64 pipe of a GB300 SM is narrow.  The terrain-derivative kernel
// writes three float64 outputs per pixel, each the sum of a double-float
// pair (hi, lo); converting both floats in FP64 and adding them (three FP64
// operations per value) bounded the kernel.  A normal or zero float's double
// bits are its own bits rearranged (exponent rebiased by 1023 - 127, the
// significand shifted up by 29), so the two conversions become a few
// integer operations and only the add stays in FP64; the result is the same
// double as (double)hi + (double)lo.  Subnormal and non-finite floats are
// reported so that the caller converts them in FP64.
//
// Plain C so that the host test compiles it with gcc and compares it with
// the compiler's conversion; CUDA includes it as a host-device function.
#ifndef VSR_DF_ROUND_H
#define VSR_DF_ROUND_H

#include <stdint.h>

#if defined(__CUDACC__)
#define VSR_DF_FN __host__ __device__ __forceinline__
#else
#define VSR_DF_FN static inline
#endif

// 1 when the float with bits ``b`` is normal or a signed zero (the integer
// widening applies), 0 for subnormal, infinite and NaN values.
VSR_DF_FN int vsr_f32_widen_ok(uint32_t b) {
  const uint32_t e = b & 0x7f800000u;
  return e != 0x7f800000u && (e != 0u || (b << 1) == 0u);
}

// The double's high and low 32-bit words for a float accepted above.
VSR_DF_FN void vsr_f32_widen(uint32_t b, uint32_t* hi_word, uint32_t* lo_word) {
  const uint32_t sign = b & 0x80000000u;
  const int zero = (b << 1) == 0u;
  *hi_word = zero ? sign : (sign | (((b & 0x7fffffffu) >> 3) + 0x38000000u));
  *lo_word = zero ? 0u : b << 29;
}

#endif
