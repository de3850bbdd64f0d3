// rd_split.h -- the FP32 (hi, lo) split of a double:
//   hi = (float)v;  lo = (float)(v - (double)hi);
// formed from the double's bits with integer operations, bit for bit the same
// result.  GB300 runs FP64 (and the conversions between double and float) at a
// small fraction of its FP32 and integer rates, and the split takes four such
// operations per coordinate; here it takes one int-to-float conversion, one
// FP32 multiply and integer work.  Plain C++ as well, so that a host test can
// check it against the FP64 form (tests/test_split.py).
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define RD_HD __host__ __device__ __forceinline__
#else
#define RD_HD inline
#endif

RD_HD uint64_t rd_double_bits(double v) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t b;
  memcpy(&b, &v, sizeof b);
  return b;
#endif
}

RD_HD float rd_float_of_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, sizeof f);
  return f;
#endif
}

// v = +-m 2^(E - 1075) with the 53-bit significand m.  hi keeps the high 24
// bits of m rounded to nearest even (a carry out of them raises the float
// exponent, as the conversion does); v - hi = +-(low - up 2^29) 2^(E - 1075)
// is exact, and lo is that integer rounded to float once, times a power of
// two (exact: the result is a normal float).  Outside 2^-63 <= |v| < 2^78,
// and for zero, the FP64 form itself.
RD_HD void rd_split_exact(double v, float* hi, float* lo) {
  const uint64_t b = rd_double_bits(v);
  const int E = (int)((b >> 52) & 0x7ff);
  if (E < 960 || E > 1100) {
    const float h = (float)v;
    *hi = h;
    *lo = (float)(v - (double)h);
    return;
  }
  const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);
  const uint32_t top = (uint32_t)(m >> 29);          // high 24 bits, 2^23 <= top < 2^24
  const uint32_t low = (uint32_t)m & 0x1fffffffu;    // the other 29 bits
  const uint32_t up = (low > 0x10000000u || (low == 0x10000000u && (top & 1u))) ? 1u : 0u;
  const uint32_t sign = (uint32_t)(b >> 63);
  // float exponent field E - 1023 + 127, significand without its leading bit
  const uint32_t hb = ((uint32_t)(E - 896) << 23) + (top - 0x800000u) + up;
  *hi = rd_float_of_bits(hb | (sign << 31));
  int32_t r = (int32_t)low - (int32_t)(up << 29);   // |r| <= 2^28
  if (sign) r = -r;
  *lo = (float)r * rd_float_of_bits((uint32_t)(E - 948) << 23);   // 2^(E - 1075)
}
