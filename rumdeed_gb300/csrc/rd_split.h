// rd_split.h -- FP64 results formed from the bits with integer operations,
// bit for bit the FP64 forms they replace (GB300 runs FP64, and the
// conversions between double and float, at a small fraction of its FP32 and
// integer rates):
//  * rd_split_exact: the FP32 (hi, lo) split of a double,
//      hi = (float)v;  lo = (float)(v - (double)hi);
//    four FP64-pipe operations per coordinate in the FP64 form, here one
//    int-to-float conversion, one FP32 multiply and integer work;
//  * rd_repeat_sum: e added M times in FP64, without M dependent additions.
// Plain C++ as well, so that a host test can check both against the FP64
// forms (tests/test_split.py).
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

RD_HD double rd_float64_of_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
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

// The sum 0 + e + e + ... + e (M terms) with every addition rounded to
// nearest even in FP64, as a loop `s += e` forms it, without the M dependent
// additions (one thread's FP64 latency on GB300 makes a few thousand of them
// cost tens of microseconds).  While the partial sum s stays in one binade
// [2^E, 2^(E+1)) it is a multiple of u = 2^(E-52), and s + e rounds to
// s + A u or s + (A + 1) u (e = (A + R) u, 0 <= R < 1) the same way every
// step, save a tie (R = 1/2), which rounds to an even multiple once and then
// keeps the increment even; the step that leaves the binade is taken on its
// own with the next binade's ulp.  Since e <= s after the first term, a step
// crosses at most one binade.  Integer arithmetic in units of u; for e = 0,
// a non-normal e, or sums near the top of the range, the loop itself.
RD_HD double rd_repeat_sum(double e, int M) {
  if (M <= 0) return 0.0;
  const uint64_t eb = rd_double_bits(e);
  const int Ee = (int)((eb >> 52) & 0x7ff);
  if ((eb >> 63) != 0 || Ee == 0 || Ee >= 0x7ff - 16 || M < 4) {
    double s = 0.0;
    for (int k = 0; k < M; ++k) s += e;
    return s;
  }
  const uint64_t me = (eb & 0xfffffffffffffull) | (1ull << 52);   // e = me 2^(Ee - 1075)
  const uint64_t top = 1ull << 53;
  int E = Ee;          // binade of s
  uint64_t S = me;     // s in units of u = 2^(E - 1075): s = e after the first term
  int left = M - 1;
  while (left > 0) {
    const int sh = E - Ee;                 // 0 .. 14 (s <= M e)
    const uint64_t A = me >> sh;           // e / u, integer part
    const uint64_t rem = me & ((1ull << sh) - 1);
    const uint64_t half = sh > 0 ? 1ull << (sh - 1) : 0;
    // one step, exactly: x = S + A + R
    auto step_rounded = [&](uint64_t s0, bool* crossed) -> uint64_t {
      uint64_t q = s0 + A;   // x = q + R
      if (q >= top) {        // leaves the binade: round x / 2 to an integer (units of 2u)
        *crossed = true;
        const uint64_t q2 = q >> 1;
        // x / 2 = q2 + ((q & 1) + R) / 2; R in units of 2^-sh
        const uint64_t frac = ((q & 1ull) << sh) | rem;    // numerator over 2^(sh + 1)
        const uint64_t h2 = 1ull << sh;                    // one half
        return q2 + ((frac > h2 || (frac == h2 && (q2 & 1ull))) ? 1 : 0);
      }
      *crossed = false;
      if (sh == 0) return q;
      if (rem > half || (rem == half && (q & 1ull))) ++q;
      return q;
    };
    bool crossed = false;
    if (sh > 0 && rem == half) {   // a tie: one step by itself, then the increment is even
      S = step_rounded(S, &crossed);
      --left;
      if (crossed) { ++E; continue; }
      if (left == 0) break;
    }
    const uint64_t inc = A + ((sh > 0 && (rem > half || (rem == half && (A & 1ull)))) ? 1 : 0);
    // steps that stay in the binade: S_k + A + R < 2^53, i.e. S_k <= 2^53 - A - 1
    if (inc > 0 && S + A + 1 <= top) {
      const uint64_t room = (top - A - 1 - S) / inc + 1;
      const uint64_t k = room < (uint64_t)left ? room : (uint64_t)left;
      S += k * inc;
      left -= (int)k;
      if (left == 0) break;
    }
    S = step_rounded(S, &crossed);   // the step that leaves the binade
    --left;
    if (crossed) ++E;
  }
  // s = S 2^(E - 1075), S in [2^52, 2^53] (2^53 only as a rounded-up crossing)
  if (S == top) { S >>= 1; ++E; }
  return rd_float64_of_bits(((uint64_t)E << 52) | (S & 0xfffffffffffffull));
}
