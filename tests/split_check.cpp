// Host check of rd_split.h against the FP64 forms it replaces: rd_split_exact
// against  hi = (float)v;  lo = (float)(v - (double)hi);  on random doubles
// over the magnitudes positions take in nm (and far outside), on rounding
// ties and carries, and on the edges of the fast range; rd_repeat_sum against
// the loop  s += e  (M terms) on random magnitudes, tie-prone values and
// small M.  Prints the numbers checked and of bit mismatches.
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include "../rumdeed_gb300/csrc/rd_split.h"

static uint32_t fb(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }
static double from_bits(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }

static long long checked = 0, bad = 0;
static void check(double v) {
  float h1, l1;
  rd_split_exact(v, &h1, &l1);
  const float h0 = (float)v;
  const float l0 = (float)(v - (double)h0);
  ++checked;
  if (fb(h0) != fb(h1) || fb(l0) != fb(l1)) {
    if (bad < 10) printf("mismatch v=%.17g: hi %08x/%08x lo %08x/%08x\n", v, fb(h0), fb(h1), fb(l0), fb(l1));
    ++bad;
  }
}

int main(int argc, char** argv) {
  const long long n = argc > 1 ? atoll(argv[1]) : 2000000;
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  for (long long k = 0; k < n; ++k) {   // log-uniform magnitudes 1e-25 .. 1e30, both signs
    const double mag = std::pow(10.0, -25.0 + 55.0 * u(rng));
    check((k & 1) ? mag : -mag);
  }
  for (long long k = 0; k < n; ++k) {   // positions in nm: uniform in +-2000 nm
    check(-2000.0 + 4000.0 * u(rng));
  }
  for (long long k = 0; k < n / 4; ++k) {   // random bit patterns (all exponents, NaN and inf excluded)
    const uint64_t b = rng();
    if (((b >> 52) & 0x7ff) == 0x7ff) continue;
    check(from_bits(b));
  }
  // ties and carries: low 29 bits at and around half, top all ones, every exponent of the fast range edges
  const uint64_t lows[] = {0, 1, 0x0fffffffull, 0x10000000ull, 0x10000001ull, 0x1fffffffull};
  const uint64_t tops[] = {0, 1, 2, 0x7ffffeull, 0x7fffffull};
  for (int E = 900; E <= 1150; ++E)
    for (uint64_t t : tops)
      for (uint64_t l : lows)
        for (int s = 0; s < 2; ++s) {
          const uint64_t mant = (t << 29) | l;
          check(from_bits(((uint64_t)s << 63) | ((uint64_t)E << 52) | mant));
        }
  check(0.0);
  check(-0.0);
  // rd_repeat_sum against the loop s += e, M terms
  long long rchecked = 0, rbad = 0;
  auto rcheck = [&](double e, int M) {
    double s = 0.0;
    for (int k = 0; k < M; ++k) s += e;
    const double r = rd_repeat_sum(e, M);
    ++rchecked;
    uint64_t a, b;
    memcpy(&a, &s, 8); memcpy(&b, &r, 8);
    if (a != b) {
      if (rbad < 10) printf("repeat-sum mismatch e=%.17g M=%d: %.17g vs %.17g\n", e, M, s, r);
      ++rbad;
    }
  };
  std::uniform_int_distribution<int> um(0, 9000);
  for (long long k = 0; k < n / 200; ++k) {   // escape probabilities and any other magnitude
    const double e = std::pow(10.0, -300.0 + 600.0 * u(rng));
    rcheck(e, um(rng));
  }
  for (long long k = 0; k < n / 200; ++k) {   // low significand bits only: ties and carries in the binades
    const uint64_t mant = (rng() & 0xffffull) | ((rng() & 1) ? (0xfffffull << 32) : 0);
    rcheck(from_bits(((uint64_t)(1023 - 40 + (int)(rng() % 80)) << 52) | mant), um(rng));
  }
  for (int sh = 1; sh <= 14; ++sh)   // exact ties: the bits below a binade's ulp are one half
    for (int M = 2; M <= 9000; M += 997)
      rcheck(from_bits(((uint64_t)1000 << 52) | (1ull << (sh - 1))), M);
  for (int M = 0; M <= 70; ++M) {
    rcheck(1.0, M); rcheck(0.1, M); rcheck(3.0e-13, M); rcheck(0.0, M); rcheck(1.5, M);
  }
  printf("checked %lld mismatches %lld repeat-sums %lld mismatches %lld\n", checked, bad, rchecked, rbad);
  return (bad != 0) || (rbad != 0);
}
