// Checks the integer-pipe binary64 routines of fp64emu.cuh against the host
// CPU's IEEE-754 arithmetic (SSE2, round to nearest even, no FTZ/DAZ), bit for
// bit (any NaN matches any NaN).  Usage: fp64emu_check <cases> <seed>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>

#include "fp64emu.cuh"

static uint64_t bits(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }
static double dbl(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }
static bool same(uint64_t got, double want) {
  if (std::isnan(want)) return gxe_isnan(got);
  return got == bits(want);
}

static int64_t ref_d2ll(double x) {
  if (x != x) return 0;
  if (x >= 9223372036854775808.0) return std::numeric_limits<int64_t>::max();
  if (x < -9223372036854775808.0) return std::numeric_limits<int64_t>::min();
  return (int64_t)x;
}

struct Gen {
  std::mt19937_64 rng;
  explicit Gen(uint64_t s) : rng(s) {}
  uint64_t u64() { return rng(); }
  // a double drawn from a mix of strategies: uniform bits, moderate values,
  // subnormals, extreme exponents, integers, specials
  double any() {
    switch (rng() % 10) {
      case 0: return dbl(rng());
      case 1: return dbl((rng() & 0x800FFFFFFFFFFFFFull));                       // subnormal / zero
      case 2: return dbl((rng() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(1 + rng() % 60) << 52));  // tiny normal
      case 3: return dbl((rng() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(2046 - rng() % 60) << 52));  // huge
      case 4: { static const double S[] = {0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, 10.0, 1000.0, 0.5,
                                           1.7976931348623123e+308, 2.2250738585072014e-308, 4.9e-324};
                return S[rng() % (sizeof S / sizeof S[0])]; }
      case 5: return (double)(int64_t)(rng() >> (rng() % 64));
      case 6: return dbl((rng() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(1023 + (int)(rng() % 64) - 32) << 52));
      case 7: return dbl(0x3FF0000000000000ull | (rng() & 0xFFFFFull));        // near 1, short mantissa
      default: { std::normal_distribution<double> n(0.0, 1e3); return n(rng); }
    }
  }
};

int main(int argc, char** argv) {
  const long long cases = argc > 1 ? atoll(argv[1]) : 1000000;
  Gen g(argc > 2 ? strtoull(argv[2], nullptr, 10) : 1);
  long long bad = 0;
  for (long long i = 0; i < cases; i++) {
    const double a = g.any(), b = g.any();
    const uint64_t q = gxe_div(bits(a), bits(b));
    if (!same(q, a / b)) {
      if (bad++ < 10) printf("div %.17g / %.17g: got %016llx want %016llx\n", a, b, (unsigned long long)q,
                             (unsigned long long)bits(a / b));
    }
    // constant-divisor form: reciprocal computed ahead for a normal finite divisor
    const int eb = (int)((bits(b) >> 52) & 0x7FF);
    if (eb >= 1 && eb <= 2046) {
      const uint64_t r = gxe_recip_fixed((bits(b) & GXE_FRAC) | GXE_HIDDEN);
      const uint64_t q2 = gxe_div_r(bits(a), bits(b), r);
      // the FMA-unit form (Markstein's correction step inside its window)
      int lo = 0, hi = 0;
      gxe_div_c_window(eb, &lo, &hi);
      const uint64_t q3 = gxe_div_c(bits(a), bits(b), r, bits(1.0 / b), lo, hi);
      if (!same(q3, a / b)) {
        if (bad++ < 10) printf("div_c %.17g / %.17g: got %016llx want %016llx\n", a, b, (unsigned long long)q3,
                               (unsigned long long)bits(a / b));
      }
      if (!same(q2, a / b)) {
        if (bad++ < 10) printf("div_r %.17g / %.17g: got %016llx want %016llx\n", a, b, (unsigned long long)q2,
                               (unsigned long long)bits(a / b));
      }
    }
    if (!same(gxe_add(bits(a), bits(b)), a + b) || !same(gxe_sub(bits(a), bits(b)), a - b)) {
      if (bad++ < 10) printf("add/sub %.17g %.17g\n", a, b);
    }
    if (!same(gxe_mul(bits(a), bits(b)), a * b)) {
      if (bad++ < 10) printf("mul %.17g * %.17g: got %016llx want %016llx\n", a, b,
                             (unsigned long long)gxe_mul(bits(a), bits(b)), (unsigned long long)bits(a * b));
    }
    // close magnitudes exercise cancellation
    const double c = a * (1.0 + (double)(g.u64() % 1000) * 1e-16);
    if (!same(gxe_sub(bits(a), bits(c)), a - c) || !same(gxe_add(bits(a), bits(-c)), a + -c)) {
      if (bad++ < 10) printf("cancel %.17g %.17g\n", a, c);
    }
    const int64_t iv = (int64_t)g.u64() >> (g.u64() % 64);
    if (gxe_i2d(iv) != bits((double)iv)) {
      if (bad++ < 10) printf("i2d %lld\n", (long long)iv);
    }
    const uint32_t fb = (uint32_t)g.u64();
    float fv;
    std::memcpy(&fv, &fb, 4);
    if (!same(gxe_f2d(fb), (double)fv)) {
      if (bad++ < 10) printf("f2d %08x\n", fb);
    }
    if (!same(gxe_floor(bits(a)), std::floor(a)) || !same(gxe_ceil(bits(a)), std::ceil(a))) {
      if (bad++ < 10) printf("floor/ceil %.17g\n", a);
    }
    if (gxe_lt(bits(a), bits(b)) != (a < b) || gxe_le(bits(a), bits(b)) != (a <= b) ||
        gxe_eq(bits(a), bits(b)) != (a == b) || gxe_nz(bits(a)) != (a != 0.0)) {
      if (bad++ < 10) printf("cmp %.17g %.17g\n", a, b);
    }
    if (gxe_d2ll(bits(a)) != ref_d2ll(a)) {
      if (bad++ < 10) printf("d2ll %.17g\n", a);
    }
  }
  // the FMA-unit constant division against literal divisors of the kind plans
  // use, with dividends spread over the whole exponent window and its edges
  {
    static const double D[] = {100.0, 10.0, 1000.0, 3.0, 7.0, 0.1, 1e-3, 1.5, 86400.0, 1e9, 1e-300, 1e300,
                               0.3333333333333333, 1.0000000000000002, 1.9999999999999998, 255.0, -100.0, 6.0};
    for (double b : D) {
      const uint64_t bb = bits(b);
      const int eb = (int)((bb >> 52) & 0x7FF);
      const uint64_t r = gxe_recip_fixed((bb & GXE_FRAC) | GXE_HIDDEN);
      const uint64_t y = bits(1.0 / b);
      int lo = 0, hi = 0;
      gxe_div_c_window(eb, &lo, &hi);
      for (long long i = 0; i < cases; i++) {
        uint64_t ab;
        switch (g.u64() % 4) {
          case 0: ab = bits(g.any()); break;
          case 1: ab = (g.u64() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(lo + (int)(g.u64() % (hi - lo + 1))) << 52); break;
          case 2: ab = (g.u64() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(1023 + (int)(g.u64() % 80) - 40) << 52); break;
          default: ab = bits((double)(int64_t)(g.u64() >> (g.u64() % 64)) / (double)(1 + g.u64() % 1000)); break;
        }
        const double a = dbl(ab);
        const uint64_t q = gxe_div_c(ab, bb, r, y, lo, hi);
        if (!same(q, a / b)) {
          if (bad++ < 10) printf("div_c %.17g / %.17g: got %016llx want %016llx\n", a, b, (unsigned long long)q,
                                 (unsigned long long)bits(a / b));
        }
      }
    }
  }
  // integer divisors through the reciprocal table (and past its end)
  {
    const int n = 256;
    static gxe_u64 rcp[256];
    for (int i = 0; i < n; i++) rcp[i] = bits(1.0 / (double)(i + 1));
    for (long long i = 0; i < cases * 4; i++) {
      const int64_t k = (int64_t)(g.u64() % 600) - 300;  // -300 .. 299, zero and beyond the table included
      uint64_t ab;
      switch (g.u64() % 3) {
        case 0: ab = bits(g.any()); break;
        case 1: ab = (g.u64() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(300 + (int)(g.u64() % 1420)) << 52); break;
        default: ab = bits((double)(int64_t)(g.u64() >> (g.u64() % 64)) * (double)(1 + g.u64() % 1000)); break;
      }
      const double a = dbl(ab), b = (double)k;
      const uint64_t q = gxe_div_small(ab, k, rcp, n);
      if (!same(q, a / b)) {
        if (bad++ < 10) printf("div_small %.17g / %lld: got %016llx want %016llx\n", a, (long long)k,
                               (unsigned long long)q, (unsigned long long)bits(a / b));
      }
    }
  }
  printf("cases=%lld mismatches=%lld\n", cases, bad);
  return bad ? 1 : 0;
}
