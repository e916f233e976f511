// fp64emu.cuh -- IEEE-754 binary64 operations computed on the integer and
// FP32 pipes, bit-identical to the hardware's round-to-nearest-even results.
//
// GB300 executes FP64 at about 1/57 of its FP32 rate (measured: DFMA 0.6 Top/s,
// DDIV 59 Gop/s vs IMAD 19 Top/s), so a plan that divides or compares doubles
// per row is bound by the FP64 pipe long before HBM.  These routines give the
// exact same bits as the native instructions using 32/64-bit integer
// arithmetic: division by a float-seeded fixed-point Newton reciprocal with an
// exact integer remainder correction (Muller et al., "Handbook of
// Floating-Point Arithmetic", ch. 9: reciprocal iteration + remainder-based
// correction), conversions and comparisons by bit manipulation.
//
// The header compiles for the host too (g++), where the tests check it against
// the CPU's IEEE arithmetic.
#pragma once

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define GXE_FN __device__ __forceinline__
#define GXE_ON_DEVICE 1
#else
#include <cstdint>
#include <cstring>
#define GXE_FN static inline
#define GXE_ON_DEVICE 0
#endif

typedef unsigned long long gxe_u64;
typedef long long gxe_i64;

#define GXE_SIGN 0x8000000000000000ull
#define GXE_FRAC 0x000FFFFFFFFFFFFFull
#define GXE_HIDDEN 0x0010000000000000ull
#define GXE_INF 0x7FF0000000000000ull
#define GXE_QNAN 0x7FF8000000000000ull

GXE_FN gxe_u64 gxe_umulhi(gxe_u64 a, gxe_u64 b) {
#if GXE_ON_DEVICE
  return __umul64hi(a, b);
#else
  return (gxe_u64)(((unsigned __int128)a * b) >> 64);
#endif
}

GXE_FN int gxe_clz(gxe_u64 x) {
#if GXE_ON_DEVICE
  return __clzll((gxe_i64)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

GXE_FN float gxe_rcp_approx(float x) {
#if GXE_ON_DEVICE
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#elif defined(GXE_TEST_PERTURB_RCP)
  // host test mode: a seed up to +-2 ulp off (worse than rcp.approx's 1 ulp)
  float r = 1.0f / x;
  unsigned u;
  std::memcpy(&u, &r, 4);
  unsigned xb;
  std::memcpy(&xb, &x, 4);
  u += (unsigned)((xb * 2654435761u) >> 29) % 5u - 2u;
  std::memcpy(&r, &u, 4);
  return r;
#else
  return 1.0f / x;
#endif
}

GXE_FN unsigned gxe_f2u(float f) {
#if GXE_ON_DEVICE
  return __float_as_uint(f);
#else
  unsigned u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}

GXE_FN float gxe_u2f(unsigned u) {
#if GXE_ON_DEVICE
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}

GXE_FN bool gxe_isnan_(gxe_u64 a) { return (a & ~GXE_SIGN) > GXE_INF; }

// Rounds Q * 2^(e - 54) (Q in [2^54, 2^55), `rem` nonzero if inexact beyond Q)
// to binary64 with round-to-nearest-even; handles overflow and subnormals.
GXE_FN gxe_u64 gxe_round_pack(gxe_u64 sign, int e, gxe_u64 q, bool rem) {
  int eb = e + 1023;
  if (eb >= 1) {
    gxe_u64 m = q >> 2;
    const bool round = (q >> 1) & 1u;
    const bool sticky = (q & 1u) || rem;
    m += (round && (sticky || (m & 1u))) ? 1u : 0u;
    if (m == (1ull << 53)) {
      m >>= 1;
      eb++;
    }
    if (eb >= 2047) return sign | GXE_INF;
    return sign | ((gxe_u64)eb << 52) | (m & GXE_FRAC);
  }
  const int sh = 3 - eb;  // >= 3
  if (sh > 55) return sign;
  gxe_u64 m = q >> sh;
  const bool round = (q >> (sh - 1)) & 1u;
  const bool sticky = (q & ((1ull << (sh - 1)) - 1u)) != 0 || rem;
  m += (round && (sticky || (m & 1u))) ? 1u : 0u;
  return sign | m;  // m == 2^52 encodes the smallest normal
}

// r ~ 2^116 / mb for a significand mb in [2^52, 2^53): an FP32 reciprocal of
// mb's top 24 bits refined by two Newton steps in 64-bit fixed point
// (r += r * (2^116 - mb*r) / 2^116).  Any r within a few units of the exact
// value serves gxe_div_finish, whose remainder correction absorbs the error.
GXE_FN gxe_u64 gxe_recip_fixed(gxe_u64 mb) {
  const unsigned d24 = (unsigned)(mb >> 29);                      // [2^23, 2^24)
  const float df = gxe_u2f((150u << 23) | (d24 & 0x7FFFFFu));    // == (float)d24
  const unsigned rb = gxe_f2u(gxe_rcp_approx(df));                // ~1/d24 in (2^-24, 2^-23]
  const int rexp = (int)((rb >> 23) & 0xFF) - 127;                // -24 or -23
  gxe_u64 r = (gxe_u64)((rb & 0x7FFFFFu) | 0x800000u) << (40 + (rexp + 24));  // * 2^(87+rexp-23)
  if (rexp >= -23) r = ~0ull;                                     // 1/d24 == 2^-23 -> clamp 2^64
#if GXE_ON_DEVICE
#pragma unroll
#endif
  for (int it = 0; it < 2; it++) {
    const gxe_u64 ph = gxe_umulhi(mb, r), pl = mb * r;
    const gxe_u64 t = (ph << 12) | (pl >> 52);   // (mb*r) >> 52, modulo 2^64
    const gxe_i64 err = -(gxe_i64)t;             // (2^116 - mb*r) / 2^52
    const gxe_u64 corr = gxe_umulhi(r, (gxe_u64)(err < 0 ? -err : err));
    r = err < 0 ? r - corr : r + corr;
  }
  return r;
}

// Quotient of significands ma, mb in [2^52, 2^53) with r = gxe_recip_fixed(mb):
// Q0 ~ floor(ma * 2^54 / mb) = (ma * r) >> 62, exact remainder correction, then
// rounding of the result with exponent e (before the ma < mb adjustment).
GXE_FN gxe_u64 gxe_div_finish(gxe_u64 sign, int e, gxe_u64 ma, gxe_u64 mb, gxe_u64 r) {
  if (ma < mb) {
    ma <<= 1;
    e -= 1;
  }
  gxe_u64 q = (gxe_umulhi(ma, r) << 2) | ((ma * r) >> 62);
  gxe_i64 rem = (gxe_i64)((ma << 54) - q * mb);  // exact: |rem| < 2^55
  if (rem < 0) { q--; rem += (gxe_i64)mb; }
  if (rem < 0) { q--; rem += (gxe_i64)mb; }
  if (rem >= (gxe_i64)mb) { q++; rem -= (gxe_i64)mb; }
  if (rem >= (gxe_i64)mb) { q++; rem -= (gxe_i64)mb; }
  return gxe_round_pack(sign, e, q, rem != 0);
}

// x / y, correctly rounded (round to nearest even), as bits.
GXE_FN gxe_u64 gxe_div(gxe_u64 a, gxe_u64 b) {
  const gxe_u64 sign = (a ^ b) & GXE_SIGN;
  int ea = (int)((a >> 52) & 0x7FF), eb = (int)((b >> 52) & 0x7FF);
  gxe_u64 fa = a & GXE_FRAC, fb = b & GXE_FRAC;
  if ((unsigned)(ea - 1) >= 2046u || (unsigned)(eb - 1) >= 2046u) {
    const bool nan_a = ea == 0x7FF && fa != 0, nan_b = eb == 0x7FF && fb != 0;
    if (nan_a || nan_b) return GXE_QNAN | (nan_a ? fa : fb) | (nan_a ? (a & GXE_SIGN) : (b & GXE_SIGN));
    const bool inf_a = ea == 0x7FF, inf_b = eb == 0x7FF;
    const bool zero_a = ea == 0 && fa == 0, zero_b = eb == 0 && fb == 0;
    if ((inf_a && inf_b) || (zero_a && zero_b)) return GXE_QNAN | GXE_SIGN;
    if (inf_a || zero_b) return sign | GXE_INF;
    if (inf_b || zero_a) return sign;
    if (ea == 0) {
      const int lz = gxe_clz(fa) - 11;
      fa <<= lz;
      ea = 1 - lz;
    }
    if (eb == 0) {
      const int lz = gxe_clz(fb) - 11;
      fb <<= lz;
      eb = 1 - lz;
    }
  }
  const gxe_u64 mb = fb | GXE_HIDDEN;
  return gxe_div_finish(sign, ea - eb, fa | GXE_HIDDEN, mb, gxe_recip_fixed(mb));
}

// x / y for a constant y that is normal and finite, with r =
// gxe_recip_fixed(y's significand) computed ahead: same bits as gxe_div(x, y).
GXE_FN gxe_u64 gxe_div_r(gxe_u64 a, gxe_u64 b, gxe_u64 r) {
  const gxe_u64 sign = (a ^ b) & GXE_SIGN;
  int ea = (int)((a >> 52) & 0x7FF);
  const int eb = (int)((b >> 52) & 0x7FF);
  gxe_u64 fa = a & GXE_FRAC;
  if ((unsigned)(ea - 1) >= 2046u) {
    if (ea == 0x7FF) return fa != 0 ? (GXE_QNAN | fa | (a & GXE_SIGN)) : (sign | GXE_INF);
    if (fa == 0) return sign;
    const int lz = gxe_clz(fa) - 11;
    fa <<= lz;
    ea = 1 - lz;
  }
  return gxe_div_finish(sign, ea - eb, fa | GXE_HIDDEN, (b & GXE_FRAC) | GXE_HIDDEN, r);
}

// x / b for a constant b (normal, finite) on the FMA unit, with y = RN(1/b)
// and bd = b: Markstein's correction step (Muller et al., "Handbook of
// Floating-Point Arithmetic", the theorem on the final correction of a
// quotient): q = RN(x * y) is within an ulp of x / b, so r = x - q * b is
// exact (one FMA), and RN(q + r * y) (one FMA) is the correctly rounded
// quotient, provided nothing underflows or overflows.  So the step is taken
// for x whose exponent field lies in [lo, hi] (chosen with b's exponent so
// that x, the quotient and r stay normal); a zero gives the signed zero;
// every other x (tiny, huge, subnormal, infinite, NaN) goes to gxe_div_r
// with rr = gxe_recip_fixed(b's significand).  Same bits as gxe_div(x, b).
GXE_FN double gxe_fma_(double a, double b, double c) {
#if GXE_ON_DEVICE
  return __fma_rn(a, b, c);
#else
  return __builtin_fma(a, b, c);
#endif
}
GXE_FN double gxe_mul_rn_(double a, double b) {
#if GXE_ON_DEVICE
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
GXE_FN gxe_u64 gxe_div_c(gxe_u64 a, gxe_u64 b, gxe_u64 rr, gxe_u64 ybits, int lo, int hi) {
  if ((a & ~GXE_SIGN) == 0) return (a ^ b) & GXE_SIGN;
  const int ea = (int)((a >> 52) & 0x7FF);
  if (ea < lo || ea > hi) return gxe_div_r(a, b, rr);
  double x, bd, y;
#if GXE_ON_DEVICE
  x = __longlong_as_double((long long)a);
  bd = __longlong_as_double((long long)b);
  y = __longlong_as_double((long long)ybits);
#else
  std::memcpy(&x, &a, 8);
  std::memcpy(&bd, &b, 8);
  std::memcpy(&y, &ybits, 8);
#endif
  const double q = gxe_mul_rn_(x, y);
  const double r = gxe_fma_(-q, bd, x);
  const double z = gxe_fma_(r, y, q);
  gxe_u64 zb;
#if GXE_ON_DEVICE
  zb = (gxe_u64)__double_as_longlong(z);
#else
  std::memcpy(&zb, &z, 8);
#endif
  return zb;
}
// the exponent-field window of gxe_div_c for a divisor whose exponent field is eb
GXE_FN void gxe_div_c_window(int eb, int* lo, int* hi) {
  // x, x / b and the remainder (about 2^-106 |x|) all normal and far from overflow
  *lo = 300 + (eb > 1023 ? eb - 1023 : 0);
  *hi = 1700 + (eb < 1023 ? eb - 1023 : 0);
}

// x + y, correctly rounded, as bits (guard / round / sticky alignment).
GXE_FN gxe_u64 gxe_add(gxe_u64 a, gxe_u64 b) {
  int ea = (int)((a >> 52) & 0x7FF), eb = (int)((b >> 52) & 0x7FF);
  if (ea == 0x7FF || eb == 0x7FF) {
    if (gxe_isnan_(a)) return a | (1ull << 51);
    if (gxe_isnan_(b)) return b | (1ull << 51);
    if (ea == 0x7FF && eb == 0x7FF) return ((a ^ b) & GXE_SIGN) ? (GXE_QNAN | GXE_SIGN) : a;  // inf - inf
    return ea == 0x7FF ? a : b;
  }
  gxe_u64 aa = a & ~GXE_SIGN, bb = b & ~GXE_SIGN;
  if (aa < bb) {  // |a| >= |b|
    gxe_u64 t = a; a = b; b = t;
    t = aa; aa = bb; bb = t;
    int te = ea; ea = eb; eb = te;
  }
  if (bb == 0) return aa == 0 ? (a & b & GXE_SIGN) : a;
  const int xa = ea ? ea : 1, xb = eb ? eb : 1;
  gxe_u64 ma = ((a & GXE_FRAC) | (ea ? GXE_HIDDEN : 0)) << 3;
  gxe_u64 mb = ((b & GXE_FRAC) | (eb ? GXE_HIDDEN : 0)) << 3;
  const int d = xa - xb;
  if (d >= 58) {
    mb = 1;
  } else if (d > 0) {
    const gxe_u64 lost = mb & ((1ull << d) - 1u);
    mb = (mb >> d) | (lost != 0 ? 1u : 0u);
  }
  const gxe_u64 sign = a & GXE_SIGN;
  gxe_u64 s;
  int e = xa;
  if (((a ^ b) & GXE_SIGN) == 0) {
    s = ma + mb;
    if (s >> 56) {
      s = (s >> 1) | (s & 1u);
      e++;
    }
  } else {
    s = ma - mb;
    if (s == 0) return 0;
    int lz = gxe_clz(s) - 8;
    if (lz > 0) {
      if (e - lz < 1) lz = e - 1;
      s <<= lz;
      e -= lz;
    }
  }
  gxe_u64 m = s >> 3;
  const unsigned low = (unsigned)(s & 7u);
  if (low > 4u || (low == 4u && (m & 1u))) m++;
  if (m >> 53) {
    m >>= 1;
    e++;
  }
  if (e >= 2047) return sign | GXE_INF;
  if (!(m & GXE_HIDDEN)) return sign | m;  // subnormal
  return sign | ((gxe_u64)e << 52) | (m & GXE_FRAC);
}

GXE_FN gxe_u64 gxe_sub(gxe_u64 a, gxe_u64 b) { return gxe_add(a, b ^ GXE_SIGN); }

// x * y, correctly rounded, as bits (106-bit product).
GXE_FN gxe_u64 gxe_mul(gxe_u64 a, gxe_u64 b) {
  const gxe_u64 sign = (a ^ b) & GXE_SIGN;
  int ea = (int)((a >> 52) & 0x7FF), eb = (int)((b >> 52) & 0x7FF);
  gxe_u64 fa = a & GXE_FRAC, fb = b & GXE_FRAC;
  if ((unsigned)(ea - 1) >= 2046u || (unsigned)(eb - 1) >= 2046u) {
    const bool nan_a = ea == 0x7FF && fa != 0, nan_b = eb == 0x7FF && fb != 0;
    if (nan_a) return a | (1ull << 51);
    if (nan_b) return b | (1ull << 51);
    const bool inf_a = ea == 0x7FF, inf_b = eb == 0x7FF;
    const bool zero_a = ea == 0 && fa == 0, zero_b = eb == 0 && fb == 0;
    if ((inf_a && zero_b) || (inf_b && zero_a)) return GXE_QNAN | GXE_SIGN;
    if (inf_a || inf_b) return sign | GXE_INF;
    if (zero_a || zero_b) return sign;
    if (ea == 0) {
      const int lz = gxe_clz(fa) - 11;
      fa <<= lz;
      ea = 1 - lz;
    }
    if (eb == 0) {
      const int lz = gxe_clz(fb) - 11;
      fb <<= lz;
      eb = 1 - lz;
    }
  }
  const gxe_u64 ma = fa | GXE_HIDDEN, mb = fb | GXE_HIDDEN;
  const gxe_u64 hi = gxe_umulhi(ma, mb), lo = ma * mb;  // product in [2^104, 2^106)
  if (hi >> 41) {  // >= 2^105
    return gxe_round_pack(sign, ea + eb - 2045, (hi << 13) | (lo >> 51), (lo & ((1ull << 51) - 1u)) != 0);
  }
  return gxe_round_pack(sign, ea + eb - 2046, (hi << 14) | (lo >> 50), (lo & ((1ull << 50) - 1u)) != 0);
}

// (double)(int64) with round-to-nearest-even, as bits.
GXE_FN gxe_u64 gxe_i2d(gxe_i64 v) {
  if (v == 0) return 0;
  const gxe_u64 sign = v < 0 ? GXE_SIGN : 0;
  gxe_u64 u = v < 0 ? 0ull - (gxe_u64)v : (gxe_u64)v;
  const int lz = gxe_clz(u);
  const int msb = 63 - lz;                     // exponent
  if (msb <= 52) return sign | ((gxe_u64)(msb + 1023) << 52) | ((u << (52 - msb)) & GXE_FRAC);
  const int sh = msb - 52;                     // 1..11
  gxe_u64 m = u >> sh;
  const bool round = (u >> (sh - 1)) & 1u;
  const bool sticky = (u & ((1ull << (sh - 1)) - 1u)) != 0;
  m += (round && (sticky || (m & 1u))) ? 1u : 0u;
  int eb = msb + 1023;
  if (m == (1ull << 53)) {
    m >>= 1;
    eb++;
  }
  return sign | ((gxe_u64)eb << 52) | (m & GXE_FRAC);
}

// (double)(float) (exact), as bits.
GXE_FN gxe_u64 gxe_f2d(unsigned f) {
  const gxe_u64 sign = (gxe_u64)(f >> 31) << 63;
  const unsigned ef = (f >> 23) & 0xFF, mf = f & 0x7FFFFFu;
  if (ef == 0xFF) return sign | GXE_INF | ((gxe_u64)mf << 29) | (mf ? (1ull << 51) : 0);
  if (ef == 0) {
    if (mf == 0) return sign;
    const int lz = gxe_clz((gxe_u64)mf) - 40;     // bring the leading 1 to bit 23
    return sign | ((gxe_u64)(1 - lz - 127 + 1023) << 52) | (((gxe_u64)(mf << lz) & 0x7FFFFFu) << 29);
  }
  return sign | ((gxe_u64)(ef - 127 + 1023) << 52) | ((gxe_u64)mf << 29);
}

// x / k for an integer divisor k: when 1 <= |k| <= n, Markstein's
// correction step (as gxe_div_c) on the FMA unit with y = RN(1/|k|) read from
// the table rcp (rcp[i] = RN(1 / (i + 1)) as bits) and the quotient's sign
// flipped for a negative k (x / -k = -(x / k) exactly); a zero x gives the
// signed zero.  Other k, and x outside the exponent window, take gxe_div.
// Same bits as gxe_div(x, (double)k).
GXE_FN gxe_u64 gxe_div_small(gxe_u64 a, gxe_i64 k, const gxe_u64* rcp, int n) {
  const gxe_u64 ak = k < 0 ? 0ull - (gxe_u64)k : (gxe_u64)k;
  const int ea = (int)((a >> 52) & 0x7FF);
  const bool zero = (a & ~GXE_SIGN) == 0;
  if (ak - 1ull >= (gxe_u64)n || (!zero && (ea < 310 || ea > 1700))) return gxe_div(a, gxe_i2d(k));
  gxe_u64 q;
  if (zero) {
    q = a & GXE_SIGN;
  } else {
#if GXE_ON_DEVICE
    const double y = __longlong_as_double((long long)__ldg(rcp + (ak - 1ull)));
    const double x = __longlong_as_double((long long)a);
    const double b = (double)(long long)ak;  // exact: |k| <= n
#else
    double y, x;
    std::memcpy(&y, rcp + (ak - 1ull), 8);
    std::memcpy(&x, &a, 8);
    const double b = (double)(long long)ak;
#endif
    const double q0 = gxe_mul_rn_(x, y);
    const double r = gxe_fma_(-q0, b, x);
    const double z = gxe_fma_(r, y, q0);
#if GXE_ON_DEVICE
    q = (gxe_u64)__double_as_longlong(z);
#else
    std::memcpy(&q, &z, 8);
#endif
  }
  return k < 0 ? q ^ GXE_SIGN : q;
}

GXE_FN bool gxe_isnan(gxe_u64 a) { return (a & ~GXE_SIGN) > GXE_INF; }

// total order key for non-NaN values with -0 == +0
GXE_FN gxe_u64 gxe_key(gxe_u64 a) {
  if ((a << 1) == 0) a = 0;
  return (a & GXE_SIGN) ? ~a : (a | GXE_SIGN);
}
GXE_FN bool gxe_lt(gxe_u64 a, gxe_u64 b) { return !gxe_isnan(a) && !gxe_isnan(b) && gxe_key(a) < gxe_key(b); }
GXE_FN bool gxe_le(gxe_u64 a, gxe_u64 b) { return !gxe_isnan(a) && !gxe_isnan(b) && gxe_key(a) <= gxe_key(b); }
GXE_FN bool gxe_eq(gxe_u64 a, gxe_u64 b) { return !gxe_isnan(a) && !gxe_isnan(b) && gxe_key(a) == gxe_key(b); }
GXE_FN bool gxe_nz(gxe_u64 a) { return (a << 1) != 0; }  // != 0.0 (NaN counts as nonzero)

// floor / ceil (exact), as bits
GXE_FN gxe_u64 gxe_floor(gxe_u64 a) {
  const int e = (int)((a >> 52) & 0x7FF) - 1023;
  if (e >= 52) return gxe_isnan(a) ? (a | (1ull << 51)) : a;  // integral, inf, nan
  if (e < 0) {
    if ((a << 1) == 0) return a;                                 // +-0
    return (a & GXE_SIGN) ? 0xBFF0000000000000ull : 0;           // -1 or +0
  }
  const gxe_u64 fmask = GXE_FRAC >> e;
  if ((a & fmask) == 0) return a;
  if (a & GXE_SIGN) a += (GXE_HIDDEN >> e);  // round toward -inf in magnitude
  return a & ~fmask;
}
GXE_FN gxe_u64 gxe_ceil(gxe_u64 a) {
  const int e = (int)((a >> 52) & 0x7FF) - 1023;
  if (e >= 52) return gxe_isnan(a) ? (a | (1ull << 51)) : a;
  if (e < 0) {
    if ((a << 1) == 0) return a;
    return (a & GXE_SIGN) ? GXE_SIGN : 0x3FF0000000000000ull;    // -0 or +1
  }
  const gxe_u64 fmask = GXE_FRAC >> e;
  if ((a & fmask) == 0) return a;
  if (!(a & GXE_SIGN)) a += (GXE_HIDDEN >> e);
  return a & ~fmask;
}

// static_cast<int64_t>(double) as the GPU does it: truncate, saturate, NaN -> 0
GXE_FN gxe_i64 gxe_d2ll(gxe_u64 a) {
  if (gxe_isnan(a)) return 0;
  const int e = (int)((a >> 52) & 0x7FF) - 1023;
  const bool neg = (a & GXE_SIGN) != 0;
  if (e < 0) return 0;
  if (e >= 63) return neg ? (gxe_i64)GXE_SIGN : 0x7FFFFFFFFFFFFFFFll;
  const gxe_u64 m = (a & GXE_FRAC) | GXE_HIDDEN;
  const gxe_u64 mag = e >= 52 ? (m << (e - 52)) : (m >> (52 - e));
  return neg ? -(gxe_i64)mag : (gxe_i64)mag;
}
