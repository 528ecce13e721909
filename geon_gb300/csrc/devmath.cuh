// Deterministic FP64 sin/cos/tanh for the parity path.
//
// The reference calls the platform libm (Rust f64::sin/cos/tanh -> glibc). A
// GPU cannot call glibc, and CUDA's own functions differ from it by an ulp on
// some inputs, which a 20,000-step RK4 trace (or a double finite difference in
// curvature.rs) amplifies far beyond the 1e-9..1e-10 parity tolerances. So the
// FP64 path evaluates these three functions with one fixed method, restated
// identically in the CPU oracle, and both sides agree bit for bit:
//
//  * sin/cos: Cody & Waite argument reduction by pi/2 (W. J. Cody and W. Waite,
//    "Software Manual for the Elementary Functions", 1980) with a three-part
//    pi/2 and an exact tail term, then the Taylor series of sin (to t^17) and
//    cos (to t^18) by Horner's rule with fused multiply-adds.
//  * tanh and expm1: the published fdlibm method (Sun Microsystems, 1993),
//    which the reference's libm (glibc's dbl-64 tanh and expm1) implements:
//    tanh(x) = sign(x) (1 - 2 / (expm1(2|x|) + 2)) for 1 <= |x| < 22,
//    sign(x) (-m / (m + 2)) with m = expm1(-2|x|) for 2^-55 <= |x| < 1,
//    x (1 + x) below 2^-55 and sign(x) from 22 on; expm1 reduces
//    x = k ln2 + r (r carried as hi - lo with a correction c), evaluates
//    expm1(r) = r - (r e - z), z = r^2 / 2, e = z (R - t) / (6 - r t),
//    t = 3 - R r / 2, with the published minimax R(z) = 1 + Q1 z + ... + Q5 z^5,
//    and rebuilds 2^k (1 + expm1(r)) - 1 in a form chosen per range of k.
//    glibc groups R as (1 + Q1 z) + z^2 (Q2 + Q3 z) + z^4 (Q4 + Q5 z) and its
//    compiler fuses the multiply-adds written as fma() below; with exactly
//    these fusions tanh equals glibc 2.39's bit for bit (5e7 random arguments
//    compared on x86-64; the curvature outputs, which call tanh 62 times per
//    grid point, are bit-identical on aarch64 too).
//
// sin/cos constants are the doubles nearest pi/2 (three parts), 2/pi and
// +-1/n!, produced by gen_math_constants.py in this directory; the expm1
// constants are the published ones (ln 2 split so that k * EX_LN2_HI is exact).
// This file must be compiled without mul+add contraction (--fmad=false); the
// fma() calls below are the only fused operations.
//
// The expm1/tanh method, its range thresholds and its constants follow fdlibm,
// whose notice is kept here as its licence asks:
//   Copyright (C) 1993 by Sun Microsystems, Inc. All rights reserved.
//   Developed at SunSoft, a Sun Microsystems, Inc. business.
//   Permission to use, copy, modify, and distribute this
//   software is freely granted, provided that this notice
//   is preserved.
#pragma once

namespace geon {
namespace dm {

constexpr double PIO2_1 = 0x1.921fb54442d18p+0;
constexpr double PIO2_2 = 0x1.1a62633145c07p-54;
constexpr double PIO2_3 = -0x1.f1976b7ed8fbcp-110;
constexpr double TWO_OVER_PI = 0x1.45f306dc9c883p-1;
constexpr double S3 = -0x1.5555555555555p-3;
constexpr double S5 = 0x1.1111111111111p-7;
constexpr double S7 = -0x1.a01a01a01a01ap-13;
constexpr double S9 = 0x1.71de3a556c734p-19;
constexpr double S11 = -0x1.ae64567f544e4p-26;
constexpr double S13 = 0x1.6124613a86d09p-33;
constexpr double S15 = -0x1.ae7f3e733b81fp-41;
constexpr double S17 = 0x1.952c77030ad4ap-49;
constexpr double C4 = 0x1.5555555555555p-5;
constexpr double C6 = -0x1.6c16c16c16c17p-10;
constexpr double C8 = 0x1.a01a01a01a01ap-16;
constexpr double C10 = -0x1.27e4fb7789f5cp-22;
constexpr double C12 = 0x1.1eed8eff8d898p-29;
constexpr double C14 = -0x1.93974a8c07c9dp-37;
constexpr double C16 = 0x1.ae7f3e733b81fp-45;
constexpr double C18 = -0x1.6827863b97d97p-53;
constexpr double EX_LN2_HI = 0x1.62e42fee00000p-1;
constexpr double EX_LN2_LO = 0x1.a39ef35793c76p-33;
constexpr double EX_INV_LN2 = 0x1.71547652b82fep+0;
constexpr double EX_O_THRESHOLD = 0x1.62e42fefa39efp+9;  // largest x with finite expm1
constexpr double EX_Q1 = -0x1.11111111110f4p-5;
constexpr double EX_Q2 = 0x1.a01a019fe5585p-10;
constexpr double EX_Q3 = -0x1.4ce199eaadbb7p-14;
constexpr double EX_Q4 = 0x1.0cfca86e65239p-18;
constexpr double EX_Q5 = -0x1.afdb76e09c32dp-23;

__device__ __forceinline__ void sincos_det(double x, double* sp, double* cp) {
  if (!isfinite(x)) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    *sp = nan;
    *cp = nan;
    return;
  }
  const double k = rint(x * TWO_OVER_PI);
  const double r1 = fma(-k, PIO2_1, x);
  const double t = fma(-k, PIO2_2, r1);
  const double d = r1 - t;
  const double tl = fma(-k, PIO2_3, fma(-k, PIO2_2, d));
  const double z = t * t;
  double ps = S17;
  ps = fma(ps, z, S15);
  ps = fma(ps, z, S13);
  ps = fma(ps, z, S11);
  ps = fma(ps, z, S9);
  ps = fma(ps, z, S7);
  ps = fma(ps, z, S5);
  ps = fma(ps, z, S3);
  const double tz = t * z;
  const double sv = t + fma(tz, ps, tl * fma(-0.5, z, 1.0));
  double pc = C18;
  pc = fma(pc, z, C16);
  pc = fma(pc, z, C14);
  pc = fma(pc, z, C12);
  pc = fma(pc, z, C10);
  pc = fma(pc, z, C8);
  pc = fma(pc, z, C6);
  pc = fma(pc, z, C4);
  const double hz = 0.5 * z;
  const double wc = 1.0 - hz;
  const double zl = fma(t, t, -z);
  const double cv = wc + (((1.0 - wc) - hz) + (fma(z * z, pc, -0.5 * zl) - tl * t));
  // q = k mod 4 in [0, 4), exactly (the CPU oracle computes k - 4 floor(k / 4)).
  // Below 2^52 the integer conversion is exact and two's-complement & 3 is the
  // mathematical residue; above it k is an even integer and the double formula
  // is exact, and no integer type would hold k.
  int q;
  if (fabs(k) < 0x1p52) {
    q = (int)(__double2ll_rn(k) & 3);
  } else {
    q = (int)(k - 4.0 * floor(k * 0.25));
  }
  double s, c;
  if (q == 0) { s = sv; c = cv; }
  else if (q == 1) { s = cv; c = -sv; }
  else if (q == 2) { s = -sv; c = -cv; }
  else { s = -cv; c = sv; }
  *sp = s;
  *cp = c;
}

__device__ __forceinline__ unsigned hi_word(double x) {
  return (unsigned)((unsigned long long)__double_as_longlong(x) >> 32);
}
__device__ __forceinline__ double from_hi_word(unsigned hi) {
  return __longlong_as_double((long long)((unsigned long long)hi << 32));
}

// e^x - 1 for every double x (the thresholds compare the high word, so each
// range begins at the same bit pattern as in the published method).
__device__ __forceinline__ double expm1_det(double x) {
  const unsigned hxs = hi_word(x);
  const bool neg = (hxs >> 31) != 0;
  const unsigned hx = hxs & 0x7fffffffu;
  if (hx >= 0x4043687Au) {                  // |x| >= 56 ln 2
    if (hx >= 0x40862E42u) {                // |x| >= 709.78
      if (hx >= 0x7ff00000u) return isnan(x) ? x + x : (neg ? -1.0 : x);
      if (x > EX_O_THRESHOLD) return INFINITY;
    }
    if (neg) return -1.0;                   // e^x below half an ulp of 1
  }
  int k = 0;
  double c = 0.0;
  if (hx > 0x3fd62e42u) {                   // |x| > ln2 / 2: reduce
    double hi, lo;
    if (hx < 0x3FF0A2B2u) {                 // |x| < 3 ln2 / 2: k = +-1
      k = neg ? -1 : 1;
      hi = neg ? x + EX_LN2_HI : x - EX_LN2_HI;
      lo = neg ? -EX_LN2_LO : EX_LN2_LO;
    } else {
      k = (int)fma(EX_INV_LN2, x, neg ? -0.5 : 0.5);
      const double tk = (double)k;
      hi = fma(-tk, EX_LN2_HI, x);          // tk * EX_LN2_HI is exact
      lo = tk * EX_LN2_LO;
    }
    x = hi - lo;
    c = (hi - x) - lo;
  } else if (hx < 0x3c900000u) {            // |x| < 2^-54
    return x;
  }
  const double hfx = 0.5 * x, z = x * hfx;
  const double z2 = z * z, z4 = z2 * z2;
  const double R = fma(z4, fma(z, EX_Q5, EX_Q4), fma(z2, fma(z, EX_Q3, EX_Q2), fma(z, EX_Q1, 1.0)));
  const double t = fma(-R, hfx, 3.0);
  double e = z * ((R - t) / fma(-x, t, 6.0));
  if (k == 0) return x - fma(x, e, -z);
  e = fma(x, e - c, -c) - z;
  if (k == -1) return fma(0.5, x - e, -0.5);
  if (k == 1) return x < -0.25 ? -2.0 * (e - (x + 0.5)) : fma(2.0, x - e, 1.0);
  const double two_k = from_hi_word(0x3ff00000u + ((unsigned)k << 20));
  if (k <= -2 || k > 56) {
    const double y = 1.0 - (e - x);
    return (k == 1024 ? y * 2.0 * 0x1p1023 : y * two_k) - 1.0;
  }
  if (k < 20) return (from_hi_word(0x3ff00000u - (0x200000u >> k)) - (e - x)) * two_k;  // (1 - 2^-k) ...
  return ((x - (e + from_hi_word((unsigned)(0x3ff - k) << 20))) + 1.0) * two_k;          // ... 2^-k
}

__device__ __forceinline__ double tanh_det(double x) {
  const unsigned jx = hi_word(x), ix = jx & 0x7fffffffu;
  const bool neg = (jx >> 31) != 0;
  if (ix >= 0x7ff00000u) return neg ? 1.0 / x - 1.0 : 1.0 / x + 1.0;  // NaN, +-inf
  double z = 1.0;                           // |x| >= 22
  if (ix < 0x40360000u) {
    if (ix < 0x3c800000u) return x * (1.0 + x);  // |x| < 2^-55
    if (ix >= 0x3ff00000u) {
      const double m = expm1_det(2.0 * fabs(x));
      z = 1.0 - 2.0 / (m + 2.0);
    } else {
      const double m = expm1_det(-2.0 * fabs(x));
      z = -m / (m + 2.0);
    }
  }
  return neg ? -z : z;
}

}  // namespace dm
}  // namespace geon
