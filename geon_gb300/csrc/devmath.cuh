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
//  * expm1 (non-negative arguments below 44): y = k ln2 + r, Taylor series of
//    e^r - 1 to r^15, then 2^k * em + (2^k - 1).
//  * tanh(a) = expm1(2a) / (expm1(2a) + 2) for 2^-28 <= |a| < 22, odd.
//
// Constants are the doubles nearest pi/2 (three parts), 2/pi, ln 2 (two parts),
// 1/ln 2 and +-1/n!, produced by gen_math_constants.py in this directory.
// This file must be compiled without mul+add contraction (--fmad=false); the
// fma() calls below are the only fused operations.
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
constexpr double LN2_1 = 0x1.62e42fefa39efp-1;
constexpr double LN2_2 = 0x1.abc9e3b39803fp-56;
constexpr double INV_LN2 = 0x1.71547652b82fep+0;
constexpr double E2 = 0x1.0000000000000p-1;
constexpr double E3 = 0x1.5555555555555p-3;
constexpr double E4 = 0x1.5555555555555p-5;
constexpr double E5 = 0x1.1111111111111p-7;
constexpr double E6 = 0x1.6c16c16c16c17p-10;
constexpr double E7 = 0x1.a01a01a01a01ap-13;
constexpr double E8 = 0x1.a01a01a01a01ap-16;
constexpr double E9 = 0x1.71de3a556c734p-19;
constexpr double E10 = 0x1.27e4fb7789f5cp-22;
constexpr double E11 = 0x1.ae64567f544e4p-26;
constexpr double E12 = 0x1.1eed8eff8d898p-29;
constexpr double E13 = 0x1.6124613a86d09p-33;
constexpr double E14 = 0x1.93974a8c07c9dp-37;
constexpr double E15 = 0x1.ae7f3e733b81fp-41;

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

__device__ __forceinline__ double expm1_pos_det(double y) {
  const double k = rint(y * INV_LN2);
  const double r = fma(-k, LN2_1, y);
  const double rl = -k * LN2_2;
  double q = E15;
  q = fma(q, r, E14);
  q = fma(q, r, E13);
  q = fma(q, r, E12);
  q = fma(q, r, E11);
  q = fma(q, r, E10);
  q = fma(q, r, E9);
  q = fma(q, r, E8);
  q = fma(q, r, E7);
  q = fma(q, r, E6);
  q = fma(q, r, E5);
  q = fma(q, r, E4);
  q = fma(q, r, E3);
  q = fma(q, r, E2);
  const double em = r + fma(r * r, q, fma(rl, r, rl));
  if (k == 0.0) return em;
  const int ki = (int)k;
  return ldexp(em, ki) + (ldexp(1.0, ki) - 1.0);
}

__device__ __forceinline__ double tanh_det(double x) {
  if (isnan(x)) return x;
  const double a = fabs(x);
  double t;
  if (!(a < 22.0)) {
    t = 1.0;
  } else if (a < 0x1p-28) {
    return x;
  } else {
    const double e = expm1_pos_det(2.0 * a);
    t = e / (e + 2.0);
  }
  return copysign(t, x);
}

}  // namespace dm
}  // namespace geon
