// geon oracle: CPU FP64 restatement of the geon reference's ray-tracing and
// curvature path. TEST INFRASTRUCTURE ONLY (the checker), never the product.
//
// Build: g++ -O2 -ffp-contract=off -fno-fast-math -shared -fPIC (oracle/build.py).
// -ffp-contract=off matters: Rust never fuses a*b+c, and aarch64 gcc would
// otherwise contract by default. Explicit fma() appears only inside the
// deterministic math functions, where the method asks for it.
//
// Each function cites the reference file:line it restates. Operation order
// (left-associated sums, multiplication grouping) is kept exactly.
#include "geon_oracle.h"

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <thread>
#include <vector>

namespace {

typedef double Scalar;
struct Vec4 { double v[4]; double& operator[](int i) { return v[i]; } double operator[](int i) const { return v[i]; } };
struct Mat4 { double m[4][4]; };
struct Chr { double c[4][4][4]; };
struct State { double y[8]; };

constexpr double PI = 3.14159265358979323846;
constexpr double FRAC_PI_2 = 1.57079632679489661923;
constexpr double TAU = 6.28318530717958647692;

enum { DIVERGED = 0, CAPTURED = 1, ESCAPED = 2, NONE = -1 };

// ---------------------------------------------------------------------------
// Deterministic math ("geon" mode). Published methods:
//  * sin/cos: Cody & Waite argument reduction by pi/2 (Software Manual for the
//    Elementary Functions, 1980) with a three-part constant and a TwoSum tail,
//    then the Taylor series of sin and cos (coefficients (-1)^k/n!, rounded to
//    double) evaluated by Horner's rule with fma.
//  * tanh and expm1: the published fdlibm method (Sun Microsystems, 1993), the
//    one glibc's dbl-64 tanh and expm1 implement, with glibc's grouping of the
//    expm1 polynomial and the multiply-adds its compiler fuses written as
//    std::fma: equal to glibc 2.39's tanh bit for bit (see devmath.cuh, which
//    holds the same steps; the two must stay identical).
// The sin/cos constants are the double roundings of pi/2, 2/pi and 1/n!,
// derived with mpmath by geon_gb300/csrc/gen_math_constants.py; the expm1
// constants are the published ones.
//
// The expm1/tanh method, its range thresholds and its constants follow fdlibm,
// whose notice is kept here as its licence asks:
//   Copyright (C) 1993 by Sun Microsystems, Inc. All rights reserved.
//   Developed at SunSoft, a Sun Microsystems, Inc. business.
//   Permission to use, copy, modify, and distribute this
//   software is freely granted, provided that this notice
//   is preserved.
// ---------------------------------------------------------------------------
constexpr double GM_PIO2_1 = 0x1.921fb54442d18p+0;
constexpr double GM_PIO2_2 = 0x1.1a62633145c07p-54;
constexpr double GM_PIO2_3 = -0x1.f1976b7ed8fbcp-110;
constexpr double GM_2_OVER_PI = 0x1.45f306dc9c883p-1;
constexpr double GM_S3 = -0x1.5555555555555p-3;
constexpr double GM_S5 = 0x1.1111111111111p-7;
constexpr double GM_S7 = -0x1.a01a01a01a01ap-13;
constexpr double GM_S9 = 0x1.71de3a556c734p-19;
constexpr double GM_S11 = -0x1.ae64567f544e4p-26;
constexpr double GM_S13 = 0x1.6124613a86d09p-33;
constexpr double GM_S15 = -0x1.ae7f3e733b81fp-41;
constexpr double GM_S17 = 0x1.952c77030ad4ap-49;
constexpr double GM_C4 = 0x1.5555555555555p-5;
constexpr double GM_C6 = -0x1.6c16c16c16c17p-10;
constexpr double GM_C8 = 0x1.a01a01a01a01ap-16;
constexpr double GM_C10 = -0x1.27e4fb7789f5cp-22;
constexpr double GM_C12 = 0x1.1eed8eff8d898p-29;
constexpr double GM_C14 = -0x1.93974a8c07c9dp-37;
constexpr double GM_C16 = 0x1.ae7f3e733b81fp-45;
constexpr double GM_C18 = -0x1.6827863b97d97p-53;
constexpr double GM_EX_LN2_HI = 0x1.62e42fee00000p-1;
constexpr double GM_EX_LN2_LO = 0x1.a39ef35793c76p-33;
constexpr double GM_EX_INV_LN2 = 0x1.71547652b82fep+0;
constexpr double GM_EX_O_THRESHOLD = 0x1.62e42fefa39efp+9;
constexpr double GM_EX_Q1 = -0x1.11111111110f4p-5;
constexpr double GM_EX_Q2 = 0x1.a01a019fe5585p-10;
constexpr double GM_EX_Q3 = -0x1.4ce199eaadbb7p-14;
constexpr double GM_EX_Q4 = 0x1.0cfca86e65239p-18;
constexpr double GM_EX_Q5 = -0x1.afdb76e09c32dp-23;

void geon_sincos(double x, double* sp, double* cp) {
  if (!std::isfinite(x)) {
    *sp = std::numeric_limits<double>::quiet_NaN();
    *cp = *sp;
    return;
  }
  const double k = std::nearbyint(x * GM_2_OVER_PI);
  const double r1 = std::fma(-k, GM_PIO2_1, x);   // exact while |r1| < 1
  const double t = std::fma(-k, GM_PIO2_2, r1);    // reduced argument, rounded
  const double d = r1 - t;                         // exact (Sterbenz, or both multiples of ulp(t))
  const double tl = std::fma(-k, GM_PIO2_3, std::fma(-k, GM_PIO2_2, d));  // reduced argument is t + tl
  const double z = t * t;
  double ps = GM_S17;
  ps = std::fma(ps, z, GM_S15);
  ps = std::fma(ps, z, GM_S13);
  ps = std::fma(ps, z, GM_S11);
  ps = std::fma(ps, z, GM_S9);
  ps = std::fma(ps, z, GM_S7);
  ps = std::fma(ps, z, GM_S5);
  ps = std::fma(ps, z, GM_S3);
  const double tz = t * z;
  const double sv = t + std::fma(tz, ps, tl * std::fma(-0.5, z, 1.0));
  double pc = GM_C18;
  pc = std::fma(pc, z, GM_C16);
  pc = std::fma(pc, z, GM_C14);
  pc = std::fma(pc, z, GM_C12);
  pc = std::fma(pc, z, GM_C10);
  pc = std::fma(pc, z, GM_C8);
  pc = std::fma(pc, z, GM_C6);
  pc = std::fma(pc, z, GM_C4);
  const double hz = 0.5 * z;
  const double wc = 1.0 - hz;
  const double zl = std::fma(t, t, -z);            // exact error of z
  const double cv = wc + (((1.0 - wc) - hz) + (std::fma(z * z, pc, -0.5 * zl) - tl * t));
  const double q = k - 4.0 * std::floor(k * 0.25);  // k mod 4 in [0, 4), exact for every finite k
  if (q == 0.0) { *sp = sv; *cp = cv; }
  else if (q == 1.0) { *sp = cv; *cp = -sv; }
  else if (q == 2.0) { *sp = -sv; *cp = -cv; }
  else { *sp = -cv; *cp = sv; }
}

static uint32_t gm_hi_word(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return (uint32_t)(b >> 32);
}
static double gm_from_hi_word(uint32_t hi) {
  const uint64_t b = (uint64_t)hi << 32;
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}

// e^x - 1 for every double x; the same steps as devmath.cuh's expm1_det.
double geon_expm1(double x) {
  const uint32_t hxs = gm_hi_word(x);
  const bool neg = (hxs >> 31) != 0;
  const uint32_t hx = hxs & 0x7fffffffu;
  if (hx >= 0x4043687Au) {                  // |x| >= 56 ln 2
    if (hx >= 0x40862E42u) {                // |x| >= 709.78
      if (hx >= 0x7ff00000u) return std::isnan(x) ? x + x : (neg ? -1.0 : x);
      if (x > GM_EX_O_THRESHOLD) return INFINITY;
    }
    if (neg) return -1.0;
  }
  int k = 0;
  double c = 0.0;
  if (hx > 0x3fd62e42u) {                   // |x| > ln2 / 2
    double hi, lo;
    if (hx < 0x3FF0A2B2u) {                 // |x| < 3 ln2 / 2
      k = neg ? -1 : 1;
      hi = neg ? x + GM_EX_LN2_HI : x - GM_EX_LN2_HI;
      lo = neg ? -GM_EX_LN2_LO : GM_EX_LN2_LO;
    } else {
      k = (int)std::fma(GM_EX_INV_LN2, x, neg ? -0.5 : 0.5);
      const double tk = (double)k;
      hi = std::fma(-tk, GM_EX_LN2_HI, x);
      lo = tk * GM_EX_LN2_LO;
    }
    x = hi - lo;
    c = (hi - x) - lo;
  } else if (hx < 0x3c900000u) {            // |x| < 2^-54
    return x;
  }
  const double hfx = 0.5 * x, z = x * hfx;
  const double z2 = z * z, z4 = z2 * z2;
  const double R = std::fma(z4, std::fma(z, GM_EX_Q5, GM_EX_Q4),
                            std::fma(z2, std::fma(z, GM_EX_Q3, GM_EX_Q2), std::fma(z, GM_EX_Q1, 1.0)));
  const double t = std::fma(-R, hfx, 3.0);
  double e = z * ((R - t) / std::fma(-x, t, 6.0));
  if (k == 0) return x - std::fma(x, e, -z);
  e = std::fma(x, e - c, -c) - z;
  if (k == -1) return std::fma(0.5, x - e, -0.5);
  if (k == 1) return x < -0.25 ? -2.0 * (e - (x + 0.5)) : std::fma(2.0, x - e, 1.0);
  const double two_k = gm_from_hi_word(0x3ff00000u + ((uint32_t)k << 20));
  if (k <= -2 || k > 56) {
    const double y = 1.0 - (e - x);
    return (k == 1024 ? y * 2.0 * 0x1p1023 : y * two_k) - 1.0;
  }
  if (k < 20) return (gm_from_hi_word(0x3ff00000u - (0x200000u >> k)) - (e - x)) * two_k;
  return ((x - (e + gm_from_hi_word((uint32_t)(0x3ff - k) << 20))) + 1.0) * two_k;
}

double geon_tanh(double x) {
  const uint32_t jx = gm_hi_word(x), ix = jx & 0x7fffffffu;
  const bool neg = (jx >> 31) != 0;
  if (ix >= 0x7ff00000u) return neg ? 1.0 / x - 1.0 : 1.0 / x + 1.0;
  double z = 1.0;
  if (ix < 0x40360000u) {
    if (ix < 0x3c800000u) return x * (1.0 + x);
    if (ix >= 0x3ff00000u) {
      const double m = geon_expm1(2.0 * std::fabs(x));
      z = 1.0 - 2.0 / (m + 2.0);
    } else {
      const double m = geon_expm1(-2.0 * std::fabs(x));
      z = -m / (m + 2.0);
    }
  }
  return neg ? -z : z;
}

struct MathLibm {
  static double sin(double x) { return std::sin(x); }
  static double cos(double x) { return std::cos(x); }
  static double tanh(double x) { return std::tanh(x); }
};
// libm with every result moved one ulp up: measures how far a 1-ulp change in a
// transcendental moves each output (the reference's own sensitivity floor).
struct MathNudge {
  static double sin(double x) { return std::nextafter(std::sin(x), INFINITY); }
  static double cos(double x) { return std::nextafter(std::cos(x), INFINITY); }
  static double tanh(double x) { return std::nextafter(std::tanh(x), INFINITY); }
};
struct MathGeon {
  static double sin(double x) { double s, c; geon_sincos(x, &s, &c); return s; }
  static double cos(double x) { double s, c; geon_sincos(x, &s, &c); return c; }
  static double tanh(double x) { return geon_tanh(x); }
};

// ---------------------------------------------------------------------------
// types.rs
// ---------------------------------------------------------------------------
// types.rs:22-30 dot4: s += g[i][j] * a[i] * b[j], i-major.
inline double dot4(const Mat4& g, const Vec4& a, const Vec4& b) {
  double s = 0.0;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) s += g.m[i][j] * a[i] * b[j];
  return s;
}

// types.rs:34-47 inv4 calls nalgebra's Matrix4::try_inverse (not vendored in the
// reference). Stand-in: the adjugate by 2x2 minors (Laplace expansion, as in
// D. Eberly, "The Laplace Expansion Theorem: Computing the Determinants and
// Inverses of Matrices", Geometric Tools 2008). Singular iff det == 0, which is
// when try_inverse returns None (and the reference panics).
bool inv4(const Mat4& a, Mat4& out) {
  const double a00 = a.m[0][0], a01 = a.m[0][1], a02 = a.m[0][2], a03 = a.m[0][3];
  const double a10 = a.m[1][0], a11 = a.m[1][1], a12 = a.m[1][2], a13 = a.m[1][3];
  const double a20 = a.m[2][0], a21 = a.m[2][1], a22 = a.m[2][2], a23 = a.m[2][3];
  const double a30 = a.m[3][0], a31 = a.m[3][1], a32 = a.m[3][2], a33 = a.m[3][3];
  const double s0 = a00 * a11 - a10 * a01;
  const double s1 = a00 * a12 - a10 * a02;
  const double s2 = a00 * a13 - a10 * a03;
  const double s3 = a01 * a12 - a11 * a02;
  const double s4 = a01 * a13 - a11 * a03;
  const double s5 = a02 * a13 - a12 * a03;
  const double c5 = a22 * a33 - a32 * a23;
  const double c4 = a21 * a33 - a31 * a23;
  const double c3 = a21 * a32 - a31 * a22;
  const double c2 = a20 * a33 - a30 * a23;
  const double c1 = a20 * a32 - a30 * a22;
  const double c0 = a20 * a31 - a30 * a21;
  const double det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
  if (det == 0.0) return false;
  const double id = 1.0 / det;
  out.m[0][0] = (a11 * c5 - a12 * c4 + a13 * c3) * id;
  out.m[0][1] = (-a01 * c5 + a02 * c4 - a03 * c3) * id;
  out.m[0][2] = (a31 * s5 - a32 * s4 + a33 * s3) * id;
  out.m[0][3] = (-a21 * s5 + a22 * s4 - a23 * s3) * id;
  out.m[1][0] = (-a10 * c5 + a12 * c2 - a13 * c1) * id;
  out.m[1][1] = (a00 * c5 - a02 * c2 + a03 * c1) * id;
  out.m[1][2] = (-a30 * s5 + a32 * s2 - a33 * s1) * id;
  out.m[1][3] = (a20 * s5 - a22 * s2 + a23 * s1) * id;
  out.m[2][0] = (a10 * c4 - a11 * c2 + a13 * c0) * id;
  out.m[2][1] = (-a00 * c4 + a01 * c2 - a03 * c0) * id;
  out.m[2][2] = (a30 * s4 - a31 * s2 + a33 * s0) * id;
  out.m[2][3] = (-a20 * s4 + a21 * s2 - a23 * s0) * id;
  out.m[3][0] = (-a10 * c3 + a11 * c1 - a12 * c0) * id;
  out.m[3][1] = (a00 * c3 - a01 * c1 + a02 * c0) * id;
  out.m[3][2] = (-a30 * s3 + a31 * s1 - a32 * s0) * id;
  out.m[3][3] = (a20 * s3 - a21 * s1 + a22 * s0) * id;
  return true;
}

// A singular metric makes the reference panic (types.rs:39). The oracle records
// it in a thread-local flag and the exported entry points report -2.
thread_local bool g_singular = false;

Mat4 inv4_or_flag(const Mat4& a) {
  Mat4 out;
  if (!inv4(a, out)) {
    g_singular = true;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) out.m[i][j] = std::numeric_limits<double>::quiet_NaN();
  }
  return out;
}

Mat4 zero_mat() { Mat4 m; std::memset(&m, 0, sizeof m); return m; }

// ---------------------------------------------------------------------------
// metric/mod.rs: the Metric trait's defaults, as CRTP over concrete metrics.
// ---------------------------------------------------------------------------
template <class Derived>
struct MetricBase {
  const Derived& self() const { return *static_cast<const Derived*>(this); }
  // mod.rs:73-75
  void fd_step(const Vec4&, double h[4]) const { h[0] = h[1] = h[2] = h[3] = 1e-5; }
  // mod.rs:25-43
  void dg_default(const Vec4& x, Mat4 out[4]) const {
    double h[4];
    self().fd_step(x, h);
    for (int alpha = 0; alpha < 4; ++alpha) {
      Vec4 xp = x, xm = x;
      xp[alpha] += h[alpha];
      xm[alpha] -= h[alpha];
      const Mat4 gp = self().g(xp);
      const Mat4 gm = self().g(xm);
      const double two_h = 2.0 * h[alpha];
      for (int mu = 0; mu < 4; ++mu)
        for (int nu = 0; nu < 4; ++nu) out[alpha].m[mu][nu] = (gp.m[mu][nu] - gm.m[mu][nu]) / two_h;
    }
  }
  // mod.rs:46-48
  Mat4 g_inv_default(const Vec4& x) const { return inv4_or_flag(self().g(x)); }
  // mod.rs:51-69
  Chr christoffel_default(const Vec4& x) const {
    const Mat4 ginv = self().g_inv(x);
    Mat4 dg[4];
    self().dg(x, dg);
    Chr gamma;
    for (int mu = 0; mu < 4; ++mu)
      for (int alpha = 0; alpha < 4; ++alpha)
        for (int beta = 0; beta < 4; ++beta) {
          double s = 0.0;
          for (int sigma = 0; sigma < 4; ++sigma)
            s += ginv.m[mu][sigma] *
                 (dg[alpha].m[sigma][beta] + dg[beta].m[sigma][alpha] - dg[sigma].m[alpha][beta]);
          gamma.c[mu][alpha][beta] = 0.5 * s;
        }
    return gamma;
  }
  // mod.rs:91-108 (spherical chart default)
  template <class M>
  void asym_spherical(const Vec4& x, const Vec4& p, double out[3]) const {
    const double r = x[1], theta = x[2], phi = x[3];
    const double sin_t = M::sin(theta), cos_t = M::cos(theta);
    const double sin_p = M::sin(phi), cos_p = M::cos(phi);
    const double pr = p[1], pt = p[2], pp = p[3];
    const double vx = sin_t * cos_p * pr + r * cos_t * cos_p * pt - r * sin_t * sin_p * pp;
    const double vy = sin_t * sin_p * pr + r * cos_t * sin_p * pt + r * sin_t * cos_p * pp;
    const double vz = cos_t * pr - r * sin_t * pt;
    const double n = std::fmax(std::sqrt(vx * vx + vy * vy + vz * vz), 1e-30);
    out[0] = vx / n; out[1] = vy / n; out[2] = vz / n;
  }
};

// metric/minkowski.rs:8-43
template <class M>
struct Minkowski : MetricBase<Minkowski<M>> {
  Mat4 g(const Vec4&) const {
    Mat4 m = zero_mat();
    m.m[0][0] = -1.0; m.m[1][1] = 1.0; m.m[2][2] = 1.0; m.m[3][3] = 1.0;
    return m;
  }
  void dg(const Vec4&, Mat4 out[4]) const { for (int a = 0; a < 4; ++a) out[a] = zero_mat(); }
  Mat4 g_inv(const Vec4& x) const { return g(x); }
  Chr christoffel(const Vec4&) const { Chr c; std::memset(&c, 0, sizeof c); return c; }
  int terminate(const Vec4& x) const {
    const double r2 = x[1] * x[1] + x[2] * x[2] + x[3] * x[3];
    return r2 > 1e6 ? ESCAPED : NONE;
  }
  // No override: the spherical default applies even on this Cartesian chart.
  void asymptotic_direction(const Vec4& x, const Vec4& p, double out[3]) const {
    this->template asym_spherical<M>(x, p, out);
  }
};

// metric/schwarzschild.rs:12-126
template <class M>
struct Schwarzschild : MetricBase<Schwarzschild<M>> {
  double mass, horizon_pad, escape_radius;
  Mat4 g(const Vec4& x) const {
    const double r = x[1], theta = x[2], m = mass;
    const double f = 1.0 - 2.0 * m / r;
    const double sin_t = M::sin(theta);
    Mat4 gm = zero_mat();
    gm.m[0][0] = -f;
    gm.m[1][1] = 1.0 / f;
    gm.m[2][2] = r * r;
    gm.m[3][3] = r * r * sin_t * sin_t;
    return gm;
  }
  void dg(const Vec4& x, Mat4 out[4]) const { this->dg_default(x, out); }
  Mat4 g_inv(const Vec4& x) const {
    const double r = x[1], theta = x[2], m = mass;
    const double f = 1.0 - 2.0 * m / r;
    const double sin_t = M::sin(theta);
    Mat4 gm = zero_mat();
    gm.m[0][0] = -1.0 / f;
    gm.m[1][1] = f;
    gm.m[2][2] = 1.0 / (r * r);
    gm.m[3][3] = 1.0 / (r * r * sin_t * sin_t);
    return gm;
  }
  Chr christoffel(const Vec4& x) const {
    const double r = x[1], theta = x[2], m = mass;
    const double f = 1.0 - 2.0 * m / r;
    const double sin_t = M::sin(theta);
    const double cos_t = M::cos(theta);
    Chr g; std::memset(&g, 0, sizeof g);
    const double gtr = m / (r * r * f);
    g.c[0][0][1] = gtr;
    g.c[0][1][0] = gtr;
    g.c[1][0][0] = m * f / (r * r);
    g.c[1][1][1] = -m / (r * r * f);
    g.c[1][2][2] = -(r - 2.0 * m);
    g.c[1][3][3] = -(r - 2.0 * m) * sin_t * sin_t;
    const double gtheta_rt = 1.0 / r;
    g.c[2][1][2] = gtheta_rt;
    g.c[2][2][1] = gtheta_rt;
    g.c[2][3][3] = -sin_t * cos_t;
    g.c[3][1][3] = 1.0 / r;
    g.c[3][3][1] = 1.0 / r;
    const double cot = std::fabs(sin_t) < 1e-8 ? 0.0 : cos_t / sin_t;
    g.c[3][2][3] = cot;
    g.c[3][3][2] = cot;
    return g;
  }
  int terminate(const Vec4& x) const {
    const double r = x[1];
    if (!std::isfinite(r)) return DIVERGED;
    if (r < horizon_pad * 2.0 * mass) return CAPTURED;
    if (r > escape_radius * mass) return ESCAPED;
    return NONE;
  }
  void asymptotic_direction(const Vec4& x, const Vec4& p, double out[3]) const {
    this->template asym_spherical<M>(x, p, out);
  }
};

// metric/alcubierre.rs:14-89
template <class M>
struct Alcubierre : MetricBase<Alcubierre<M>> {
  double bubble_radius, bubble_thickness, ship_velocity, ship_x;
  double shape(const Vec4& x) const {
    const double dx = x[1] - ship_x, dy = x[2], dz = x[3];
    const double r_s = std::sqrt(dx * dx + dy * dy + dz * dz);
    const double s = bubble_thickness, r = bubble_radius;
    const double t_plus = M::tanh((r_s + r) / s);
    const double t_minus = M::tanh((r_s - r) / s);
    const double denom = 2.0 * M::tanh(r / s);
    return (t_plus - t_minus) / denom;
  }
  Mat4 g(const Vec4& x) const {
    const double v = ship_velocity;
    const double f = shape(x);
    Mat4 gm = zero_mat();
    gm.m[0][0] = -1.0 + v * v * f * f;
    gm.m[0][1] = -v * f;
    gm.m[1][0] = -v * f;
    gm.m[1][1] = 1.0;
    gm.m[2][2] = 1.0;
    gm.m[3][3] = 1.0;
    return gm;
  }
  void dg(const Vec4& x, Mat4 out[4]) const { this->dg_default(x, out); }
  Mat4 g_inv(const Vec4& x) const { return this->g_inv_default(x); }
  Chr christoffel(const Vec4& x) const { return this->christoffel_default(x); }
  int terminate(const Vec4& x) const {
    const double r2 = x[1] * x[1] + x[2] * x[2] + x[3] * x[3];
    if (!std::isfinite(r2)) return DIVERGED;
    return r2 > 1e6 ? ESCAPED : NONE;
  }
  void asymptotic_direction(const Vec4&, const Vec4& p, double out[3]) const {
    const double vx = p[1], vy = p[2], vz = p[3];
    const double n = std::fmax(std::sqrt(vx * vx + vy * vy + vz * vz), 1e-30);
    out[0] = vx / n; out[1] = vy / n; out[2] = vz / n;
  }
};

// metric/morris_thorne.rs:11-78
template <class M>
struct MorrisThorne : MetricBase<MorrisThorne<M>> {
  double throat_radius;
  Mat4 g(const Vec4& x) const {
    const double l = x[1], theta = x[2], b0 = throat_radius;
    const double r2 = b0 * b0 + l * l;
    const double sin_t = M::sin(theta);
    Mat4 gm = zero_mat();
    gm.m[0][0] = -1.0;
    gm.m[1][1] = 1.0;
    gm.m[2][2] = r2;
    gm.m[3][3] = r2 * sin_t * sin_t;
    return gm;
  }
  void dg(const Vec4& x, Mat4 out[4]) const { this->dg_default(x, out); }
  Mat4 g_inv(const Vec4& x) const { return this->g_inv_default(x); }
  Chr christoffel(const Vec4& x) const { return this->christoffel_default(x); }
  int terminate(const Vec4& x) const {
    const double l = x[1];
    if (!std::isfinite(l)) return DIVERGED;
    return std::fabs(l) > 1000.0 ? ESCAPED : NONE;
  }
  void asymptotic_direction(const Vec4& x, const Vec4& p, double out[3]) const {
    const double l = x[1], theta = x[2], phi = x[3];
    const double sin_t = M::sin(theta), cos_t = M::cos(theta);
    const double sin_p = M::sin(phi), cos_p = M::cos(phi);
    const double pl = p[1], pt = p[2], pp = p[3];
    const double r_eff = std::fmax(std::fabs(l), 1e-30);
    const double vx = sin_t * cos_p * pl + r_eff * cos_t * cos_p * pt - r_eff * sin_t * sin_p * pp;
    const double vy = sin_t * sin_p * pl + r_eff * cos_t * sin_p * pt + r_eff * sin_t * cos_p * pp;
    const double vz = cos_t * pl - r_eff * sin_t * pt;
    const double n = std::fmax(std::sqrt(vx * vx + vy * vy + vz * vz), 1e-30);
    const double sign = l < 0.0 ? -1.0 : 1.0;
    out[0] = sign * vx / n; out[1] = vy / n; out[2] = vz / n;
  }
};

// ---------------------------------------------------------------------------
// integrator.rs + geodesic.rs
// ---------------------------------------------------------------------------
inline Vec4 pos(const State& y) { return Vec4{{y.y[0], y.y[1], y.y[2], y.y[3]}}; }
inline Vec4 mom(const State& y) { return Vec4{{y.y[4], y.y[5], y.y[6], y.y[7]}}; }

// geodesic.rs:38-59
template <class Met>
State rhs(const Met& metric, const State& y) {
  const Vec4 x = pos(y), p = mom(y);
  const Chr g = metric.christoffel(x);
  State out;
  for (int mu = 0; mu < 4; ++mu) out.y[mu] = p[mu];
  for (int mu = 0; mu < 4; ++mu) {
    double s = 0.0;
    for (int alpha = 0; alpha < 4; ++alpha)
      for (int beta = 0; beta < 4; ++beta) s += g.c[mu][alpha][beta] * p[alpha] * p[beta];
    out.y[4 + mu] = -s;
  }
  return out;
}

// integrator.rs:16-40
template <class Met>
State rk4_step(const Met& metric, const State& y, double h) {
  const State k1 = rhs(metric, y);
  State y2 = y;
  for (int i = 0; i < 8; ++i) y2.y[i] = y.y[i] + 0.5 * h * k1.y[i];
  const State k2 = rhs(metric, y2);
  State y3 = y;
  for (int i = 0; i < 8; ++i) y3.y[i] = y.y[i] + 0.5 * h * k2.y[i];
  const State k3 = rhs(metric, y3);
  State y4 = y;
  for (int i = 0; i < 8; ++i) y4.y[i] = y.y[i] + h * k3.y[i];
  const State k4 = rhs(metric, y4);
  State out = y;
  const double sixth = h / 6.0;
  for (int i = 0; i < 8; ++i) out.y[i] += sixth * (k1.y[i] + 2.0 * k2.y[i] + 2.0 * k3.y[i] + k4.y[i]);
  return out;
}

struct TraceResult { int term; State final_state; int64_t steps; double resid; };

// geodesic.rs:62-117
template <class Met>
TraceResult trace(const Met& metric, const State& y0, double step, int64_t max_steps) {
  State y = y0;
  for (int64_t n = 0; n < max_steps; ++n) {
    const Vec4 x = pos(y);
    const int reason = metric.terminate(x);
    if (reason != NONE) {
      const Mat4 g = metric.g(x);
      const Vec4 p = mom(y);
      return TraceResult{reason, y, n, std::fabs(dot4(g, p, p))};
    }
    const State yn = rk4_step(metric, y, step);
    bool bad = false;
    for (int i = 0; i < 8; ++i) bad |= !std::isfinite(yn.y[i]);
    if (bad) {
      const Mat4 g = metric.g(x);
      const Vec4 p = mom(y);
      return TraceResult{DIVERGED, y, n, std::fabs(dot4(g, p, p))};
    }
    y = yn;
  }
  const Vec4 x = pos(y);
  const Mat4 g = metric.g(x);
  const Vec4 p = mom(y);
  return TraceResult{DIVERGED, y, max_steps, std::fabs(dot4(g, p, p))};
}

// Adaptive stepping, the restatement of the GPU's GEON_ADAPTIVE mode (not a
// reference feature: integrator.rs:5-7 lists it as a TODO). Dormand & Prince
// 5(4) (J. Comput. Appl. Math. 6 (1980) 19-26) with first-same-as-last reuse,
// the Hairer-Norsett-Wanner RMS error norm and a controller made of IEEE
// operations only: accept when err <= 1, next h = h * clamp(0.9 / sqrt(sqrt(err)),
// 0.2, 5); a non-finite trial is a rejection; 64 consecutive rejections end the
// ray Diverged; max_steps counts accepted steps. Every expression keeps the
// GPU's evaluation order, so both give the same bits.
namespace dp5 {
constexpr double A21 = 1.0 / 5.0;
constexpr double A31 = 3.0 / 40.0, A32 = 9.0 / 40.0;
constexpr double A41 = 44.0 / 45.0, A42 = -56.0 / 15.0, A43 = 32.0 / 9.0;
constexpr double A51 = 19372.0 / 6561.0, A52 = -25360.0 / 2187.0, A53 = 64448.0 / 6561.0, A54 = -212.0 / 729.0;
constexpr double A61 = 9017.0 / 3168.0, A62 = -355.0 / 33.0, A63 = 46732.0 / 5247.0, A64 = 49.0 / 176.0,
                 A65 = -5103.0 / 18656.0;
constexpr double B1 = 35.0 / 384.0, B3 = 500.0 / 1113.0, B4 = 125.0 / 192.0, B5 = -2187.0 / 6784.0,
                 B6 = 11.0 / 84.0;
constexpr double E1 = 71.0 / 57600.0, E3 = -71.0 / 16695.0, E4 = 71.0 / 1920.0, E5 = -17253.0 / 339200.0,
                 E6 = 22.0 / 525.0, E7 = -1.0 / 40.0;
constexpr int MAX_REJECT = 64;
}  // namespace dp5

template <class Met>
TraceResult trace_adaptive(const Met& metric, const State& y0, double h0, int64_t max_steps, double rtol,
                           double atol) {
  using namespace dp5;
  State y = y0, k1;
  bool fresh = true;
  double h = h0;
  auto result = [&](int reason, int64_t n) {
    const Vec4 x = pos(y);
    const Mat4 g = metric.g(x);
    const Vec4 p = mom(y);
    return TraceResult{reason, y, n, std::fabs(dot4(g, p, p))};
  };
  for (int64_t n = 0; n < max_steps; ++n) {
    const int reason = metric.terminate(pos(y));
    if (reason != NONE) return result(reason, n);
    if (fresh) {
      k1 = rhs(metric, y);
      fresh = false;
    }
    bool accepted = false;
    for (int attempt = 0; attempt < MAX_REJECT && !accepted; ++attempt) {
      State ys, yn;
      for (int i = 0; i < 8; ++i) ys.y[i] = y.y[i] + h * (A21 * k1.y[i]);
      const State k2 = rhs(metric, ys);
      for (int i = 0; i < 8; ++i) ys.y[i] = y.y[i] + h * (A31 * k1.y[i] + A32 * k2.y[i]);
      const State k3 = rhs(metric, ys);
      for (int i = 0; i < 8; ++i) ys.y[i] = y.y[i] + h * ((A41 * k1.y[i] + A42 * k2.y[i]) + A43 * k3.y[i]);
      const State k4 = rhs(metric, ys);
      for (int i = 0; i < 8; ++i)
        ys.y[i] = y.y[i] + h * (((A51 * k1.y[i] + A52 * k2.y[i]) + A53 * k3.y[i]) + A54 * k4.y[i]);
      const State k5 = rhs(metric, ys);
      for (int i = 0; i < 8; ++i)
        ys.y[i] = y.y[i] + h * ((((A61 * k1.y[i] + A62 * k2.y[i]) + A63 * k3.y[i]) + A64 * k4.y[i]) +
                                A65 * k5.y[i]);
      const State k6 = rhs(metric, ys);
      for (int i = 0; i < 8; ++i)
        yn.y[i] = y.y[i] + h * ((((B1 * k1.y[i] + B3 * k3.y[i]) + B4 * k4.y[i]) + B5 * k5.y[i]) + B6 * k6.y[i]);
      const State k7 = rhs(metric, yn);
      double sum = 0.0;
      bool finite = true;
      for (int i = 0; i < 8; ++i) {
        const double e = h * (((((E1 * k1.y[i] + E3 * k3.y[i]) + E4 * k4.y[i]) + E5 * k5.y[i]) + E6 * k6.y[i]) +
                              E7 * k7.y[i]);
        const double ay = std::fabs(y.y[i]), an = std::fabs(yn.y[i]);
        const double sc = atol + rtol * (ay > an ? ay : an);
        const double q = e / sc;
        sum = sum + q * q;
        finite = finite && std::isfinite(yn.y[i]) && std::isfinite(k7.y[i]);
      }
      const double err = finite ? std::sqrt(sum / 8.0) : INFINITY;
      if (!(err <= 1.0)) {
        double fac = 0.2;
        if (std::isfinite(err)) {
          fac = 0.9 / std::sqrt(std::sqrt(err));
          if (fac < 0.2) fac = 0.2;
        }
        h = h * fac;
        continue;
      }
      double fac = 5.0;
      if (err > 0.0) {
        fac = 0.9 / std::sqrt(std::sqrt(err));
        if (fac > 5.0) fac = 5.0;
        if (fac < 0.2) fac = 0.2;
      }
      y = yn;
      k1 = k7;
      h = h * fac;
      accepted = true;
    }
    if (!accepted) return result(DIVERGED, n);
  }
  return result(DIVERGED, max_steps);
}

// ---------------------------------------------------------------------------
// camera.rs
// ---------------------------------------------------------------------------
// Rust f64::to_radians multiplies by the double constant PI/180.
inline double to_radians(double deg) { return deg * (PI / 180.0); }

// camera.rs:47-97. Returns 0, -3 (g_tt >= 0, assert at :53), -4 (n2 <= 0, :85-88).
template <class Met>
int tetrad(const Met& metric, const Vec4& observer, Mat4& tet) {
  const Mat4 g = metric.g(observer);
  tet = zero_mat();
  const double gtt = g.m[0][0];
  if (!(gtt < 0.0)) return -3;
  const double n0 = 1.0 / std::sqrt(-gtt);
  tet.m[0][0] = n0;
  const double seeds[3][4] = {{0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  for (int i = 0; i < 3; ++i) {
    Vec4 v{{seeds[i][0], seeds[i][1], seeds[i][2], seeds[i][3]}};
    for (int k = 0; k <= i; ++k) {
      const Vec4 ek{{tet.m[k][0], tet.m[k][1], tet.m[k][2], tet.m[k][3]}};
      const double proj = dot4(g, ek, v);
      const double norm_k = dot4(g, ek, ek);
      const double coeff = proj / norm_k;
      for (int mu = 0; mu < 4; ++mu) v[mu] -= coeff * ek[mu];
    }
    const double n2 = dot4(g, v, v);
    if (!(n2 > 0.0)) return -4;
    const double n = std::sqrt(n2);
    for (int mu = 0; mu < 4; ++mu) v[mu] /= n;
    for (int mu = 0; mu < 4; ++mu) tet.m[i + 1][mu] = v[mu];
  }
  return 0;
}

// camera.rs:113-160. forward_sign = +1 is the reference (forward = -e1, right = +e3);
// -1 looks along +e1 with right = -e3 (an extension the reference camera lacks).
State ray_state_sub(const Mat4& tet, const double obs[4], double fov_y_rad, int64_t width,
                    int64_t height, int64_t i, int64_t j, double du, double dv, int forward_sign) {
  const double aspect = (double)width / (double)height;
  const double h = std::tan(fov_y_rad * 0.5);
  const double w = h * aspect;
  const double u = (2.0 * ((double)i + du) / (double)width - 1.0) * w;
  const double v = -(2.0 * ((double)j + dv) / (double)height - 1.0) * h;
  const double fs = (double)forward_sign;
  const double dx = -fs;
  const double dy = -v;
  const double dz = forward_sign == 1 ? u : fs * u;
  const double norm = std::sqrt(dx * dx + dy * dy + dz * dz);
  const double n1 = dx / norm, n2 = dy / norm, n3 = dz / norm;
  State s;
  for (int mu = 0; mu < 4; ++mu) s.y[mu] = obs[mu];
  for (int mu = 0; mu < 4; ++mu)
    s.y[4 + mu] = tet.m[0][mu] + n1 * tet.m[1][mu] + n2 * tet.m[2][mu] + n3 * tet.m[3][mu];
  return s;
}

// ---------------------------------------------------------------------------
// sky.rs
// ---------------------------------------------------------------------------
constexpr double PHI_OFFSET = 0.37;
constexpr double THETA_OFFSET = 0.21;

inline uint64_t hash1(uint64_t x) {  // sky.rs:26-34
  x *= 0x9E3779B97F4A7C15ull;
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  x ^= x >> 31;
  return x;
}
inline uint64_t hash2(int64_t a, int64_t b) {  // sky.rs:37-39
  return hash1(((uint64_t)a * 73856093ull) ^ ((uint64_t)b * 19349663ull));
}
// Rust `f64 as i64` saturates and maps NaN to 0.
inline int64_t sat_i64(double v) {
  if (std::isnan(v)) return 0;
  if (v >= 9223372036854775807.0) return INT64_MAX;
  if (v <= -9223372036854775808.0) return INT64_MIN;
  return (int64_t)v;
}
inline double rem_euclid(double a, double b) {
  const double r = std::fmod(a, b);
  return r < 0.0 ? r + std::fabs(b) : r;
}
inline int64_t rem_euclid_i(int64_t a, int64_t b) {
  const int64_t r = a % b;
  return r < 0 ? r + (b < 0 ? -b : b) : r;
}
inline double clampd(double x, double lo, double hi) {
  if (x < lo) x = lo;
  if (x > hi) x = hi;
  return x;
}

void stars(double theta, double phi, bool show, float out[3]) {  // sky.rs:43-68
  out[0] = out[1] = out[2] = 0.0f;
  if (!show) return;
  const double n_phi = 512.0, n_theta = 256.0;
  const double phi_shift = rem_euclid(phi + PHI_OFFSET, TAU);
  const double theta_shift = clampd(theta + THETA_OFFSET, 0.0, PI);
  const int64_t i = sat_i64(std::floor(phi_shift / TAU * n_phi));
  const int64_t j = sat_i64(std::floor(theta_shift / PI * n_theta));
  const uint64_t h = hash2(i, j);
  const double prob = (double)(h & 0xFFFF) / 65535.0;
  if (prob < 0.004) {
    const double brightness = 0.4 + 0.6 * ((double)((h >> 16) & 0xFF) / 255.0);
    const double temp = (double)((h >> 24) & 0xFF) / 255.0;
    out[0] = (float)(brightness * (1.0 - 0.3 * temp));
    out[1] = (float)(brightness * (1.0 - 0.1 * std::fabs(temp - 0.5)));
    out[2] = (float)(brightness * (0.7 + 0.3 * temp));
  }
}

void sectors(double theta, double phi, float out[3]) {  // sky.rs:72-104
  const double phi_shift = rem_euclid(phi + PHI_OFFSET, TAU);
  const double theta_shift = clampd(theta + THETA_OFFSET, 0.0, PI);
  const int64_t phi_mod = sat_i64(std::floor(phi_shift / TAU * 6.0));
  const int64_t band = sat_i64(std::floor(theta_shift / PI * 3.0));
  static const double palette[6][3] = {{0.15, 0.08, 0.20}, {0.08, 0.15, 0.22}, {0.20, 0.15, 0.08},
                                       {0.10, 0.18, 0.10}, {0.22, 0.10, 0.10}, {0.10, 0.10, 0.22}};
  const double* base = palette[rem_euclid_i(phi_mod, 6)];
  const double band_mod = rem_euclid_i(band, 2) == 0 ? 1.0 : 0.6;
  const int64_t nphi = 24, ntheta = 12;
  const int64_t ic = sat_i64(std::floor(phi_shift / TAU * (double)nphi));
  const int64_t jc = sat_i64(std::floor(theta_shift / PI * (double)ntheta));
  const double check = rem_euclid_i(ic + jc, 2) == 0 ? 1.0 : 0.55;
  out[0] = (float)(base[0] * band_mod * check);
  out[1] = (float)(base[1] * band_mod * check);
  out[2] = (float)(base[2] * band_mod * check);
}

void sky_sample(const double dir[3], bool show, float out[3]) {  // sky.rs:107-120
  const double x = dir[0], y = dir[1], z = dir[2];
  const double r = std::fmax(std::sqrt(x * x + y * y + z * z), 1e-30);
  const double theta = std::acos(clampd(z / r, -1.0, 1.0));
  const double phi = std::atan2(y, x);
  float s[3], st[3];
  sectors(theta, phi, s);
  stars(theta, phi, show, st);
  for (int c = 0; c < 3; ++c) out[c] = std::fmin(s[c] + st[c], 1.0f);
}

// ---------------------------------------------------------------------------
// Work distribution over host threads (the reference uses rayon par_iter).
// ---------------------------------------------------------------------------
int resolve_threads(int nthreads) {
  if (nthreads > 0) return nthreads;
  const unsigned hc = std::thread::hardware_concurrency();
  return hc ? (int)hc : 1;
}

void parallel_for(int64_t n, int nthreads, const std::function<void(int64_t)>& fn) {
  nthreads = resolve_threads(nthreads);
  if (nthreads <= 1 || n <= 1) {
    for (int64_t i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<int64_t> next(0);
  const int64_t chunk = 1;
  auto worker = [&]() {
    for (;;) {
      const int64_t i = next.fetch_add(chunk);
      if (i >= n) break;
      fn(i);
    }
  };
  std::vector<std::thread> pool;
  const int nt = (int)std::min<int64_t>(nthreads, n);
  for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
}

// A sampled metric (the GPU's GEON_FIELD, geon_metric_create_field): the 10
// unique components of a static g at the nodes of a regular grid, used as the
// control points of a uniform cubic B-spline; everything else (g^-1, dg,
// Christoffel, curvature, trace) is the reference's generic fallback path
// (mod.rs:25-69). The field is registered once with orc_field_set.
struct FieldData {
  std::vector<double> c;
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, inv_d[3] = {0, 0, 0};
  int64_t n[3] = {1, 1, 1};
  int chart = 0;  // 0 Cartesian, 1 spherical
};
FieldData g_field;

template <class M>
struct FieldMetric : MetricBase<FieldMetric<M>> {
  const FieldData* F = &g_field;
  void axis(int a, double x, int64_t idx[4], double w[4]) const {
    const double u = (x - F->lo[a]) * F->inv_d[a];
    const double fl = std::floor(u);
    const double t = u - fl;
    const double fc = std::fmin(std::fmax(fl, -2.0), (double)F->n[a] + 1.0);
    const int64_t i = (int64_t)fc;
    const double sixth = 1.0 / 6.0;
    const double t2 = t * t, t3 = t2 * t, s = 1.0 - t;
    w[0] = ((s * s) * s) * sixth;
    w[1] = ((3.0 * t3 - 6.0 * t2) + 4.0) * sixth;
    w[2] = (((-3.0 * t3 + 3.0 * t2) + 3.0 * t) + 1.0) * sixth;
    w[3] = t3 * sixth;
    for (int q = 0; q < 4; ++q) {
      int64_t j = i - 1 + q;
      idx[q] = j < 0 ? 0 : (j > F->n[a] - 1 ? F->n[a] - 1 : j);
    }
  }
  Mat4 g(const Vec4& x) const {
    int64_t ix[4], iy[4], iz[4];
    double wx[4], wy[4], wz[4];
    axis(0, x[1], ix, wx);
    axis(1, x[2], iy, wy);
    axis(2, x[3], iz, wz);
    double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int c = 0; c < 4; ++c) {
      double accy[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int b = 0; b < 4; ++b) {
        double accx[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        const int64_t row = F->n[0] * (iy[b] + F->n[1] * iz[c]);
        for (int a = 0; a < 4; ++a) {
          const double* s = F->c.data() + 10 * (ix[a] + row);
          for (int q = 0; q < 10; ++q) accx[q] = accx[q] + wx[a] * s[q];
        }
        for (int q = 0; q < 10; ++q) accy[q] = accy[q] + wy[b] * accx[q];
      }
      for (int q = 0; q < 10; ++q) acc[q] = acc[q] + wz[c] * accy[q];
    }
    static const int comp[4][4] = {{0, 1, 2, 3}, {1, 4, 5, 6}, {2, 5, 7, 8}, {3, 6, 8, 9}};
    Mat4 gm;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) gm.m[i][j] = acc[comp[i][j]];
    return gm;
  }
  void dg(const Vec4& x, Mat4 out[4]) const { this->dg_default(x, out); }
  Mat4 g_inv(const Vec4& x) const { return this->g_inv_default(x); }
  Chr christoffel(const Vec4& x) const { return this->christoffel_default(x); }
  int terminate(const Vec4& x) const {
    if (!std::isfinite(x[1]) || !std::isfinite(x[2]) || !std::isfinite(x[3])) return DIVERGED;
    if (F->chart == 1 && F->n[0] > 1 && x[1] < F->lo[0]) return CAPTURED;
    for (int a = 0; a < 3; ++a)
      if (F->n[a] > 1 && (x[a + 1] < F->lo[a] || x[a + 1] > F->hi[a])) return ESCAPED;
    return NONE;
  }
  void asymptotic_direction(const Vec4& x, const Vec4& p, double out[3]) const {
    if (F->chart == 1) {
      this->template asym_spherical<M>(x, p, out);
      return;
    }
    const double vx = p[1], vy = p[2], vz = p[3];
    const double n = std::fmax(std::sqrt(vx * vx + vy * vy + vz * vz), 1e-30);
    out[0] = vx / n; out[1] = vy / n; out[2] = vz / n;
  }
};

// Dispatch a callable over the (metric kind, math mode) instantiation.
template <class F>
int with_metric(int kind, const double* p, int math, F&& f) {
  if (kind == 4) {  // the sampled metric: sin/cos only in the spherical-chart escape direction
    if (math == ORC_MATH_NUDGE) { FieldMetric<MathNudge> m; return f(m); }
    if (math == ORC_MATH_GEON) { FieldMetric<MathGeon> m; return f(m); }
    FieldMetric<MathLibm> m;
    return f(m);
  }
  if (math == ORC_MATH_NUDGE) {
    switch (kind) {
      case 0: { Minkowski<MathNudge> m; return f(m); }
      case 1: { Schwarzschild<MathNudge> m; m.mass = p[0]; m.horizon_pad = p[1]; m.escape_radius = p[2]; return f(m); }
      case 2: { Alcubierre<MathNudge> m; m.bubble_radius = p[0]; m.bubble_thickness = p[1]; m.ship_velocity = p[2]; m.ship_x = p[3]; return f(m); }
      case 3: { MorrisThorne<MathNudge> m; m.throat_radius = p[0]; return f(m); }
    }
    return -1;
  }
  if (math == ORC_MATH_GEON) {
    switch (kind) {
      case 0: { Minkowski<MathGeon> m; return f(m); }
      case 1: { Schwarzschild<MathGeon> m; m.mass = p[0]; m.horizon_pad = p[1]; m.escape_radius = p[2]; return f(m); }
      case 2: { Alcubierre<MathGeon> m; m.bubble_radius = p[0]; m.bubble_thickness = p[1]; m.ship_velocity = p[2]; m.ship_x = p[3]; return f(m); }
      case 3: { MorrisThorne<MathGeon> m; m.throat_radius = p[0]; return f(m); }
    }
  } else {
    switch (kind) {
      case 0: { Minkowski<MathLibm> m; return f(m); }
      case 1: { Schwarzschild<MathLibm> m; m.mass = p[0]; m.horizon_pad = p[1]; m.escape_radius = p[2]; return f(m); }
      case 2: { Alcubierre<MathLibm> m; m.bubble_radius = p[0]; m.bubble_thickness = p[1]; m.ship_velocity = p[2]; m.ship_x = p[3]; return f(m); }
      case 3: { MorrisThorne<MathLibm> m; m.throat_radius = p[0]; return f(m); }
    }
  }
  return -1;
}

// Schwarzschild only (the shadow validation of bin/validate_shadow.rs).
template <class F>
int with_schw(const double* p, int math, F&& f) {
  if (math == ORC_MATH_NUDGE) {
    Schwarzschild<MathNudge> m; m.mass = p[0]; m.horizon_pad = p[1]; m.escape_radius = p[2];
    return f(m);
  }
  if (math == ORC_MATH_GEON) {
    Schwarzschild<MathGeon> m; m.mass = p[0]; m.horizon_pad = p[1]; m.escape_radius = p[2];
    return f(m);
  }
  Schwarzschild<MathLibm> m; m.mass = p[0]; m.horizon_pad = p[1]; m.escape_radius = p[2];
  return f(m);
}

inline Vec4 load4(const double* p) { return Vec4{{p[0], p[1], p[2], p[3]}}; }

// ---------------------------------------------------------------------------
// curvature.rs
// ---------------------------------------------------------------------------
struct Riemann { double r[4][4][4][4]; };

// curvature.rs:25-46
template <class Met>
void d_christoffel(const Met& metric, const Vec4& x, Chr out[4]) {
  double h[4];
  metric.fd_step(x, h);
  for (int alpha = 0; alpha < 4; ++alpha) {
    Vec4 xp = x, xm = x;
    xp[alpha] += h[alpha];
    xm[alpha] -= h[alpha];
    const Chr gp = metric.christoffel(xp);
    const Chr gm = metric.christoffel(xm);
    const double inv_2h = 1.0 / (2.0 * h[alpha]);
    for (int mu = 0; mu < 4; ++mu)
      for (int beta = 0; beta < 4; ++beta)
        for (int gamma = 0; gamma < 4; ++gamma)
          out[alpha].c[mu][beta][gamma] = (gp.c[mu][beta][gamma] - gm.c[mu][beta][gamma]) * inv_2h;
  }
}

// curvature.rs:48-70
template <class Met>
void riemann(const Met& metric, const Vec4& x, Riemann& r) {
  const Chr gamma = metric.christoffel(x);
  Chr dgamma[4];
  d_christoffel(metric, x, dgamma);
  for (int rho = 0; rho < 4; ++rho)
    for (int sigma = 0; sigma < 4; ++sigma)
      for (int mu = 0; mu < 4; ++mu)
        for (int nu = 0; nu < 4; ++nu) {
          const double term1 = dgamma[mu].c[rho][nu][sigma];
          const double term2 = dgamma[nu].c[rho][mu][sigma];
          double term3 = 0.0, term4 = 0.0;
          for (int lambda = 0; lambda < 4; ++lambda) {
            term3 += gamma.c[rho][mu][lambda] * gamma.c[lambda][nu][sigma];
            term4 += gamma.c[rho][nu][lambda] * gamma.c[lambda][mu][sigma];
          }
          r.r[rho][sigma][mu][nu] = term1 - term2 + term3 - term4;
        }
}

// curvature.rs:72-85
Mat4 ricci_from(const Riemann& r) {
  Mat4 ric;
  for (int mu = 0; mu < 4; ++mu)
    for (int nu = 0; nu < 4; ++nu) {
      double s = 0.0;
      for (int alpha = 0; alpha < 4; ++alpha) s += r.r[alpha][mu][alpha][nu];
      ric.m[mu][nu] = s;
    }
  return ric;
}
template <class Met>
Mat4 ricci(const Met& metric, const Vec4& x) {
  Riemann r;
  riemann(metric, x, r);
  return ricci_from(r);
}
// curvature.rs:87-97
double ricci_scalar_from(const Mat4& g_inv, const Mat4& ric) {
  double s = 0.0;
  for (int mu = 0; mu < 4; ++mu)
    for (int nu = 0; nu < 4; ++nu) s += g_inv.m[mu][nu] * ric.m[mu][nu];
  return s;
}
// curvature.rs:99-110
Mat4 einstein_from(const Mat4& g, const Mat4& ric, double r) {
  Mat4 ein;
  for (int mu = 0; mu < 4; ++mu)
    for (int nu = 0; nu < 4; ++nu) ein.m[mu][nu] = ric.m[mu][nu] - 0.5 * g.m[mu][nu] * r;
  return ein;
}
// curvature.rs:112-122
Mat4 stress_from(const Mat4& ein) {
  const double factor = 1.0 / (8.0 * PI);
  Mat4 t;
  for (int mu = 0; mu < 4; ++mu)
    for (int nu = 0; nu < 4; ++nu) t.m[mu][nu] = ein.m[mu][nu] * factor;
  return t;
}
// curvature.rs:127-136
double nec_from(const Mat4& t, const Vec4& k) {
  double s = 0.0;
  for (int mu = 0; mu < 4; ++mu)
    for (int nu = 0; nu < 4; ++nu) s += t.m[mu][nu] * k[mu] * k[nu];
  return s;
}

// The reference call graph: einstein = g, ricci(riemann), ricci_scalar(g_inv, ricci(riemann)).
// Riemann is deterministic, so computing it once (faithful=0) gives identical bits.
template <class Met>
void curvature_point(const Met& metric, const Vec4& x, int faithful, Riemann* riem_out, Mat4& ric,
                     double& rs, Mat4& ein, Mat4& t) {
  Riemann r;
  riemann(metric, x, r);
  if (riem_out) *riem_out = r;
  ric = ricci_from(r);
  const Mat4 g_inv = metric.g_inv(x);
  if (faithful) {
    const Mat4 ric2 = ricci(metric, x);  // ricci_scalar's own ricci() call
    rs = ricci_scalar_from(g_inv, ric2);
  } else {
    rs = ricci_scalar_from(g_inv, ric);
  }
  ein = einstein_from(metric.g(x), ric, rs);
  t = stress_from(ein);
}

// bin/validate_shadow.rs:20-35
template <class M>
State equatorial_ray_t(double m, double r_obs, double alpha) {
  const double f = 1.0 - 2.0 * m / r_obs;
  const double sin_a = M::sin(alpha);
  const double cos_a = M::cos(alpha);
  const double pt = 1.0 / std::sqrt(f);
  const double pr = -cos_a * std::sqrt(f);
  const double pphi = sin_a / r_obs;
  State s = {{0.0, r_obs, FRAC_PI_2, 0.0, pt, pr, 0.0, pphi}};
  return s;
}

State equatorial_ray(double m, double r_obs, int math, double alpha) {
  if (math == ORC_MATH_NUDGE) return equatorial_ray_t<MathNudge>(m, r_obs, alpha);
  return math == ORC_MATH_GEON ? equatorial_ray_t<MathGeon>(m, r_obs, alpha)
                               : equatorial_ray_t<MathLibm>(m, r_obs, alpha);
}

}  // namespace

// ===========================================================================
// exported C API
// ===========================================================================
extern "C" {

int orc_hardware_threads(void) { return resolve_threads(0); }

void orc_geon_sincos(const double* x, int64_t n, double* s, double* c) {
  for (int64_t i = 0; i < n; ++i) geon_sincos(x[i], &s[i], &c[i]);
}
void orc_geon_tanh(const double* x, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = geon_tanh(x[i]);
}
void orc_geon_expm1(const double* x, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = geon_expm1(x[i]);
}
int orc_inv4(const double* m16, double* out16) {
  Mat4 a, o;
  std::memcpy(&a, m16, sizeof a);
  const bool ok = inv4(a, o);
  if (ok) std::memcpy(out16, &o, sizeof o);
  return ok ? 1 : 0;
}

int orc_metric_g(int kind, const double* params, int math, const double* x, int64_t n, double* out) {
  return with_metric(kind, params, math, [&](auto& m) {
    for (int64_t i = 0; i < n; ++i) {
      const Mat4 g = m.g(load4(x + 4 * i));
      std::memcpy(out + 16 * i, &g, sizeof g);
    }
    return 0;
  });
}
int orc_metric_dg(int kind, const double* params, int math, const double* x, int64_t n, double* out) {
  return with_metric(kind, params, math, [&](auto& m) {
    for (int64_t i = 0; i < n; ++i) {
      Mat4 dg[4];
      m.dg(load4(x + 4 * i), dg);
      std::memcpy(out + 64 * i, dg, sizeof dg);
    }
    return 0;
  });
}
int orc_metric_g_inv(int kind, const double* params, int math, const double* x, int64_t n, double* out) {
  return with_metric(kind, params, math, [&](auto& m) {
    g_singular = false;
    for (int64_t i = 0; i < n; ++i) {
      const Mat4 g = m.g_inv(load4(x + 4 * i));
      std::memcpy(out + 16 * i, &g, sizeof g);
    }
    return g_singular ? -2 : 0;
  });
}
int orc_metric_christoffel(int kind, const double* params, int math, const double* x, int64_t n,
                           double* out) {
  return with_metric(kind, params, math, [&](auto& m) {
    g_singular = false;
    for (int64_t i = 0; i < n; ++i) {
      const Chr c = m.christoffel(load4(x + 4 * i));
      std::memcpy(out + 64 * i, &c, sizeof c);
    }
    return g_singular ? -2 : 0;
  });
}
int orc_metric_terminate(int kind, const double* params, int math, const double* x, int64_t n,
                         int32_t* term) {
  return with_metric(kind, params, math, [&](auto& m) {
    for (int64_t i = 0; i < n; ++i) term[i] = m.terminate(load4(x + 4 * i));
    return 0;
  });
}
int orc_asymptotic_direction(int kind, const double* params, int math, const double* xp, int64_t n,
                             double* out) {
  return with_metric(kind, params, math, [&](auto& m) {
    for (int64_t i = 0; i < n; ++i)
      m.asymptotic_direction(load4(xp + 8 * i), load4(xp + 8 * i + 4), out + 3 * i);
    return 0;
  });
}

int orc_trace(int kind, const double* params, int math, const double* y0, int64_t n, double step,
              int64_t max_steps, int nthreads, int32_t* term, double* yfinal, int64_t* steps,
              double* resid) {
  return with_metric(kind, params, math, [&](auto& m) {
    std::atomic<bool> singular(false);
    parallel_for(n, nthreads, [&](int64_t i) {
      g_singular = false;
      State s;
      std::memcpy(s.y, y0 + 8 * i, sizeof s.y);
      const TraceResult r = trace(m, s, step, max_steps);
      if (g_singular) singular = true;
      term[i] = r.term;
      if (yfinal) std::memcpy(yfinal + 8 * i, r.final_state.y, sizeof r.final_state.y);
      if (steps) steps[i] = r.steps;
      if (resid) resid[i] = r.resid;
    });
    return singular ? -2 : 0;
  });
}

int orc_trace_adaptive(int kind, const double* params, int math, const double* y0, int64_t n, double h0,
                       int64_t max_steps, double rtol, double atol, int nthreads, int32_t* term, double* yfinal,
                       int64_t* steps, double* resid) {
  return with_metric(kind, params, math, [&](auto& m) {
    std::atomic<bool> singular(false);
    parallel_for(n, nthreads, [&](int64_t i) {
      g_singular = false;
      State s;
      std::memcpy(s.y, y0 + 8 * i, sizeof s.y);
      const TraceResult r = trace_adaptive(m, s, h0, max_steps, rtol, atol);
      if (g_singular) singular = true;
      term[i] = r.term;
      if (yfinal) std::memcpy(yfinal + 8 * i, r.final_state.y, sizeof r.final_state.y);
      if (steps) steps[i] = r.steps;
      if (resid) resid[i] = r.resid;
    });
    return singular ? -2 : 0;
  });
}

int orc_field_set(const double* lo3, const double* hi3, const int64_t* n3, int chart, const double* samples) {
  int64_t nodes = 1;
  for (int a = 0; a < 3; ++a) {
    if (n3[a] < 1) return -1;
    g_field.lo[a] = lo3[a];
    g_field.hi[a] = hi3[a];
    g_field.n[a] = n3[a];
    g_field.inv_d[a] = n3[a] > 1 ? (double)(n3[a] - 1) / (hi3[a] - lo3[a]) : 0.0;
    nodes *= n3[a];
  }
  g_field.chart = chart;
  g_field.c.assign(samples, samples + 10 * nodes);
  return 0;
}

int orc_camera_tetrad(int kind, const double* params, int math, const double* observer, double* out16) {
  return with_metric(kind, params, math, [&](auto& m) {
    Mat4 tet;
    const int rc = tetrad(m, load4(observer), tet);
    std::memcpy(out16, &tet, sizeof tet);
    return rc;
  });
}

int orc_camera_rays(const double* tetrad16, const double* observer, double fov_y_deg, int64_t width,
                    int64_t height, int64_t row0, int64_t nrows, double du, double dv,
                    int forward_sign, double* y0_out) {
  Mat4 tet;
  std::memcpy(&tet, tetrad16, sizeof tet);
  const double fov = to_radians(fov_y_deg);
  for (int64_t jj = 0; jj < nrows; ++jj)
    for (int64_t i = 0; i < width; ++i) {
      const State s = ray_state_sub(tet, observer, fov, width, height, i, row0 + jj, du, dv, forward_sign);
      std::memcpy(y0_out + 8 * (jj * width + i), s.y, sizeof s.y);
    }
  return 0;
}

void orc_sky_sample(const double* dir3, int64_t n, int show_stars, float* rgb_out) {
  for (int64_t i = 0; i < n; ++i) sky_sample(dir3 + 3 * i, show_stars != 0, rgb_out + 3 * i);
}

// render.rs:169-183 (write_png): `c.clamp(0.0, 1.0).powf(1.0 / 2.2)` in f32,
// then `(v * 255.0).round() as u8` (round half away from zero; the cast
// saturates and maps NaN to 0).
void orc_tonemap_u8(const float* rgb, int64_t n, uint8_t* out) {
  const float gamma_inv = 1.0f / 2.2f;
  for (int64_t i = 0; i < n; ++i) {
    float v = rgb[i];
    if (v < 0.0f) v = 0.0f;
    if (v > 1.0f) v = 1.0f;
    const float p = powf(v, gamma_inv);
    const float y = roundf(p * 255.0f);
    out[i] = !(y > 0.0f) ? 0 : (y >= 255.0f ? 255 : (uint8_t)y);
  }
}

// render.rs:55-166
int orc_render(int kind, const double* params, int math, const double* observer, double fov_y_deg,
               int64_t width, int64_t height, int64_t row0, int64_t nrows, double step,
               int64_t max_steps, int64_t samples_per_axis, int show_stars, int forward_sign,
               int nthreads, float* rgb_out, int32_t* pclass_out, int64_t* psteps_out,
               orc_render_stats* stats) {
  return with_metric(kind, params, math, [&](auto& m) {
    Mat4 tet;
    const int rc = tetrad(m, load4(observer), tet);
    if (rc != 0) return rc;
    const double fov = to_radians(fov_y_deg);
    const int64_t w = width;
    const int64_t npix = w * nrows;
    const int64_t spa = samples_per_axis < 1 ? 1 : samples_per_axis;
    const double inv_spa = 1.0 / (double)spa;
    const float captured_rgb[3] = {0.0f, 0.0f, 0.0f};
    const float diverged_rgb[3] = {1.0f, 0.0f, 1.0f};
    std::vector<int32_t> cls(npix);
    std::vector<int64_t> pst(npix), tot(npix);
    std::vector<double> mres(npix);
    std::atomic<bool> singular(false);
    parallel_for(npix, nthreads, [&](int64_t idx) {
      g_singular = false;
      const int64_t i = idx % w;
      const int64_t j = row0 + idx / w;
      float acc[3] = {0.0f, 0.0f, 0.0f};
      int64_t total_steps_pix = 0;
      double max_resid_pix = 0.0;
      uint32_t nc = 0, ne = 0, nd = 0;
      for (int64_t sj = 0; sj < spa; ++sj)
        for (int64_t si = 0; si < spa; ++si) {
          const double du = ((double)si + 0.5) * inv_spa;
          const double dv = ((double)sj + 0.5) * inv_spa;
          const State y0 = ray_state_sub(tet, observer, fov, width, height, i, j, du, dv, forward_sign);
          const TraceResult res = trace(m, y0, step, max_steps);
          float rgb[3];
          if (res.term == CAPTURED) {
            ++nc;
            std::memcpy(rgb, captured_rgb, sizeof rgb);
          } else if (res.term == DIVERGED) {
            ++nd;
            std::memcpy(rgb, diverged_rgb, sizeof rgb);
          } else {
            ++ne;
            double dir[3];
            m.asymptotic_direction(pos(res.final_state), mom(res.final_state), dir);
            sky_sample(dir, show_stars != 0, rgb);
          }
          acc[0] += rgb[0]; acc[1] += rgb[1]; acc[2] += rgb[2];
          total_steps_pix += res.steps;
          if (std::isfinite(res.resid) && res.resid > max_resid_pix) max_resid_pix = res.resid;
        }
      if (g_singular) singular = true;
      const float nf = (float)(spa * spa);
      rgb_out[3 * idx + 0] = acc[0] / nf;
      rgb_out[3 * idx + 1] = acc[1] / nf;
      rgb_out[3 * idx + 2] = acc[2] / nf;
      int term;
      if (nd > 0 && nd >= nc && nd >= ne) term = DIVERGED;
      else if (nc >= ne) term = CAPTURED;
      else term = ESCAPED;
      cls[idx] = term;
      pst[idx] = total_steps_pix / (spa * spa);
      tot[idx] = total_steps_pix;
      mres[idx] = max_resid_pix;
    });
    orc_render_stats st{0, 0, 0, 0.0, 0.0, 0};
    int64_t total_steps = 0;
    for (int64_t idx = 0; idx < npix; ++idx) {
      if (cls[idx] == CAPTURED) ++st.captured;
      else if (cls[idx] == ESCAPED) ++st.escaped;
      else ++st.diverged;
      total_steps += pst[idx];
      st.total_steps += tot[idx];
      if (mres[idx] > st.max_null_residual) st.max_null_residual = mres[idx];
      if (pclass_out) pclass_out[idx] = cls[idx];
      if (psteps_out) psteps_out[idx] = pst[idx];
    }
    st.avg_steps = (double)total_steps / (double)npix;
    if (stats) *stats = st;
    return singular ? -2 : 0;
  });
}

int orc_curvature(int kind, const double* params, int math, const double* x, int64_t n, int what,
                  int faithful, int nthreads, double* out) {
  return with_metric(kind, params, math, [&](auto& m) {
    std::atomic<bool> singular(false);
    parallel_for(n, nthreads, [&](int64_t i) {
      g_singular = false;
      const Vec4 xi = load4(x + 4 * i);
      Riemann riem;
      Mat4 ric, ein, t;
      double rs;
      curvature_point(m, xi, faithful, what == 0 ? &riem : nullptr, ric, rs, ein, t);
      if (g_singular) singular = true;
      switch (what) {
        case 0: std::memcpy(out + 256 * i, &riem, sizeof riem); break;
        case 1: std::memcpy(out + 16 * i, &ric, sizeof ric); break;
        case 2: out[i] = rs; break;
        case 3: std::memcpy(out + 16 * i, &ein, sizeof ein); break;
        default: std::memcpy(out + 16 * i, &t, sizeof t); break;
      }
    });
    return singular ? -2 : 0;
  });
}

int orc_nec(int kind, const double* params, int math, const double* x, int64_t n, const double* k,
            int64_t nk, int k_shared, int faithful, int nthreads, double* out) {
  return with_metric(kind, params, math, [&](auto& m) {
    std::atomic<bool> singular(false);
    parallel_for(n, nthreads, [&](int64_t i) {
      g_singular = false;
      const Vec4 xi = load4(x + 4 * i);
      Mat4 ric, ein, t;
      double rs;
      if (!faithful) curvature_point(m, xi, 0, nullptr, ric, rs, ein, t);
      for (int64_t q = 0; q < nk; ++q) {
        // The reference recomputes stress_energy for every k (curvature.rs:127-136).
        if (faithful) curvature_point(m, xi, 1, nullptr, ric, rs, ein, t);
        const double* kp = k_shared ? k + 4 * q : k + 4 * (i * nk + q);
        out[i * nk + q] = nec_from(t, load4(kp));
      }
      if (g_singular) singular = true;
    });
    return singular ? -2 : 0;
  });
}

void orc_equatorial_ray(double mass, double r_obs, int math, const double* alpha, int64_t n,
                        double* y0_out) {
  for (int64_t i = 0; i < n; ++i) {
    const State s = equatorial_ray(mass, r_obs, math, alpha[i]);
    std::memcpy(y0_out + 8 * i, s.y, sizeof s.y);
  }
}

int orc_shadow_classify(const double* schw_params, double r_obs, int math, const double* alpha,
                        int64_t n, double step, int64_t max_steps, int nthreads, int32_t* term_out,
                        int64_t* steps_out) {
  return with_schw(schw_params, math, [&](auto& m) {
    parallel_for(n, nthreads, [&](int64_t i) {
      const State y0 = equatorial_ray(m.mass, r_obs, math, alpha[i]);
      const TraceResult r = trace(m, y0, step, max_steps);
      term_out[i] = r.term;
      if (steps_out) steps_out[i] = r.steps;
    });
    return 0;
  });
}

// bin/validate_shadow.rs:70-79 (bisection loop) for nb independent brackets.
int orc_shadow_bisect(const double* schw_params, double r_obs, int math, const double* lo_in,
                      const double* hi_in, int64_t nb, int iters, double step, int64_t max_steps,
                      int nthreads, double* alpha_c_out, double* lo_out, double* hi_out,
                      int64_t* steps_out) {
  return with_schw(schw_params, math, [&](auto& m) {
    parallel_for(nb, nthreads, [&](int64_t b) {
      double lo = lo_in[b], hi = hi_in[b];
      int64_t st = 0;
      for (int it = 0; it < iters; ++it) {
        const double mid = 0.5 * (lo + hi);
        const State y0 = equatorial_ray(m.mass, r_obs, math, mid);
        const TraceResult r = trace(m, y0, step, max_steps);
        st += r.steps;
        if (r.term == CAPTURED) lo = mid;
        else hi = mid;
      }
      alpha_c_out[b] = 0.5 * (lo + hi);
      if (lo_out) lo_out[b] = lo;
      if (hi_out) hi_out[b] = hi;
      if (steps_out) steps_out[b] = st;
    });
    return 0;
  });
}

// bin/energy_conditions.rs:37-156
int orc_energy_conditions(int math, double* out) {
  int w = 0;
  auto nec1 = [&](int kind, const double* p, const double* x, const double* k) {
    double v = 0.0;
    orc_nec(kind, p, math, x, 1, k, 1, 1, 1, 1, &v);
    return v;
  };
  auto rs1 = [&](int kind, const double* p, const double* x) {
    double v = 0.0;
    orc_curvature(kind, p, math, x, 1, 2, 1, 1, &v);
    return v;
  };
  {  // Minkowski (:38-48)
    const double p[4] = {0, 0, 0, 0};
    const double x[4] = {0.0, 1.0, 1.0, 1.0};
    const double k[4] = {1.0, 1.0, 0.0, 0.0};
    out[w++] = nec1(0, p, x, k);
    out[w++] = rs1(0, p, x);
  }
  {  // Schwarzschild (:50-67)
    const double p[4] = {1.0, 1.001, 1000.0, 0.0};
    const double rs[3] = {5.0, 10.0, 30.0};
    for (double r : rs) {
      const double x[4] = {0.0, r, FRAC_PI_2, 0.0};
      const double f = 1.0 - 2.0 / r;
      const double k[4] = {1.0 / std::sqrt(f), -std::sqrt(f), 0.0, 0.0};
      out[w++] = nec1(1, p, x, k);
      out[w++] = rs1(1, p, x);
    }
  }
  {  // Alcubierre (:69-121)
    const double p[4] = {2.0, 0.5, 2.0, 0.0};
    const double k[4] = {1.0, 1.0, 0.0, 0.0};
    double min_val = INFINITY, min_x = 0.0;
    for (int n = 0; n < 41; ++n) {
      const double x_pos = -4.0 + 0.2 * (double)n;
      const double x[4] = {0.0, x_pos, 0.0, 0.0};
      const double nec = nec1(2, p, x, k);
      if (nec < min_val) { min_val = nec; min_x = x_pos; }
      out[w++] = nec;
    }
    out[w++] = min_val;
    out[w++] = min_x;
    double integral = 0.0;
    const double dx = 0.05;
    double x_pos = -5.0;
    while (x_pos <= 5.0) {
      const double x[4] = {0.0, x_pos, 0.0, 0.0};
      const double nec = nec1(2, p, x, k);
      if (nec < 0.0) integral += nec * dx;
      x_pos += dx;
    }
    out[w++] = integral;
  }
  {  // Morris-Thorne (:123-156)
    const double p[4] = {1.0, 0, 0, 0};
    const double k[4] = {1.0, 1.0, 0.0, 0.0};
    double min_val = INFINITY, min_l = 0.0;
    for (int n = 0; n < 41; ++n) {
      const double l = -4.0 + 0.2 * (double)n;
      const double x[4] = {0.0, l, FRAC_PI_2, 0.0};
      const double nec = nec1(3, p, x, k);
      if (nec < min_val) { min_val = nec; min_l = l; }
      out[w++] = nec;
    }
    out[w++] = min_val;
    out[w++] = min_l;
    const double xt[4] = {0.0, 0.0, FRAC_PI_2, 0.0};
    double t[16];
    orc_curvature(3, p, math, xt, 1, 4, 1, 1, t);
    for (int i = 0; i < 4; ++i) out[w++] = t[5 * i];
  }
  return w;
}

}  // extern "C"
