// Closed-form geodesic right-hand sides for the mixed-precision path.
//
// The reference differentiates g numerically for Alcubierre and Morris-Thorne
// (metric/mod.rs:25-69, central differences with h = 1e-5). In FP32 that
// difference is pure rounding noise (eps/h ~ 1e-2), so the mixed path uses the
// Christoffel symbols in closed form, derived from the same metric functions:
//
//  Schwarzschild (t, r, th, ph), f = 1 - 2m/r, A = m/r^2:
//    Gamma^t_tr = A/f, Gamma^r_tt = A f, Gamma^r_rr = -A/f, Gamma^r_thth = -(r - 2m),
//    Gamma^r_phph = -(r - 2m) sin^2, Gamma^th_rth = Gamma^ph_rph = 1/r,
//    Gamma^th_phph = -sin cos, Gamma^ph_thph = cot             (schwarzschild.rs:61-107)
//  Morris-Thorne (t, l, th, ph), r2 = b0^2 + l^2 (morris_thorne.rs:22-36):
//    Gamma^l_thth = -l, Gamma^l_phph = -l sin^2, Gamma^th_lth = Gamma^ph_lph = l/r2,
//    Gamma^th_phph = -sin cos, Gamma^ph_thph = cot
//  Alcubierre (t, x, y, z), g_tt = -1 + v^2 f^2, g_tx = -v f (alcubierre.rs:48-63):
//    with A_i = d_i g_tt = 2 v^2 f f_i and B_i = d_i g_tx = -v f_i,
//    Q_t = p^t (A.p) + (B.p) p^x, Q_i = -A_i (p^t)^2 / 2 + p^t (delta_ix (B.p) - B_i p^x),
//    dp^t = Q_t + v f Q_x, dp^x = v f Q_t - (1 - v^2 f^2) Q_x, dp^y = -Q_y, dp^z = -Q_z
//    (g^tt = -1, g^tx = -v f, g^xx = 1 - v^2 f^2), f_i = f'(r_s) (x^i - x_s^i) / r_s,
//    f'(r_s) = (tanh^2((r_s - R)/s) - tanh^2((r_s + R)/s)) / (2 s tanh(R/s)).
//
// The FP32 step evaluates each stage at the high words plus the stage
// increment (the low words are below the FP32 evaluation error), except the
// polar angle, which keeps its low word: angles use sin/cos of the base once per
// step and the angle-addition formula per stage, so theta keeps its compensated
// precision near the equator (cos theta ~ 1e-8 there).
#pragma once
#include "internal.h"

namespace geon {

template <typename T>
struct AMath;

template <>
struct AMath<float> {
  static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
  // approximate reciprocal (one MUFU op, ~1 ulp): the RHS tolerates FP32 error
  static __device__ __forceinline__ float rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  static __device__ __forceinline__ float div(float a, float b) { return a * rcp(b); }
  // approximate square root (one MUFU op, relative error below 2^-23; 0 at 0):
  // the RHS tolerates FP32 error
  static __device__ __forceinline__ float sqrt(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
  // tanh(x) = sign(x) (1 - 2 / (e^{2|x|} + 1)) with the hardware exponential
  // and reciprocal (two MUFU ops): absolute error ~2e-7, which is what the
  // Alcubierre RHS needs (it uses differences of tanh values near +-1). Large
  // |x| gives e = inf and exactly +-1.
  static __device__ __forceinline__ float tanh(float x) {
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(fabsf(x) * 2.8853900817779268f));  // 2 / ln 2
    return copysignf(__fmaf_rn(-2.0f, rcp(e + 1.0f), 1.0f), x);
  }
  static __device__ __forceinline__ void sincos(float x, float* s, float* c) { sincosf(x, s, c); }
};

template <>
struct AMath<double> {
  static __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ double rcp(double x) { return 1.0 / x; }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
  static __device__ __forceinline__ double tanh(double x) { return ::tanh(x); }
  static __device__ __forceinline__ void sincos(double x, double* s, double* c) { ::sincos(x, s, c); }
};

// Metric constants in the working precision.
template <typename T>
struct AConsts {
  T m, two_m;          // Schwarzschild
  T b0sq;              // Morris-Thorne
  T R, inv_s, v, ship_x, fnorm, dfnorm;  // Alcubierre: fnorm = 1/(2 tanh(R/s)), dfnorm = fnorm/s
  __device__ __forceinline__ void init(const MetricDesc& M) {
    m = (T)M.p[0];
    two_m = (T)(2.0 * M.p[0]);
    b0sq = (T)(M.p[0] * M.p[0]);
    R = (T)M.p[0];
    inv_s = (T)(1.0 / M.p[1]);
    v = (T)M.p[2];
    ship_x = (T)M.p[3];
    const double dn = M.kind == KIND_ALCUBIERRE ? M.alc_denom : 1.0;  // 2 tanh(R/s)
    fnorm = (T)(1.0 / dn);
    dfnorm = (T)(1.0 / (dn * M.p[1]));
  }
};

// sin/cos of (base angle + d) from sin/cos of the base: d is a stage offset.
template <typename T>
__device__ __forceinline__ void angle_add(T s0, T c0, T base, T d, T* s, T* c) {
  using Mt = AMath<T>;
  const T ad = d < (T)0 ? -d : d;
  if (ad < (T)0.03) {
    const T d2 = d * d;
    const T sd = d * Mt::fma(d2, (T)(-1.0 / 6.0), (T)1);       // sin d to d^3
    const T cd = Mt::fma(d2, Mt::fma(d2, (T)(1.0 / 24.0), (T)(-0.5)), (T)1);  // cos d to d^4
    *s = Mt::fma(s0, cd, c0 * sd);
    *c = Mt::fma(c0, cd, -(s0 * sd));
  } else {
    Mt::sincos(base + d, s, c);
  }
}

// k = (p, dp/dlambda) at the point xb + d.
// k = (p, dp/dlambda) at one stage point given directly: the position x1 (r,
// l or x), x2 and x3 (y, z: Alcubierre only), the polar angle as th_base + dth
// (Schwarzschild, Morris-Thorne: sin/cos of th_base are s0, c0) and the
// momentum p. Unused arguments cost nothing (the compiler drops them).
template <int K, typename T>
__device__ __forceinline__ void rhs_stage(const AConsts<T>& C, T x1, T x2, T x3, T th_base, T dth, const T p[4],
                                          T s0, T c0, T k[8]) {
  using Mt = AMath<T>;
  const T p0 = p[0], p1 = p[1], p2 = p[2], p3 = p[3];
  k[0] = p0; k[1] = p1; k[2] = p2; k[3] = p3;
  if (K == KIND_MINKOWSKI) {
    k[4] = (T)0; k[5] = (T)0; k[6] = (T)0; k[7] = (T)0;
  } else if (K == KIND_SCHWARZSCHILD || K == KIND_MORRIS_THORNE) {
    T s, c;
    angle_add<T>(s0, c0, th_base, dth, &s, &c);
    const T as = s < (T)0 ? -s : s;
    const T cot = as < (T)1e-8 ? (T)0 : Mt::div(c, s);
    const T p3sq = p3 * p3;
    const T th_term = s * c * p3sq;                                  // -Gamma^th_phph p^ph p^ph
    const T ang = Mt::fma(s * s, p3sq, p2 * p2);                    // (p^th)^2 + sin^2 (p^ph)^2
    if (K == KIND_SCHWARZSCHILD) {
      const T r = x1;
      const T ir = Mt::rcp(r);
      const T f = Mt::fma(-C.two_m, ir, (T)1);
      const T A = C.m * ir * ir;
      const T gtr = Mt::div(A, f);
      k[4] = (T)(-2) * gtr * p0 * p1;
      k[5] = Mt::fma(-A * f, p0 * p0, Mt::fma(gtr, p1 * p1, (r - C.two_m) * ang));
      k[6] = Mt::fma((T)(-2) * ir * p1, p2, th_term);
      k[7] = (T)(-2) * p3 * Mt::fma(ir, p1, cot * p2);
    } else {
      const T l = x1;
      const T r2 = Mt::fma(l, l, C.b0sq);
      const T q = Mt::div(l, r2);
      k[4] = (T)0;
      k[5] = l * ang;
      k[6] = Mt::fma((T)(-2) * q * p1, p2, th_term);
      k[7] = (T)(-2) * p3 * Mt::fma(q, p1, cot * p2);
    }
  } else {  // Alcubierre
    const T X = x1 - C.ship_x, Y = x2, Z = x3;
    const T rs = Mt::sqrt(Mt::fma(X, X, Mt::fma(Y, Y, Z * Z)));
    const T tp = Mt::tanh((rs + C.R) * C.inv_s);
    const T tm = Mt::tanh((rs - C.R) * C.inv_s);
    const T f = (tp - tm) * C.fnorm;
    const T fp = (tm - tp) * (tm + tp) * C.dfnorm;  // f'(r_s)
    const T g = rs > (T)1e-30 ? Mt::div(fp, rs) : (T)0;
    const T fx = g * X, fy = g * Y, fz = g * Z;
    const T vf = C.v * f;
    const T a2 = (T)2 * C.v * vf;                   // A_i = a2 f_i
    const T mv = -C.v;                              // B_i = mv f_i
    const T fdotp = Mt::fma(fx, p1, Mt::fma(fy, p2, fz * p3));
    const T Ap = a2 * fdotp, Bp = mv * fdotp;
    const T Qt = Mt::fma(p0, Ap, Bp * p1);
    const T hp0sq = (T)0.5 * p0 * p0;
    const T Qx = Mt::fma(-a2 * fx, hp0sq, p0 * (Bp - mv * fx * p1));
    const T Qy = Mt::fma(-a2 * fy, hp0sq, -p0 * mv * fy * p1);
    const T Qz = Mt::fma(-a2 * fz, hp0sq, -p0 * mv * fz * p1);
    k[4] = Mt::fma(vf, Qx, Qt);
    k[5] = Mt::fma(vf, Qt, -Mt::fma(-vf, vf, (T)1) * Qx);
    k[6] = -Qy;
    k[7] = -Qz;
  }
}

// k at the point xb + d (xb the state at the start of the step, d the stage
// offset, which carries the low words).
template <int K, typename T>
__device__ __forceinline__ void rhs_analytic(const AConsts<T>& C, const T xb[8], const T d[8], T s0, T c0,
                                             T k[8]) {
  const T p[4] = {xb[4] + d[4], xb[5] + d[5], xb[6] + d[6], xb[7] + d[7]};
  rhs_stage<K, T>(C, xb[1] + d[1], xb[2] + d[2], xb[3] + d[3], xb[2], d[2], p, s0, c0, k);
}

// Null re-projection: solve g(p, p) = 0 for p^t at the point x, keeping the
// spatial momentum and the sign of p^t. Returns the new p^t.
template <int K, typename T>
__device__ __forceinline__ T null_pt(const AConsts<T>& C, const T x[4], const T p[4], T s, T pt_now) {
  using Mt = AMath<T>;
  T pt;
  if (K == KIND_MINKOWSKI) {
    pt = Mt::sqrt(Mt::fma(p[1], p[1], Mt::fma(p[2], p[2], p[3] * p[3])));
  } else if (K == KIND_SCHWARZSCHILD) {
    const T r = x[1];
    const T f = Mt::fma(-C.two_m, Mt::rcp(r), (T)1);
    const T sp = Mt::fma(r * r, Mt::fma(s * s, p[3] * p[3], p[2] * p[2]), Mt::div(p[1] * p[1], f));
    pt = Mt::sqrt(Mt::div(sp, f));
  } else if (K == KIND_MORRIS_THORNE) {
    const T r2 = Mt::fma(x[1], x[1], C.b0sq);
    pt = Mt::sqrt(Mt::fma(r2, Mt::fma(s * s, p[3] * p[3], p[2] * p[2]), p[1] * p[1]));
  } else {
    const T X = x[1] - C.ship_x, Y = x[2], Z = x[3];
    const T rs = Mt::sqrt(Mt::fma(X, X, Mt::fma(Y, Y, Z * Z)));
    const T f = (Mt::tanh((rs + C.R) * C.inv_s) - Mt::tanh((rs - C.R) * C.inv_s)) * C.fnorm;
    const T vf = C.v * f;
    const T a = Mt::fma(vf, vf, (T)(-1));       // g_tt
    const T b = -vf * p[1];                     // g_tx p^x
    const T c = Mt::fma(p[1], p[1], Mt::fma(p[2], p[2], p[3] * p[3]));
    const T disc = Mt::fma(b, b, -a * c);
    if (!(disc >= (T)0) || a == (T)0) return pt_now;
    const T sq = Mt::sqrt(disc);
    const T r1 = Mt::div(-b + sq, a), r2v = Mt::div(-b - sq, a);
    const T e1 = r1 - pt_now, e2 = r2v - pt_now;
    return (e1 < (T)0 ? -e1 : e1) <= (e2 < (T)0 ? -e2 : e2) ? r1 : r2v;
  }
  return pt_now < (T)0 ? -pt : pt;
}

// Is the point inside the metric's FP64 band (photon sphere / horizon /
// throat / bubble wall), where the mixed path integrates in FP64?
template <int K>
__device__ __forceinline__ bool in_band(const MetricDesc& M, float x1, float x2, float x3, float band) {
  if (K == KIND_SCHWARZSCHILD) return x1 < band * (float)M.p[0];
  if (K == KIND_MORRIS_THORNE) return fabsf(x1) < band * (float)M.p[0];
  if (K == KIND_ALCUBIERRE) {
    const float X = x1 - (float)M.p[3];
    const float rs = sqrtf(X * X + x2 * x2 + x3 * x3);
    return fabsf(rs - (float)M.p[0]) < band * (float)M.p[1];
  }
  return false;
}

}  // namespace geon
