// FP64 device functors for the four metrics: g, g^-1, Christoffel symbols, the
// geodesic right-hand side, termination and the escape direction.
//
// Parity contract: with --fmad=false and the deterministic sin/cos/tanh of
// devmath.cuh, every function here returns the bits the reference's Rust code
// returns for the same inputs (the CPU oracle in oracle/ checks this). Rules
// that keep it so:
//  * operations appear in the reference's order, sums left-associated;
//  * a term of an accumulation that starts at +0.0 (all of the reference's sums
//    do) may be skipped when it is exactly zero: x + (+-0) == x for x != 0, and
//    such a sum can never become -0, so the sign of a skipped zero is
//    irrelevant. The sparse functors below use only this and exact identities
//    (x * 1.0 == x, -(a/b) == (-a)/b, 2.0 * x exact).
#pragma once
#include "devmath.cuh"
#include "internal.h"

namespace geon {

constexpr double FD_H = 1e-5;  // Metric::fd_step default (metric/mod.rs:73-75)

// x + 0.0 (the first addition of a sum that starts at +0.0) without spending an
// FP64 instruction: only -0.0 changes (to +0.0).
__device__ __forceinline__ double plus_zero(double x) {
  const long long b = __double_as_longlong(x);
  return b == (long long)0x8000000000000000ULL ? 0.0 : x;
}

// types.rs:22-30
__device__ __forceinline__ double dot4(const double g[16], const double a[4], const double b[4]) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) s += g[4 * i + j] * a[i] * b[j];
  return s;
}

// Stand-in for nalgebra's Matrix4::try_inverse (types.rs:34-47): adjugate by 2x2
// minors (Laplace expansion; D. Eberly, Geometric Tools 2008). The CPU oracle
// uses the identical sequence. Returns false when det == 0.
__device__ __forceinline__ bool inv4(const double a[16], double out[16]) {
  const double a00 = a[0], a01 = a[1], a02 = a[2], a03 = a[3];
  const double a10 = a[4], a11 = a[5], a12 = a[6], a13 = a[7];
  const double a20 = a[8], a21 = a[9], a22 = a[10], a23 = a[11];
  const double a30 = a[12], a31 = a[13], a32 = a[14], a33 = a[15];
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
  const bool ok = det != 0.0;
  const double id = 1.0 / det;
  out[0] = (a11 * c5 - a12 * c4 + a13 * c3) * id;
  out[1] = (-a01 * c5 + a02 * c4 - a03 * c3) * id;
  out[2] = (a31 * s5 - a32 * s4 + a33 * s3) * id;
  out[3] = (-a21 * s5 + a22 * s4 - a23 * s3) * id;
  out[4] = (-a10 * c5 + a12 * c2 - a13 * c1) * id;
  out[5] = (a00 * c5 - a02 * c2 + a03 * c1) * id;
  out[6] = (-a30 * s5 + a32 * s2 - a33 * s1) * id;
  out[7] = (a20 * s5 - a22 * s2 + a23 * s1) * id;
  out[8] = (a10 * c4 - a11 * c2 + a13 * c0) * id;
  out[9] = (-a00 * c4 + a01 * c2 - a03 * c0) * id;
  out[10] = (a30 * s4 - a31 * s2 + a33 * s0) * id;
  out[11] = (-a20 * s4 + a21 * s2 - a23 * s0) * id;
  out[12] = (-a10 * c3 + a11 * c1 - a12 * c0) * id;
  out[13] = (a00 * c3 - a01 * c1 + a02 * c0) * id;
  out[14] = (-a30 * s3 + a31 * s1 - a32 * s0) * id;
  out[15] = (a20 * s3 - a21 * s1 + a22 * s0) * id;
  if (!ok) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
#pragma unroll
    for (int i = 0; i < 16; ++i) out[i] = nan;
  }
  return ok;
}

// ---------------------------------------------------------------------------
// The varying entries of g for the metrics whose Christoffel symbols use the
// finite-difference fallback. metric_g and the sparse Christoffel code both
// call these, so both see the same bits.
// ---------------------------------------------------------------------------
// alcubierre.rs:33-63: g_tt = -1 + v^2 f^2, g_tx = g_xt = -v f
__device__ __forceinline__ void alc_g00_g01(const MetricDesc& M, const double x[4], double* g00, double* g01) {
  const double R = M.p[0], s = M.p[1], v = M.p[2], ship_x = M.p[3];
  const double dx = x[1] - ship_x, dy = x[2], dz = x[3];
  const double r_s = sqrt(dx * dx + dy * dy + dz * dz);
  const double t_plus = dm::tanh_det((r_s + R) / s);
  const double t_minus = dm::tanh_det((r_s - R) / s);
  const double f = (t_plus - t_minus) / M.alc_denom;
  *g00 = -1.0 + v * v * f * f;
  *g01 = -v * f;
}

// morris_thorne.rs:22-36: g_thth = b0^2 + l^2, g_phph = (b0^2 + l^2) sin^2(theta)
__device__ __forceinline__ void mt_g22_g33(const MetricDesc& M, const double x[4], double* g22, double* g33) {
  const double l = x[1], theta = x[2], b0 = M.p[0];
  const double r2 = b0 * b0 + l * l;
  double sin_t, cos_t;
  dm::sincos_det(theta, &sin_t, &cos_t);
  *g22 = r2;
  *g33 = r2 * sin_t * sin_t;
}

// ---------------------------------------------------------------------------
// g(x) for each metric (dense 4x4, row-major)
// ---------------------------------------------------------------------------
// Sampled metric (GEON_FIELD): uniform cubic B-spline weights of the local
// coordinate t in [0, 1) and the first of the four node indices along one axis
// (nodes beyond an edge repeat the edge node). Everything here is fully
// unrolled so that no array of the evaluation lives in local memory.
struct FieldAxis {
  int64_t i0, i1, i2, i3;
  double w0, w1, w2, w3;
};

__device__ __forceinline__ int64_t field_clamp(int64_t j, int64_t n) { return j < 0 ? 0 : (j > n - 1 ? n - 1 : j); }

__device__ __forceinline__ FieldAxis field_axis(double lo, double inv_d, int64_t n, double x) {
  const double u = (x - lo) * inv_d;
  const double fl = floor(u);
  const double t = u - fl;
  const double fc = fmin(fmax(fl, -2.0), (double)n + 1.0);  // NaN -> -2: g becomes NaN through t
  const int64_t i = (int64_t)fc;
  const double sixth = 1.0 / 6.0;
  const double t2 = t * t, t3 = t2 * t, s = 1.0 - t;
  FieldAxis A;
  A.w0 = ((s * s) * s) * sixth;
  A.w1 = ((3.0 * t3 - 6.0 * t2) + 4.0) * sixth;
  A.w2 = (((-3.0 * t3 + 3.0 * t2) + 3.0 * t) + 1.0) * sixth;
  A.w3 = t3 * sixth;
  A.i0 = field_clamp(i - 1, n);
  A.i1 = field_clamp(i, n);
  A.i2 = field_clamp(i + 1, n);
  A.i3 = field_clamp(i + 2, n);
  return A;
}

// acc[q] = acc[q] + w * s[q] over the 10 components of one node
__device__ __forceinline__ void field_madd(double acc[10], double w, const double* __restrict__ s) {
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = acc[q] + w * __ldg(s + q);
}

// One row along x: the 4 nodes of (j, k), weighted by the x weights.
__device__ __forceinline__ void field_row(const FieldDesc& F, const FieldAxis& X, int64_t j, int64_t k,
                                          double out[10]) {
#pragma unroll
  for (int q = 0; q < 10; ++q) out[q] = 0.0;
  const int64_t row = F.n[0] * (j + F.n[1] * k);
  field_madd(out, X.w0, F.c + 10 * (X.i0 + row));
  field_madd(out, X.w1, F.c + 10 * (X.i1 + row));
  field_madd(out, X.w2, F.c + 10 * (X.i2 + row));
  field_madd(out, X.w3, F.c + 10 * (X.i3 + row));
}

// One plane along y at slice k: 4 rows weighted by the y weights.
__device__ __forceinline__ void field_plane(const FieldDesc& F, const FieldAxis& X, const FieldAxis& Y, int64_t k,
                                            double out[10]) {
#pragma unroll
  for (int q = 0; q < 10; ++q) out[q] = 0.0;
  double r[10];
  field_row(F, X, Y.i0, k, r);
#pragma unroll
  for (int q = 0; q < 10; ++q) out[q] = out[q] + Y.w0 * r[q];
  field_row(F, X, Y.i1, k, r);
#pragma unroll
  for (int q = 0; q < 10; ++q) out[q] = out[q] + Y.w1 * r[q];
  field_row(F, X, Y.i2, k, r);
#pragma unroll
  for (int q = 0; q < 10; ++q) out[q] = out[q] + Y.w2 * r[q];
  field_row(F, X, Y.i3, k, r);
#pragma unroll
  for (int q = 0; q < 10; ++q) out[q] = out[q] + Y.w3 * r[q];
}

// g at x: the B-spline sum over the 4x4x4 neighbouring nodes, separable (x,
// then y, then z), for the 10 unique components (00 01 02 03 11 12 13 22 23 33).
// Not inlined: the finite-difference chain calls it 6 times per Christoffel
// evaluation, and one copy of its 640 multiply-adds per kernel is enough.
static __device__ __noinline__ void field_g(const FieldDesc& F, const double x[4], double g[16]) {
  const FieldAxis X = field_axis(F.lo[0], F.inv_d[0], F.n[0], x[1]);
  const FieldAxis Y = field_axis(F.lo[1], F.inv_d[1], F.n[1], x[2]);
  const FieldAxis Z = field_axis(F.lo[2], F.inv_d[2], F.n[2], x[3]);
  double acc[10], pl[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = 0.0;
  field_plane(F, X, Y, Z.i0, pl);
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = acc[q] + Z.w0 * pl[q];
  field_plane(F, X, Y, Z.i1, pl);
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = acc[q] + Z.w1 * pl[q];
  field_plane(F, X, Y, Z.i2, pl);
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = acc[q] + Z.w2 * pl[q];
  field_plane(F, X, Y, Z.i3, pl);
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = acc[q] + Z.w3 * pl[q];
  g[0] = acc[0]; g[1] = acc[1]; g[2] = acc[2]; g[3] = acc[3];
  g[4] = acc[1]; g[5] = acc[4]; g[6] = acc[5]; g[7] = acc[6];
  g[8] = acc[2]; g[9] = acc[5]; g[10] = acc[7]; g[11] = acc[8];
  g[12] = acc[3]; g[13] = acc[6]; g[14] = acc[8]; g[15] = acc[9];
}

template <int K>
__device__ __forceinline__ void metric_g(const MetricDesc& M, const double x[4], double g[16]) {
  if (K == KIND_FIELD) {
    field_g(M.f, x, g);
    return;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) g[i] = 0.0;
  if (K == KIND_MINKOWSKI) {  // minkowski.rs:11-18
    g[0] = -1.0; g[5] = 1.0; g[10] = 1.0; g[15] = 1.0;
  } else if (K == KIND_SCHWARZSCHILD) {  // schwarzschild.rs:33-45
    const double r = x[1], theta = x[2], m = M.p[0];
    const double f = 1.0 - 2.0 * m / r;
    double sin_t, cos_t;
    dm::sincos_det(theta, &sin_t, &cos_t);
    g[0] = -f;
    g[5] = 1.0 / f;
    g[10] = r * r;
    g[15] = r * r * sin_t * sin_t;
  } else if (K == KIND_ALCUBIERRE) {  // alcubierre.rs:33-63
    double g00, g01;
    alc_g00_g01(M, x, &g00, &g01);
    g[0] = g00;
    g[1] = g01;
    g[4] = g01;
    g[5] = 1.0;
    g[10] = 1.0;
    g[15] = 1.0;
  } else {  // morris_thorne.rs:22-36
    double g22, g33;
    mt_g22_g33(M, x, &g22, &g33);
    g[0] = -1.0;
    g[5] = 1.0;
    g[10] = g22;
    g[15] = g33;
  }
}

// g^-1: overrides for Minkowski and Schwarzschild, inv4(g) otherwise (mod.rs:46-48).
template <int K>
__device__ __forceinline__ bool metric_g_inv(const MetricDesc& M, const double x[4], double gi[16]) {
  if (K == KIND_MINKOWSKI) {
    metric_g<K>(M, x, gi);
    return true;
  } else if (K == KIND_SCHWARZSCHILD) {  // schwarzschild.rs:47-59
#pragma unroll
    for (int i = 0; i < 16; ++i) gi[i] = 0.0;
    const double r = x[1], theta = x[2], m = M.p[0];
    const double f = 1.0 - 2.0 * m / r;
    double sin_t, cos_t;
    dm::sincos_det(theta, &sin_t, &cos_t);
    gi[0] = -1.0 / f;
    gi[5] = f;
    gi[10] = 1.0 / (r * r);
    gi[15] = 1.0 / (r * r * sin_t * sin_t);
    return true;
  } else {
    double g[16];
    metric_g<K>(M, x, g);
    return inv4(g, gi);
  }
}

// g^-1 for a point whose g is already at hand: the same values as
// metric_g_inv (the default inverts g(x), which is g; the overrides ignore it).
template <int K>
__device__ __forceinline__ bool metric_g_inv_given(const MetricDesc& M, const double x[4], const double g[16],
                                                   double gi[16]) {
  if (K == KIND_MINKOWSKI || K == KIND_SCHWARZSCHILD) return metric_g_inv<K>(M, x, gi);
  return inv4(g, gi);
}

// Default dg: central differences with (gp - gm) / two_h (mod.rs:25-43).
template <int K>
__device__ __forceinline__ void metric_dg_fd(const MetricDesc& M, const double x[4], double dg[64]) {
#pragma unroll 1
  for (int alpha = 0; alpha < 4; ++alpha) {
    double xp[4] = {x[0], x[1], x[2], x[3]};
    double xm[4] = {x[0], x[1], x[2], x[3]};
    xp[alpha] += FD_H;
    xm[alpha] -= FD_H;
    double gp[16], gm[16];
    metric_g<K>(M, xp, gp);
    metric_g<K>(M, xm, gm);
    const double two_h = 2.0 * FD_H;
#pragma unroll
    for (int i = 0; i < 16; ++i) dg[16 * alpha + i] = (gp[i] - gm[i]) / two_h;
  }
}

template <int K>
__device__ __forceinline__ void metric_dg(const MetricDesc& M, const double x[4], double dg[64]) {
  if (K == KIND_MINKOWSKI) {
#pragma unroll
    for (int i = 0; i < 64; ++i) dg[i] = 0.0;
  } else if (K == KIND_FIELD) {
    // The field does not depend on t: the t difference is g - g = +0 exactly
    // (for finite g), so only the three spatial differences are evaluated.
#pragma unroll
    for (int alpha = 1; alpha < 4; ++alpha) {
      double xp[4] = {x[0], x[1], x[2], x[3]};
      double xm[4] = {x[0], x[1], x[2], x[3]};
      xp[alpha] += FD_H;
      xm[alpha] -= FD_H;
      double gp[16], gm[16];
      field_g(M.f, xp, gp);
      field_g(M.f, xm, gm);
      const double two_h = 2.0 * FD_H;
#pragma unroll
      for (int i = 0; i < 16; ++i) dg[16 * alpha + i] = (gp[i] - gm[i]) / two_h;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) dg[i] = 0.0;
  } else {
    metric_dg_fd<K>(M, x, dg);
  }
}

// Schwarzschild analytic Christoffel symbols (schwarzschild.rs:61-107).
__device__ __forceinline__ void christoffel_schw(const MetricDesc& M, const double x[4], double G[64]) {
#pragma unroll
  for (int i = 0; i < 64; ++i) G[i] = 0.0;
  const double r = x[1], theta = x[2], m = M.p[0];
  const double f = 1.0 - 2.0 * m / r;
  double sin_t, cos_t;
  dm::sincos_det(theta, &sin_t, &cos_t);
  const double gtr = m / (r * r * f);
  G[0 * 16 + 0 * 4 + 1] = gtr;
  G[0 * 16 + 1 * 4 + 0] = gtr;
  G[1 * 16 + 0 * 4 + 0] = m * f / (r * r);
  G[1 * 16 + 1 * 4 + 1] = -m / (r * r * f);
  G[1 * 16 + 2 * 4 + 2] = -(r - 2.0 * m);
  G[1 * 16 + 3 * 4 + 3] = -(r - 2.0 * m) * sin_t * sin_t;
  const double gtheta_rt = 1.0 / r;
  G[2 * 16 + 1 * 4 + 2] = gtheta_rt;
  G[2 * 16 + 2 * 4 + 1] = gtheta_rt;
  G[2 * 16 + 3 * 4 + 3] = -sin_t * cos_t;
  G[3 * 16 + 1 * 4 + 3] = 1.0 / r;
  G[3 * 16 + 3 * 4 + 1] = 1.0 / r;
  const double cot = fabs(sin_t) < 1e-8 ? 0.0 : cos_t / sin_t;
  G[3 * 16 + 2 * 4 + 3] = cot;
  G[3 * 16 + 3 * 4 + 2] = cot;
}

// Generic Christoffel symbols from g^-1 and the FD dg (mod.rs:51-69), dense.
template <int K>
__device__ __forceinline__ bool christoffel_generic(const MetricDesc& M, const double x[4], double G[64]) {
  double ginv[16];
  const bool ok = metric_g_inv<K>(M, x, ginv);
  double dg[64];
  metric_dg<K>(M, x, dg);
#pragma unroll 1
  for (int mu = 0; mu < 4; ++mu)
#pragma unroll
    for (int alpha = 0; alpha < 4; ++alpha)
#pragma unroll
      for (int beta = 0; beta < 4; ++beta) {
        double s = 0.0;
#pragma unroll
        for (int sigma = 0; sigma < 4; ++sigma)
          s += ginv[4 * mu + sigma] *
               (dg[16 * alpha + 4 * sigma + beta] + dg[16 * beta + 4 * sigma + alpha] -
                dg[16 * sigma + 4 * alpha + beta]);
        G[16 * mu + 4 * alpha + beta] = 0.5 * s;
      }
  return ok;
}

// Generated: the sparse finite-difference Christoffel symbols and geodesic
// right-hand sides of Alcubierre and Morris-Thorne (in this namespace).
#include "christoffel_sparse.cuh"

// Christoffel symbols: analytic for Minkowski and Schwarzschild (their
// overrides), the finite-difference fallback for the others, evaluated by the
// generated sparse code (same bits as christoffel_generic).
template <int K>
__device__ __forceinline__ bool metric_christoffel(const MetricDesc& M, const double x[4], double G[64]) {
  if (K == KIND_MINKOWSKI) {
#pragma unroll
    for (int i = 0; i < 64; ++i) G[i] = 0.0;
    return true;
  } else if (K == KIND_SCHWARZSCHILD) {
    christoffel_schw(M, x, G);
    return true;
  } else if (K == KIND_ALCUBIERRE) {
    return christoffel_alcubierre_sparse(M, x, G);
  } else if (K == KIND_MORRIS_THORNE) {
    return christoffel_morris_thorne_sparse(M, x, G);
  } else {
    return christoffel_generic<K>(M, x, G);
  }
}

// Termination tests (minkowski.rs:32-39, schwarzschild.rs:109-121, alcubierre.rs:65-75,
// morris_thorne.rs:38-48).
template <int K>
__device__ __forceinline__ int metric_terminate(const MetricDesc& M, const double x[4]) {
  if (K == KIND_MINKOWSKI) {
    const double r2 = x[1] * x[1] + x[2] * x[2] + x[3] * x[3];
    return r2 > 1e6 ? TERM_ESCAPED : TERM_NONE;
  } else if (K == KIND_SCHWARZSCHILD) {
    const double r = x[1];
    if (!isfinite(r)) return TERM_DIVERGED;
    if (r < M.capture_r) return TERM_CAPTURED;
    if (r > M.escape_r) return TERM_ESCAPED;
    return TERM_NONE;
  } else if (K == KIND_ALCUBIERRE) {
    const double r2 = x[1] * x[1] + x[2] * x[2] + x[3] * x[3];
    if (!isfinite(r2)) return TERM_DIVERGED;
    return r2 > 1e6 ? TERM_ESCAPED : TERM_NONE;
  } else if (K == KIND_MORRIS_THORNE) {
    const double l = x[1];
    if (!isfinite(l)) return TERM_DIVERGED;
    return fabs(l) > 1000.0 ? TERM_ESCAPED : TERM_NONE;
  } else {  // sampled metric: leaving the grid ends the ray (below the inner radius of a spherical chart: Captured)
    if (!isfinite(x[1]) || !isfinite(x[2]) || !isfinite(x[3])) return TERM_DIVERGED;
    const FieldDesc& F = M.f;
    if (F.chart == GEON_CHART_SPHERICAL && F.n[0] > 1 && x[1] < F.lo[0]) return TERM_CAPTURED;
#pragma unroll
    for (int a = 0; a < 3; ++a)
      if (F.n[a] > 1 && (x[a + 1] < F.lo[a] || x[a + 1] > F.hi[a])) return TERM_ESCAPED;
    return TERM_NONE;
  }
}

// Escape direction (mod.rs:91-108 default; alcubierre.rs:81-88; morris_thorne.rs:54-77).
template <int K>
__device__ __forceinline__ void metric_asymptotic_direction(const MetricDesc& M, const double x[4],
                                                            const double p[4], double out[3]) {
  if (K == KIND_ALCUBIERRE || (K == KIND_FIELD && M.f.chart == GEON_CHART_CARTESIAN)) {
    const double vx = p[1], vy = p[2], vz = p[3];
    const double n = fmax(sqrt(vx * vx + vy * vy + vz * vz), 1e-30);
    out[0] = vx / n; out[1] = vy / n; out[2] = vz / n;
    return;
  }
  double sin_t, cos_t, sin_p, cos_p;
  dm::sincos_det(x[2], &sin_t, &cos_t);
  dm::sincos_det(x[3], &sin_p, &cos_p);
  const double pr = p[1], pt = p[2], pp = p[3];
  if (K == KIND_MORRIS_THORNE) {
    const double l = x[1];
    const double r_eff = fmax(fabs(l), 1e-30);
    const double vx = sin_t * cos_p * pr + r_eff * cos_t * cos_p * pt - r_eff * sin_t * sin_p * pp;
    const double vy = sin_t * sin_p * pr + r_eff * cos_t * sin_p * pt + r_eff * sin_t * cos_p * pp;
    const double vz = cos_t * pr - r_eff * sin_t * pt;
    const double n = fmax(sqrt(vx * vx + vy * vy + vz * vz), 1e-30);
    const double sign = l < 0.0 ? -1.0 : 1.0;
    out[0] = sign * vx / n; out[1] = vy / n; out[2] = vz / n;
  } else {
    const double r = x[1];
    const double vx = sin_t * cos_p * pr + r * cos_t * cos_p * pt - r * sin_t * sin_p * pp;
    const double vy = sin_t * sin_p * pr + r * cos_t * sin_p * pt + r * sin_t * cos_p * pp;
    const double vz = cos_t * pr - r * sin_t * pt;
    const double n = fmax(sqrt(vx * vx + vy * vy + vz * vz), 1e-30);
    out[0] = vx / n; out[1] = vy / n; out[2] = vz / n;
  }
}


// ---------------------------------------------------------------------------
// Geodesic right-hand side (geodesic.rs:38-59): k = (p, -Gamma^mu_ab p^a p^b).
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ bool geodesic_rhs(const MetricDesc& M, const double y[8], double k[8]) {
  k[0] = y[4]; k[1] = y[5]; k[2] = y[6]; k[3] = y[7];
  const double p0 = y[4], p1 = y[5], p2 = y[6], p3 = y[7];
  if (K == KIND_MINKOWSKI) {
    // Every term is 0 * p * p: the sum is +0.0 and the derivative -0.0.
    k[4] = -0.0; k[5] = -0.0; k[6] = -0.0; k[7] = -0.0;
    return true;
  } else if (K == KIND_SCHWARZSCHILD) {
    // schwarzschild.rs:61-107 fused with the sum; only the nonzero entries
    // contribute (alpha-major, beta-minor order kept).
    const double r = y[1], theta = y[2], m = M.p[0];
    const double f = 1.0 - 2.0 * m / r;
    double sin_t, cos_t;
    dm::sincos_det(theta, &sin_t, &cos_t);
    const double rr = r * r;
    const double rrf = rr * f;
    const double gtr = m / rrf;            // Gamma^t_tr = Gamma^t_rt
    const double g_r_tt = m * f / rr;      // Gamma^r_tt
    const double g_r_rr = -gtr;            // -m/(r r f) == -(m/(r r f))
    const double r2m = r - 2.0 * m;
    const double g_r_thth = -r2m;          // Gamma^r_thth
    const double g_r_phph = -r2m * sin_t * sin_t;
    const double ir = 1.0 / r;             // Gamma^th_rth, Gamma^ph_rph
    const double g_th_phph = -sin_t * cos_t;
    const double cot = fabs(sin_t) < 1e-8 ? 0.0 : cos_t / sin_t;
    double s;
    s = plus_zero(gtr * p0 * p1);
    s += gtr * p1 * p0;
    k[4] = -s;
    s = plus_zero(g_r_tt * p0 * p0);
    s += g_r_rr * p1 * p1;
    s += g_r_thth * p2 * p2;
    s += g_r_phph * p3 * p3;
    k[5] = -s;
    s = plus_zero(ir * p1 * p2);
    s += ir * p2 * p1;
    s += g_th_phph * p3 * p3;
    k[6] = -s;
    s = plus_zero(ir * p1 * p3);
    s += cot * p2 * p3;
    s += ir * p3 * p1;
    s += cot * p3 * p2;
    k[7] = -s;
    return true;
  } else if (K == KIND_ALCUBIERRE) {
    return rhs_alcubierre_sparse(M, y, k);
  } else if (K == KIND_MORRIS_THORNE) {
    return rhs_morris_thorne_sparse(M, y, k);
  } else {  // the reference's dense sum (geodesic.rs:38-59)
    double G[64];
    const bool ok = metric_christoffel<K>(M, y, G);
    const double p[4] = {p0, p1, p2, p3};
#pragma unroll
    for (int mu = 0; mu < 4; ++mu) {
      double s = 0.0;
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) s += G[16 * mu + 4 * a + b] * p[a] * p[b];
      k[4 + mu] = -s;
    }
    return ok;
  }
}

// Classical RK4 (integrator.rs:16-40) with the reference's grouping:
// y + (0.5*h)*k, y + h*k3, and y + (h/6)*(((k1 + 2 k2) + 2 k3) + k4).
template <int K>
__device__ __forceinline__ bool rk4_step(const MetricDesc& M, const double y[8], double h,
                                         double half_h, double sixth, double out[8]) {
  double k[8], acc[8], ys[8];
  bool ok = geodesic_rhs<K>(M, y, k);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    acc[i] = k[i];
    ys[i] = y[i] + half_h * k[i];
  }
  ok &= geodesic_rhs<K>(M, ys, k);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    acc[i] = acc[i] + 2.0 * k[i];
    ys[i] = y[i] + half_h * k[i];
  }
  ok &= geodesic_rhs<K>(M, ys, k);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    acc[i] = acc[i] + 2.0 * k[i];
    ys[i] = y[i] + h * k[i];
  }
  ok &= geodesic_rhs<K>(M, ys, k);
#pragma unroll
  for (int i = 0; i < 8; ++i) out[i] = y[i] + sixth * (acc[i] + k[i]);
  return ok;
}

// Residual |g(p, p)| at the position of y (geodesic.rs:82-84), dense dot4.
template <int K>
__device__ __forceinline__ double null_residual(const MetricDesc& M, const double y[8]) {
  double g[16];
  metric_g<K>(M, y, g);
  const double p[4] = {y[4], y[5], y[6], y[7]};
  return fabs(dot4(g, p, p));
}

}  // namespace geon
