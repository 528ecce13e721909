// GEON_FP64_FAST: an FP64 RK4 trace held to the tolerance of the reference's
// own CUDA kernel (cuda/schwarzschild_render.cu:3-5, "up to associativity")
// instead of to the reference's bits.
//
// Same chart, same fixed-step classical RK4 with the same stage points, the
// same termination tests (schwarzschild.rs:109-121) before every step and the
// same NaN guard and step cap (geodesic.rs:73-116) as the FP64 parity path, so
// a ray's class and final state differ from the reference only by rounding
// (amplified, as for any two FP64 evaluations, near the photon sphere). What is
// cheaper, per right-hand side (schwarzschild.rs:61-107 fused with
// geodesic.rs:38-59):
//   * one reciprocal, of D = r (r - 2M) sin(theta), in place of the reference's
//     five divisions: 1/r, Gamma^t_tr = M / (r (r - 2M)) and cot(theta) are
//     products with 1/D, and Gamma^r_tt = Gamma^t_tr f^2 with f = 1 - 2M/r;
//   * sin and cos of the polar angle carried from step to step: the three
//     later stages move theta by d = c h k^theta and take sin, cos of
//     theta0 + d by the angle-addition formula with Taylor polynomials of sin d
//     and cos d (|d| <= 1/32, truncation below 1e-19; larger offsets evaluate
//     sincos_det of the stage angle itself), the next step's theta0 the same
//     way from the step's own increment, and sincos_det afresh every 16 steps
//     of a ray (at load and after each group of 16 steps), so the carried
//     values stay within a few ulp;
//   * the sparse sums with fused multiply-adds, the Christoffel symbols shared
//     between their symmetric entries, and no stage positions for t and phi
//     (nothing reads them);
//   * equatorial rays (bin/validate_shadow.rs:20-35: theta = pi/2, p^theta = 0)
//     step on their invariant plane with no trigonometry at all.
// Metrics other than Schwarzschild and Minkowski run the FP64 parity stepper
// (their Christoffel symbols come from the finite-difference fallback, whose
// cost is the metric evaluations, not the combination).
//
// This unit is compiled with --fmad=false like the others: every fused
// multiply-add below is written out.
#include <cuda_runtime.h>

#include "internal.h"
#include "metric_fp64.cuh"
#include "trace_common.cuh"

namespace geon {

namespace fast {

// sin(theta0 + d), cos(theta0 + d) from s0 = sin(theta0), c0 = cos(theta0) for
// |d| <= 1/32: sin d = d (1 - d^2/3! + d^4/5! - d^6/7!) (next term d^9/9! <
// 8e-20), cos d = 1 - d^2/2! + d^4/4! - d^6/6! + d^8/8! (next term < 3e-20).
__device__ __forceinline__ void sincos_offset(double s0, double c0, double d, double* s, double* c) {
  const double z = d * d;
  double ps = fma(z, -1.0 / 5040.0, 1.0 / 120.0);
  ps = fma(z, ps, -1.0 / 6.0);
  const double sd = fma(d * z, ps, d);
  double pc = fma(z, 1.0 / 40320.0, -1.0 / 720.0);
  pc = fma(z, pc, 1.0 / 24.0);
  pc = fma(z, pc, -0.5);
  const double cm1 = z * pc;  // cos d - 1
  *s = fma(s0, cm1, fma(c0, sd, s0));
  *c = fma(c0, cm1, fma(-s0, sd, c0));
}

// Momentum derivatives of the Schwarzschild geodesic equation at radius r,
// polar angle with sin s and cos c, momentum p (k4..k7 of geodesic.rs:49-57).
// The reference's guard (schwarzschild.rs:98-102): cot(theta) = 0 where
// |sin theta| < 1e-8.
__device__ __forceinline__ void rhs(double m, double two_m, double r, double s, double c, double p0, double p1,
                                    double p2, double p3, double* k4, double* k5, double* k6, double* k7) {
  const double rm = r - two_m;
  const bool pole = fabs(s) < 1e-8;
  const double se = pole ? 1.0 : s;
  const double rrm = r * rm;
  const double iD = __drcp_rn(rrm * se);
  const double iDs = iD * se;          // 1 / (r (r - 2M))
  const double ir = rm * iDs;          // 1 / r
  const double cot = pole ? 0.0 : c * (rrm * iD);
  const double u = m * iDs;            // Gamma^t_tr = M / (r^2 f) = -Gamma^r_rr
  const double f = rm * ir;            // 1 - 2M/r
  const double grtt = u * (f * f);     // Gamma^r_tt = M f / r^2 = Gamma^t_tr f^2
  const double q = fma(s * s, p3 * p3, p2 * p2);    // p_theta^2 + sin^2 p_phi^2
  *k4 = ((-two_m * iDs) * p0) * p1;    // -2 Gamma^t_tr p^t p^r
  *k5 = fma(rm, q, fma(u, p1 * p1, -(grtt * p0) * p0));
  *k6 = fma(s * c, p3 * p3, (-2.0 * ir * p1) * p2);
  *k7 = (-2.0 * p3) * fma(ir, p1, cot * p2);
}

// The same on the equatorial plane (s = 1, c = 0, p^theta = 0).
__device__ __forceinline__ void rhs_planar(double m, double two_m, double r, double p0, double p1, double p3,
                                           double* k4, double* k5, double* k7) {
  const double rm = r - two_m;
  const double iD = __drcp_rn(r * rm);
  const double ir = rm * iD;
  const double u = m * iD;
  const double f = rm * ir;
  const double grtt = u * (f * f);
  *k4 = ((-two_m * iD) * p0) * p1;
  *k5 = fma(rm, p3 * p3, fma(u, p1 * p1, -(grtt * p0) * p0));
  *k7 = (-2.0 * p3) * (ir * p1);
}

}  // namespace fast

// PLANAR: every ray is equatorial (the shadow source). Otherwise a ray that
// starts on the equator with p^theta = 0 exactly (theta = pi/2 to the double,
// as equatorial rays and states turned into their orbit-plane frame are)
// takes the planar step too: the plane is invariant, and the general step
// would only add the ~1e-16 drift that cos(pi/2 rounded) gives theta.
template <bool PLANAR>
struct FastSchwStepper {
  double y[8];
  bool on_plane = PLANAR;
  // sin and cos of y[2] for the general step, carried from step to step by
  // the angle-addition formula and taken afresh every 16 steps of the ray (at
  // load and after each group of 16 steps)
  double sth = 0.0, cth = 1.0;
  __device__ __forceinline__ void load(const TraceLaunch&, const double y0[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = y0[i];
    if (!PLANAR) {
      on_plane = y[2] == 1.5707963267948966 && y[6] == 0.0;
      if (!on_plane) dm::sincos_det(y[2], &sth, &cth);
    }
  }
  __device__ __forceinline__ void to_double(double out[8]) const {
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = y[i];
  }
  __device__ __forceinline__ int terminate(const TraceLaunch& L) const {
    return metric_terminate<KIND_SCHWARZSCHILD>(L.M, y);
  }

  __device__ __forceinline__ int step(const TraceLaunch& L) {
    const double m = L.M.p[0], two_m = 2.0 * m;
    const double h = L.step, hh = L.half_step;
    if (PLANAR || on_plane) {
      double k4, k5, k7;
      double p0 = y[4], p1 = y[5], p3 = y[7];
      fast::rhs_planar(m, two_m, y[1], p0, p1, p3, &k4, &k5, &k7);
      double k1 = p1;
      double a0 = p0, a1 = p1, a3 = p3, a4 = k4, a5 = k5, a7 = k7;
#pragma unroll
      for (int st = 0; st < 3; ++st) {
        const double c = st < 2 ? hh : h;
        const double r = fma(c, k1, y[1]);
        p0 = fma(c, k4, y[4]);
        p1 = fma(c, k5, y[5]);
        p3 = fma(c, k7, y[7]);
        fast::rhs_planar(m, two_m, r, p0, p1, p3, &k4, &k5, &k7);
        k1 = p1;
        if (st < 2) {
          a0 = fma(2.0, p0, a0);
          a1 = fma(2.0, p1, a1);
          a3 = fma(2.0, p3, a3);
          a4 = fma(2.0, k4, a4);
          a5 = fma(2.0, k5, a5);
          a7 = fma(2.0, k7, a7);
        }
      }
      const double sx = L.sixth;
      const double n0 = fma(sx, a0 + p0, y[0]), n1 = fma(sx, a1 + p1, y[1]), n3 = fma(sx, a3 + p3, y[3]);
      const double n4 = fma(sx, a4 + k4, y[4]), n5 = fma(sx, a5 + k5, y[5]), n7 = fma(sx, a7 + k7, y[7]);
      // t and phi advance by sums of the stage values of p^t and p^phi, which
      // the momentum increments contain: the guard on r and the momenta covers
      // them, and a sink that reads neither (the shadow sink) drops them.
      if (!(isfinite(n1) && isfinite(n4) && isfinite(n5) && isfinite(n7))) return STEP_NONFINITE;
      y[0] = n0; y[1] = n1; y[3] = n3; y[4] = n4; y[5] = n5; y[7] = n7;
      return STEP_OK;
    }
    const double s0 = sth, c0 = cth;
    double k4, k5, k6, k7;
    double p0 = y[4], p1 = y[5], p2 = y[6], p3 = y[7];
    fast::rhs(m, two_m, y[1], s0, c0, p0, p1, p2, p3, &k4, &k5, &k6, &k7);
    double k1 = p1, k2 = p2;
    double acc[8] = {p0, p1, p2, p3, k4, k5, k6, k7};
#pragma unroll
    for (int st = 0; st < 3; ++st) {
      const double c = st < 2 ? hh : h;
      const double r = fma(c, k1, y[1]);
      const double d = c * k2;
      p0 = fma(c, k4, y[4]);
      p1 = fma(c, k5, y[5]);
      p2 = fma(c, k6, y[6]);
      p3 = fma(c, k7, y[7]);
      double s, cs;
      if (fabs(d) <= 0.03125) {
        fast::sincos_offset(s0, c0, d, &s, &cs);
      } else {
        dm::sincos_det(y[2] + d, &s, &cs);
      }
      fast::rhs(m, two_m, r, s, cs, p0, p1, p2, p3, &k4, &k5, &k6, &k7);
      k1 = p1;
      k2 = p2;
      if (st < 2) {
        acc[0] = fma(2.0, p0, acc[0]);
        acc[1] = fma(2.0, p1, acc[1]);
        acc[2] = fma(2.0, p2, acc[2]);
        acc[3] = fma(2.0, p3, acc[3]);
        acc[4] = fma(2.0, k4, acc[4]);
        acc[5] = fma(2.0, k5, acc[5]);
        acc[6] = fma(2.0, k6, acc[6]);
        acc[7] = fma(2.0, k7, acc[7]);
      }
    }
    const double last[8] = {p0, p1, p2, p3, k4, k5, k6, k7};
    double yn[8];
    bool finite = true;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      yn[i] = fma(L.sixth, acc[i] + last[i], y[i]);
      finite &= isfinite(yn[i]);
    }
    if (!finite) return STEP_NONFINITE;
    // sin and cos at the new theta from those at the old one (the difference of
    // two nearby doubles is exact)
    const double dth = yn[2] - y[2];
    if (fabs(dth) <= 0.03125) {
      double sn, cn;
      fast::sincos_offset(s0, c0, dth, &sn, &cn);
      sth = sn;
      cth = cn;
    } else {
      dm::sincos_det(yn[2], &sth, &cth);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = yn[i];
    return STEP_OK;
  }
  __device__ __forceinline__ void group_end(const TraceLaunch&) {
    if (!PLANAR && !on_plane) dm::sincos_det(y[2], &sth, &cth);
  }
  __device__ __forceinline__ void check_null(const TraceLaunch&, const double*) {}
  __device__ __forceinline__ void finish(const TraceLaunch&) {}
};

template <int SRC, int SINK>
__global__ void __launch_bounds__(TRACE_BLOCK) trace_fp64fast_kernel(const TraceLaunch L) {
  trace_loop<FastSchwStepper<SRC == SRC_EQUATORIAL>, KIND_SCHWARZSCHILD, SRC, SINK>(L);
}

template <int SRC, int SINK>
static cudaError_t launch_fast(const TraceLaunch& L, cudaStream_t s) {
  static int sms = 0, per_sm = 0;
  if (sms == 0) {
    int dev = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, trace_fp64fast_kernel<SRC, SINK>, TRACE_BLOCK, 0);
    per_sm = occ < 1 ? 1 : occ;
  }
  const int64_t slots = persistent_slots(sms, per_sm, L.reserve_per_sm);
  const int64_t need = (L.n + TRACE_BLOCK - 1) / TRACE_BLOCK;
  int grid = (int)(need < slots ? need : slots);
  if (grid < 1) grid = 1;
  trace_fp64fast_kernel<SRC, SINK><<<grid, TRACE_BLOCK, 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_trace_fp64fast(const TraceLaunch& L, int src, int sink, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  if (L.M.kind != KIND_SCHWARZSCHILD) return launch_trace_fp64(L, src, sink, s);
  if (src == SRC_EQUATORIAL && sink == SINK_SHADOW) return launch_fast<SRC_EQUATORIAL, SINK_SHADOW>(L, s);
  if (src == SRC_EQUATORIAL && sink == SINK_TRACE) return launch_fast<SRC_EQUATORIAL, SINK_TRACE>(L, s);
  if (src == SRC_ARRAY && sink == SINK_TRACE) return launch_fast<SRC_ARRAY, SINK_TRACE>(L, s);
  if (src == SRC_CAMERA && sink == SINK_RENDER) return launch_fast<SRC_CAMERA, SINK_RENDER>(L, s);
  if (src == SRC_CAMERA && sink == SINK_TRACE) return launch_fast<SRC_CAMERA, SINK_TRACE>(L, s);
  return cudaErrorInvalidValue;
}

}  // namespace geon
