// Adaptive stepping (GEON_ADAPTIVE): the persistent trace loop of
// trace_common.cuh with an embedded Runge-Kutta pair in FP64 in place of the
// reference's fixed-step RK4 (integrator.rs:16-40; the reference lists adaptive
// stepping as a TODO at integrator.rs:5-7). Opt-in and not parity-bound to the
// reference: it changes the integration, not the geodesic equation, and ends
// the 20,000-step caps far from the hole with a few hundred steps.
//
// Method: Dormand & Prince 5(4) (J. R. Dormand, P. J. Prince, "A family of
// embedded Runge-Kutta formulae", J. Comput. Appl. Math. 6 (1980) 19-26): 7
// stages with the first-same-as-last property, the 5th-order solution
// propagated, the 4th-order embedded one for the error. Error norm (Hairer,
// Norsett, Wanner, Solving ODEs I, II.4): err = sqrt(mean_i((e_i / sc_i)^2)),
// sc_i = atol + rtol * max(|y_i|, |y_new_i|). Step control uses only IEEE
// operations (+, -, *, /, sqrt), so the CPU oracle's restatement reproduces every
// step bit for bit: accept when err <= 1; next h = h * clamp(0.9 / err^(1/4),
// 0.2, 5) (fourth root by two square roots; err = 0 gives the factor 5). A
// non-finite trial state is a rejection; after 64 consecutive rejections the
// ray ends Diverged (the reference's NaN guard). max_steps counts accepted
// steps. The right-hand side is the FP64 geodesic_rhs (sparse, bit-exact).
#include <cuda_runtime.h>

#include "internal.h"
#include "metric_fp64.cuh"
#include "trace_common.cuh"

namespace geon {

namespace dp5 {
// Butcher tableau of DOPRI5 (rational coefficients, rounded once to double).
// The geodesic equation is autonomous, so the nodes c_i are not needed.
constexpr double A21 = 1.0 / 5.0;
constexpr double A31 = 3.0 / 40.0, A32 = 9.0 / 40.0;
constexpr double A41 = 44.0 / 45.0, A42 = -56.0 / 15.0, A43 = 32.0 / 9.0;
constexpr double A51 = 19372.0 / 6561.0, A52 = -25360.0 / 2187.0, A53 = 64448.0 / 6561.0, A54 = -212.0 / 729.0;
constexpr double A61 = 9017.0 / 3168.0, A62 = -355.0 / 33.0, A63 = 46732.0 / 5247.0, A64 = 49.0 / 176.0,
                 A65 = -5103.0 / 18656.0;
constexpr double B1 = 35.0 / 384.0, B3 = 500.0 / 1113.0, B4 = 125.0 / 192.0, B5 = -2187.0 / 6784.0,
                 B6 = 11.0 / 84.0;
// error weights b - b* (b* the embedded 4th-order weights)
constexpr double E1 = 71.0 / 57600.0, E3 = -71.0 / 16695.0, E4 = 71.0 / 1920.0, E5 = -17253.0 / 339200.0,
                 E6 = 22.0 / 525.0, E7 = -1.0 / 40.0;
constexpr int MAX_REJECT = 64;
}  // namespace dp5

template <int K>
struct AdaptiveStepper {
  double y[8];
  double k1[8];  // f(y), kept across steps (first same as last)
  double h;
  bool fresh;    // k1 not yet evaluated for this ray
  bool singular = false;

  __device__ __forceinline__ void load(const TraceLaunch& L, const double y0[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = y0[i];
    h = L.step;
    fresh = true;
  }
  __device__ __forceinline__ void to_double(double out[8]) const {
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = y[i];
  }
  __device__ __forceinline__ int terminate(const TraceLaunch& L) const { return metric_terminate<K>(L.M, y); }

  // One accepted step (with its rejected attempts). Returns STEP_OK or
  // STEP_NONFINITE (the ray ends Diverged with its state unchanged).
  __device__ int step(const TraceLaunch& L) {
    using namespace dp5;
    if (fresh) {
      singular |= !geodesic_rhs<K>(L.M, y, k1);
      fresh = false;
    }
    for (int attempt = 0; attempt < MAX_REJECT; ++attempt) {
      double k2[8], k3[8], k4[8], k5[8], k6[8], k7[8], ys[8], yn[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) ys[i] = y[i] + h * (A21 * k1[i]);
      singular |= !geodesic_rhs<K>(L.M, ys, k2);
#pragma unroll
      for (int i = 0; i < 8; ++i) ys[i] = y[i] + h * (A31 * k1[i] + A32 * k2[i]);
      singular |= !geodesic_rhs<K>(L.M, ys, k3);
#pragma unroll
      for (int i = 0; i < 8; ++i) ys[i] = y[i] + h * ((A41 * k1[i] + A42 * k2[i]) + A43 * k3[i]);
      singular |= !geodesic_rhs<K>(L.M, ys, k4);
#pragma unroll
      for (int i = 0; i < 8; ++i)
        ys[i] = y[i] + h * (((A51 * k1[i] + A52 * k2[i]) + A53 * k3[i]) + A54 * k4[i]);
      singular |= !geodesic_rhs<K>(L.M, ys, k5);
#pragma unroll
      for (int i = 0; i < 8; ++i)
        ys[i] = y[i] + h * ((((A61 * k1[i] + A62 * k2[i]) + A63 * k3[i]) + A64 * k4[i]) + A65 * k5[i]);
      singular |= !geodesic_rhs<K>(L.M, ys, k6);
#pragma unroll
      for (int i = 0; i < 8; ++i)
        yn[i] = y[i] + h * ((((B1 * k1[i] + B3 * k3[i]) + B4 * k4[i]) + B5 * k5[i]) + B6 * k6[i]);
      singular |= !geodesic_rhs<K>(L.M, yn, k7);
      double sum = 0.0;
      bool finite = true;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const double e = h * (((((E1 * k1[i] + E3 * k3[i]) + E4 * k4[i]) + E5 * k5[i]) + E6 * k6[i]) + E7 * k7[i]);
        const double ay = fabs(y[i]), an = fabs(yn[i]);
        const double sc = L.atol + L.rtol * (ay > an ? ay : an);
        const double q = e / sc;
        sum = sum + q * q;
        finite &= isfinite(yn[i]) && isfinite(k7[i]);
      }
      const double err = finite ? sqrt(sum / 8.0) : INFINITY;
      if (!(err <= 1.0)) {  // reject (also NaN): shrink and retry
        double fac = 0.2;
        if (isfinite(err)) {
          fac = 0.9 / sqrt(sqrt(err));
          if (fac < 0.2) fac = 0.2;
        }
        h = h * fac;
        continue;
      }
      double fac = 5.0;
      if (err > 0.0) {
        fac = 0.9 / sqrt(sqrt(err));
        if (fac > 5.0) fac = 5.0;
        if (fac < 0.2) fac = 0.2;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        y[i] = yn[i];
        k1[i] = k7[i];
      }
      h = h * fac;
      return STEP_OK;
    }
    return STEP_NONFINITE;
  }
  __device__ __forceinline__ void group_end(const TraceLaunch&) {}
  __device__ __forceinline__ void check_null(const TraceLaunch&, const double*) {}
  __device__ __forceinline__ void finish(const TraceLaunch& L) {
    if (singular) atomicOr(L.flags, 1);
  }
};

template <int K, int SRC, int SINK>
__global__ void __launch_bounds__(TRACE_BLOCK) trace_adaptive_kernel(const TraceLaunch L) {
  trace_loop<AdaptiveStepper<K>, K, SRC, SINK>(L);
}

template <int K, int SRC, int SINK>
static cudaError_t launch_ka(const TraceLaunch& L, cudaStream_t s) {
  static int sms = 0, per_sm = 0;
  if (sms == 0) {
    int dev = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, trace_adaptive_kernel<K, SRC, SINK>, TRACE_BLOCK, 0);
    per_sm = occ < 1 ? 1 : occ;
  }
  int64_t blocks = persistent_slots(sms, per_sm, L.reserve_per_sm);
  const int64_t need = (L.n + TRACE_BLOCK - 1) / TRACE_BLOCK;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  trace_adaptive_kernel<K, SRC, SINK><<<(unsigned)blocks, TRACE_BLOCK, 0, s>>>(L);
  return cudaGetLastError();
}

template <int K>
static cudaError_t launch_k(const TraceLaunch& L, int src, int sink, cudaStream_t s) {
  if (src == SRC_ARRAY && sink == SINK_TRACE) return launch_ka<K, SRC_ARRAY, SINK_TRACE>(L, s);
  if (src == SRC_CAMERA && sink == SINK_RENDER) return launch_ka<K, SRC_CAMERA, SINK_RENDER>(L, s);
  if (src == SRC_CAMERA && sink == SINK_TRACE) return launch_ka<K, SRC_CAMERA, SINK_TRACE>(L, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_trace_adaptive(const TraceLaunch& L, int src, int sink, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  if (src == SRC_EQUATORIAL) {
    if (L.M.kind != KIND_SCHWARZSCHILD) return cudaErrorInvalidValue;
    if (sink == SINK_SHADOW) return launch_ka<KIND_SCHWARZSCHILD, SRC_EQUATORIAL, SINK_SHADOW>(L, s);
    if (sink == SINK_TRACE) return launch_ka<KIND_SCHWARZSCHILD, SRC_EQUATORIAL, SINK_TRACE>(L, s);
    return cudaErrorInvalidValue;
  }
  switch (L.M.kind) {
    case KIND_MINKOWSKI: return launch_k<KIND_MINKOWSKI>(L, src, sink, s);
    case KIND_SCHWARZSCHILD: return launch_k<KIND_SCHWARZSCHILD>(L, src, sink, s);
    case KIND_ALCUBIERRE: return launch_k<KIND_ALCUBIERRE>(L, src, sink, s);
    case KIND_MORRIS_THORNE: return launch_k<KIND_MORRIS_THORNE>(L, src, sink, s);
    case KIND_FIELD: return launch_k<KIND_FIELD>(L, src, sink, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace geon
