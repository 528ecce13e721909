// Internal types shared by the CUDA translation units and the C ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/geon_gpu.h"

namespace geon {

enum : int { TERM_NONE = -1, TERM_DIVERGED = 0, TERM_CAPTURED = 1, TERM_ESCAPED = 2 };
enum : int { KIND_MINKOWSKI = 0, KIND_SCHWARZSCHILD = 1, KIND_ALCUBIERRE = 2, KIND_MORRIS_THORNE = 3,
             KIND_FIELD = 4 };

// A sampled (tensor-field) metric: the 10 unique components of g at the nodes
// of a regular grid over the three spatial chart coordinates, used as the
// control points of a uniform cubic B-spline (geon_metric_create_field).
struct FieldDesc {
  const double* c;   // device: node (i, j, k) at 10 * (i + n0 * (j + n1 * k))
  double lo[3], hi[3];
  double inv_d[3];   // (n - 1) / (hi - lo), 0 for an axis with one node
  int64_t n[3];
  int chart;         // GEON_CHART_CARTESIAN or GEON_CHART_SPHERICAL
};

// Per-metric constants, passed by value to every kernel (kernel parameters live
// in the constant bank, so every lane reads them through the constant cache).
struct MetricDesc {
  int kind;
  double p[4];       // the reference struct's fields, in declaration order
  double capture_r;  // Schwarzschild: horizon_pad * 2.0 * mass   (schwarzschild.rs:114)
  double escape_r;   // Schwarzschild: escape_radius * mass        (schwarzschild.rs:116)
  double alc_denom;  // Alcubierre: 2.0 * tanh(R / s)               (alcubierre.rs:42)
  FieldDesc f;       // GEON_FIELD only
};

// Camera for device-side ray generation (camera.rs:113-160 with the values that
// the reference recomputes per pixel hoisted: they are identical every time).
struct CameraDesc {
  double tet[4][4];  // rows e_a^mu
  double obs[4];
  double h_img;      // tan(fov_y_rad * 0.5), from the host libm as in the reference
  double w_img;      // h_img * aspect
  double width_d, height_d;
  int64_t width, height;
  int64_t spa;       // samples per axis
  double inv_spa;
  int forward_sign;
};

enum : int { MIXED_REPROJECT = 1, MIXED_ORBIT = 2, MIXED_NULLFIX = 4 };
// mixed-kernel variants: register cap (none, 64, 51 registers) x block size
// (128, 64, 256; block sizes other than 128 only for the equatorial source)
constexpr int MIXED_CAPS = 3;
constexpr int MIXED_VARIANTS = 9;

// A regular grid of points for curvature jobs (geon_grid of the ABI).
struct GridDesc {
  double lo[3], hi[3];
  int64_t n[3];
  double t;
};

// Sources of initial states.
// SRC_STATE: a stepper state prepared by an earlier kernel (16 words per ray in
// ystate: the mixed path's (hi, lo) pairs), so the trace kernel itself runs no
// FP64 set-up code.
enum : int { SRC_ARRAY = 0, SRC_CAMERA = 1, SRC_EQUATORIAL = 2, SRC_STATE = 3 };
// Where results go.
// SINK_STATE: the stepper's final state back into ystate (with term and
// steps), shaded by a later kernel; the trace kernel runs no FP64 sink code.
enum : int { SINK_TRACE = 0, SINK_RENDER = 1, SINK_SHADOW = 2, SINK_STATE = 3 };

struct TraceLaunch {
  MetricDesc M;
  CameraDesc cam;
  int64_t n;           // rays in the job
  double step;
  double half_step;    // 0.5 * step   (integrator.rs:24: `0.5 * h * k`, left-associated)
  double sixth;        // step / 6.0   (integrator.rs:36)
  int64_t max_steps;
  // SRC_ARRAY
  const double* y0;    // n x 8 (AoS, the reference's State layout)
  // SRC_STATE / SINK_STATE: 16 words per ray (ray i at ystate + 16 i), in place
  uint32_t* ystate;
  // SRC_EQUATORIAL (bin/validate_shadow.rs:20-35)
  const double* alpha; // n launch angles
  double r_obs;
  // SINK_TRACE
  int32_t* term;
  double* yfinal;      // n x 8
  int64_t* steps;
  double* resid;
  // SINK_RENDER: per-sample results, reduced per pixel afterwards
  float* srgb;         // n x 3
  int show_stars;
  float captured_rgb[3];  // RenderConfig::captured_rgb (render.rs:20)
  float diverged_rgb[3];  // RenderConfig::diverged_rgb (render.rs:25)
  // mixed precision
  float band;          // FP64 band half-width in the metric's own scale (0 = no band)
  float reserve_per_sm;  // persistent grid leaves this many blocks per SM free (may be fractional)
  int variant;         // mixed kernel register-cap variant (0: none, 1: 8 blocks/SM, 2: 10)
  int mixed_flags;     // MIXED_* bits
  int decide;          // shadow rays whose class is all a caller needs (bisection rounds): the mixed
                       // path ends a ray as soon as its class is settled (MixedCore::decided_k)
  // adaptive stepping (GEON_ADAPTIVE): error tolerances
  double rtol, atol;
  // work queue
  const int32_t* order;       // the k-th claimed ray is order[k] (null: ray k); n < 2^31 when set
  unsigned long long* queue;  // next unclaimed ray index
  int* flags;                 // bit 0: a metric became singular (inverse of g failed)
};

// ---- launchers (trace_fp64.cu) ----
cudaError_t launch_trace_fp64(const TraceLaunch& L, int src, int sink, cudaStream_t s);
// ---- launchers (trace_mixed.cu) ----
cudaError_t launch_trace_mixed(const TraceLaunch& L, int src, int sink, cudaStream_t s);
// ---- launchers (trace_adaptive.cu) ----
// Blocks of a persistent grid: every resident slot (sms x per_sm) minus the
// slots per SM the caller keeps free for a concurrent job; a fractional reserve
// is rounded over the whole GPU (some SMs keep one slot more than others). At
// least one block per SM.
inline int64_t persistent_slots(int sms, int per_sm, float reserve) {
  double use = (double)per_sm - (double)reserve;
  if (use < 1.0) use = 1.0;
  return (int64_t)((double)sms * use);
}

cudaError_t launch_trace_adaptive(const TraceLaunch& L, int src, int sink, cudaStream_t s);
// ---- one persistent launch over several renders (trace_fp64.cu, trace_mixed.cu) ----
// Job j of the launch owns the global ray indices [start[j], start[j+1]) of its
// one work queue (trace_loop_multi in trace_common.cuh).
constexpr int MULTI_MAX_JOBS = 8;
struct MultiDesc {
  int njobs;
  int kind_mask;  // bit K set when a job of the launch has metric kind K (the mixed kernel's variant)
  int64_t start[MULTI_MAX_JOBS + 1];
  unsigned long long* queue;
};
cudaError_t launch_trace_multi_fp64(const TraceLaunch* jobs, const MultiDesc& D, float reserve, cudaStream_t s);
cudaError_t launch_trace_multi_mixed(const TraceLaunch* jobs, const MultiDesc& D, float reserve, cudaStream_t s);
// Mixed renders in three kernels (trace_mixed.cu): the camera rays' prepared
// states into L.ystate, the trace over them (SRC_STATE, SINK_STATE), and the
// shading of the final states into L.srgb / term / steps / resid (the render
// sink's outputs). launch_render_mixed runs all three for one job;
// launch_render_prepare / _shade one end each (several jobs in one trace).
cudaError_t launch_render_mixed(const TraceLaunch& L, cudaStream_t s);
cudaError_t launch_render_prepare(const TraceLaunch& L, cudaStream_t s);
cudaError_t launch_render_shade(const TraceLaunch& L, cudaStream_t s);
// ---- launchers (trace_fp64fast.cu) ----
cudaError_t launch_trace_fp64fast(const TraceLaunch& L, int src, int sink, cudaStream_t s);
// rgb and rgb8 (the tonemapped bytes) may each be null
cudaError_t launch_render_reduce(const float* srgb, const int32_t* term, const int64_t* steps,
                                 const double* resid, int64_t npix, int64_t spa, float* rgb,
                                 int32_t* pclass, int64_t* psteps, unsigned long long* stats,
                                 cudaStream_t s, uint8_t* rgb8 = nullptr);
cudaError_t launch_tonemap(const float* rgb, int64_t n, uint8_t* out, cudaStream_t s);
cudaError_t launch_pointwise(const MetricDesc& M, int what, const double* in, int64_t n, double* out,
                             int32_t* iout, int* flags, cudaStream_t s);
cudaError_t launch_tetrad(const MetricDesc& M, const double* obs, double* out16, int* status,
                          cudaStream_t s);
cudaError_t launch_metric_init(MetricDesc* d_desc, cudaStream_t s);
cudaError_t launch_sky(const double* dir, int64_t n, int show, float* rgb, cudaStream_t s);
cudaError_t launch_bisect_build(int64_t nb, int64_t per, const double* lo, const double* hi, double* alpha,
                                cudaStream_t s);
cudaError_t launch_bisect_walk(int64_t nb, int64_t per, int levels, const double* alpha, const int32_t* term,
                               const int64_t* steps, double* lo, double* hi, int64_t* path_steps,
                               cudaStream_t s);
cudaError_t launch_bisect_finish(int64_t nb, const double* lo, const double* hi, double* alpha_c,
                                 cudaStream_t s);
cudaError_t launch_fma_probe(int fp64, void* out, int blocks, int threads, int iters, cudaStream_t s);
// Claim order of a shadow sweep, longest rays first: order[] gets the indices of
// the rays whose impact parameter is at least 0.998 b_c (escaping or orbiting
// near the photon sphere: the long paths) from the front and the others from
// the back; counters (2 x u64, zeroed by the caller) are the two fill levels.
cudaError_t launch_shadow_order(double m, double r_obs, const double* alpha, int64_t n, int32_t* order,
                                unsigned long long* counters, cudaStream_t s);

// ---- launchers (curvature_fp64.cu) ----
// what: 0 riemann, 1 ricci, 2 ricci_scalar, 3 einstein, 4 stress_energy, 5 nec
cudaError_t launch_curvature(const MetricDesc& M, int what, const double* x, int64_t n,
                             const double* k, int64_t nk, int k_shared, double* out, int* flags,
                             cudaStream_t s);
cudaError_t launch_curvature_grid(const MetricDesc& M, const GridDesc& grid, int64_t nk, uint64_t seed,
                                  double* einstein, double* nec, double* kout, int* flags, cudaStream_t s);

// ---- capi.cu helpers shared with other entry-point units ----
const MetricDesc* metric_desc(geon_metric_t m);
TraceLaunch trace_launch_defaults(geon_metric_t m, double step, int64_t max_steps);
cudaError_t launch_trace_any(const TraceLaunch& L, int precision, int src, int sink, cudaStream_t s);
void note_launches(unsigned long long n);
int set_last_error(int code, const char* msg);
int bisect_levels_for(size_t nb);  // the default speculative width (fixed: the no-alloc scratch is sized for it)
int camera_desc_for(geon_metric_t m, const geon_camera* cam, int64_t spa, CameraDesc& c, cudaStream_t s);

// pointwise "what" codes
enum : int { PW_G = 0, PW_DG = 1, PW_GINV = 2, PW_CHRISTOFFEL = 3, PW_TERMINATE = 4, PW_ASYM = 5 };

}  // namespace geon
