// C ABI of the library (include/geon_gpu.h): handles, host<->device staging,
// launches and status mapping. Host arithmetic here that must match the
// reference (the bisection midpoints, camera constants) is compiled with
// -ffp-contract=off.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "internal.h"

using namespace geon;

struct geon_metric {
  MetricDesc desc;
};

namespace {

thread_local std::string g_last_error;
std::atomic<int> g_show_stars{1};
// Mixed-precision options: FP64 band half-width per metric kind (in units of
// M, b0, s; 0 disables) and the null re-projection switch.
std::atomic<float> g_band[4] = {{0.0f}, {0.0f}, {0.0f}, {0.0f}};
std::atomic<int> g_reproject{0};
std::atomic<int> g_reserve{0};
// Mixed-kernel variant per metric kind and ray source (camera/array, equatorial),
// chosen by geon_autotune_mixed (default 0).
std::atomic<int> g_variant[4][2] = {{{0}, {0}}, {{0}, {0}}, {{0}, {0}}, {{0}, {0}}};
// Kernels launched by this library since load (ours only; memsets excluded).
std::atomic<unsigned long long> g_launches{0};
inline void counted(unsigned long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(e == cudaErrorMemoryAllocation ? GEON_ERR_OOM : GEON_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

#define GEON_CUDA(call)                                  \
  do {                                                   \
    cudaError_t e__ = (call);                            \
    if (e__ != cudaSuccess) return cuda_fail(e__, #call); \
  } while (0)

// Stream-ordered device buffer freed when it leaves scope.
struct DBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() {
    if (p) cudaFreeAsync(p, s);
  }
  cudaError_t alloc(size_t bytes, cudaStream_t st) {
    s = st;
    if (bytes == 0) bytes = 16;
    return cudaMallocAsync(&p, bytes, st);
  }
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};

constexpr double RADS_PER_DEG = 3.141592653589793 / 180.0;  // f64::to_radians

cudaStream_t host_stream() { return cudaStreamPerThread; }

int check_metric(geon_metric_t m) {
  if (!m) return fail(GEON_ERR_INVALID, "null metric handle");
  return GEON_OK;
}

int sync_and_flags(cudaStream_t s, const int* d_flags, int* h_flags) {
  GEON_CUDA(cudaMemcpyAsync(h_flags, d_flags, sizeof(int), cudaMemcpyDeviceToHost, s));
  GEON_CUDA(cudaStreamSynchronize(s));
  GEON_CUDA(cudaGetLastError());
  return GEON_OK;
}

int singular_status(int flags) {
  if (flags & 1) return fail(GEON_ERR_SINGULAR_METRIC, "metric became singular - coordinate chart broke down");
  return GEON_OK;
}

// Build the device camera for a metric: the tetrad comes from the device (same
// functor as the trace), the image-plane constants from the host libm.
int make_camera(geon_metric_t m, const geon_camera* cam, int64_t spa, CameraDesc& c, cudaStream_t s) {
  if (!cam || cam->width <= 0 || cam->height <= 0) return fail(GEON_ERR_INVALID, "bad camera size");
  if (cam->forward_sign != 1 && cam->forward_sign != -1) return fail(GEON_ERR_INVALID, "forward_sign must be +1 or -1");
  DBuf d;
  GEON_CUDA(d.alloc(sizeof(double) * 20 + sizeof(int), s));
  double* d_obs = d.as<double>();
  double* d_tet = d_obs + 4;
  int* d_status = reinterpret_cast<int*>(d_obs + 20);
  GEON_CUDA(cudaMemcpyAsync(d_obs, cam->observer, sizeof(double) * 4, cudaMemcpyHostToDevice, s));
  counted();
  GEON_CUDA(launch_tetrad(m->desc, d_obs, d_tet, d_status, s));
  double tet[16];
  int status = 0;
  GEON_CUDA(cudaMemcpyAsync(tet, d_tet, sizeof tet, cudaMemcpyDeviceToHost, s));
  GEON_CUDA(cudaMemcpyAsync(&status, d_status, sizeof status, cudaMemcpyDeviceToHost, s));
  GEON_CUDA(cudaStreamSynchronize(s));
  if (status == GEON_ERR_NOT_TIMELIKE) return fail(status, "observer is not in a timelike region (g_tt >= 0)");
  if (status == GEON_ERR_GRAM_SCHMIDT) return fail(status, "Gram-Schmidt produced non-spacelike vector - chart broken at this point");
  std::memcpy(c.tet, tet, sizeof tet);
  std::memcpy(c.obs, cam->observer, sizeof c.obs);
  const double fov = cam->fov_y_deg * RADS_PER_DEG;
  const double aspect = (double)cam->width / (double)cam->height;
  c.h_img = std::tan(fov * 0.5);
  c.w_img = c.h_img * aspect;
  c.width_d = (double)cam->width;
  c.height_d = (double)cam->height;
  c.width = cam->width;
  c.height = cam->height;
  c.spa = spa < 1 ? 1 : spa;
  c.inv_spa = 1.0 / (double)c.spa;
  c.forward_sign = cam->forward_sign;
  return GEON_OK;
}

TraceLaunch base_launch(geon_metric_t m, double step, int64_t max_steps) {
  TraceLaunch L;
  std::memset(&L, 0, sizeof L);
  L.M = m->desc;
  L.step = step;
  L.half_step = 0.5 * step;
  L.sixth = step / 6.0;
  L.max_steps = max_steps;
  L.band = g_band[m->desc.kind].load();
  L.mixed_flags = g_reproject.load() ? MIXED_REPROJECT : 0;
  L.reserve_per_sm = g_reserve.load();
  L.variant = g_variant[m->desc.kind][0].load();
  return L;
}

cudaError_t launch_trace(const TraceLaunch& L0, int precision, int src, int sink, cudaStream_t s) {
  if (L0.n > 0) counted();
  TraceLaunch L = L0;
  if (src == SRC_EQUATORIAL) L.variant = g_variant[L.M.kind][1].load();
  return precision == GEON_MIXED ? launch_trace_mixed(L, src, sink, s) : launch_trace_fp64(L, src, sink, s);
}

bool valid_precision(int p) { return p == GEON_FP64 || p == GEON_MIXED; }

// Levels of the speculative bisection tree traced per round: as many as keep
// nb * (2^L - 1) launch angles within 16384 rays (at most 16).
int64_t bisect_levels(size_t nb) {
  const int64_t target_rays = 16384;
  int L = 1;
  while (L < 16 && (int64_t)nb * ((1LL << (L + 1)) - 1) <= target_rays) ++L;
  return L;
}

int copy_out(void* host, const void* dev, size_t bytes, cudaStream_t s) {
  if (host && bytes) GEON_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s));
  return GEON_OK;
}

}  // namespace

// Helpers for other translation units of the ABI (added entry points reuse the
// handle, launch defaults, launch counter and error slot defined here).
namespace geon {
const MetricDesc* metric_desc(geon_metric_t m) { return m ? &m->desc : nullptr; }
TraceLaunch trace_launch_defaults(geon_metric_t m, double step, int64_t max_steps) {
  return base_launch(m, step, max_steps);
}
cudaError_t launch_trace_any(const TraceLaunch& L, int precision, int src, int sink, cudaStream_t s) {
  return launch_trace(L, precision, src, sink, s);
}
void note_launches(unsigned long long n) { counted(n); }
int set_last_error(int code, const char* msg) { return fail(code, msg); }
int bisect_levels_for(size_t nb) { return (int)bisect_levels(nb); }
}  // namespace geon

// Kernels defined in trace_fp64.cu used only from here.
namespace geon {
cudaError_t launch_camera_rays(const CameraDesc& c, double du, double dv, double* out, cudaStream_t s);
cudaError_t launch_equatorial_rays(double m, double r_obs, const double* alpha, int64_t n, double* out,
                                   cudaStream_t s);
}  // namespace geon

extern "C" {

const char* geon_version(void) { return "geon-gb300 0.1 (sm_103a)"; }

const char* geon_last_error(void) { return g_last_error.c_str(); }

void geon_render_config_default(geon_render_config* cfg) {
  if (!cfg) return;
  cfg->step = 0.05;
  cfg->max_steps = 20000;
  cfg->captured_rgb[0] = cfg->captured_rgb[1] = cfg->captured_rgb[2] = 0.0f;
  cfg->diverged_rgb[0] = 1.0f;
  cfg->diverged_rgb[1] = 0.0f;
  cfg->diverged_rgb[2] = 1.0f;
  cfg->samples_per_axis = 1;
  cfg->show_stars = -1;
  cfg->precision = GEON_FP64;
}

void geon_set_show_stars(int on) { g_show_stars.store(on ? 1 : 0); }

int geon_set_mixed_band(int kind, double band) {
  if (kind < GEON_MINKOWSKI || kind > GEON_MORRIS_THORNE || !(band >= 0.0))
    return fail(GEON_ERR_INVALID, "bad band");
  g_band[kind].store((float)band);
  return GEON_OK;
}

double geon_get_mixed_band(int kind) {
  if (kind < GEON_MINKOWSKI || kind > GEON_MORRIS_THORNE) return -1.0;
  return (double)g_band[kind].load();
}

void geon_set_mixed_reproject(int on) { g_reproject.store(on ? 1 : 0); }

void geon_set_persistent_reserve(int blocks_per_sm) { g_reserve.store(blocks_per_sm < 0 ? 0 : blocks_per_sm); }

int geon_set_mixed_variant(int kind, int source, int variant) {
  if (kind < GEON_MINKOWSKI || kind > GEON_MORRIS_THORNE || source < 0 || source > 1 || variant < 0 ||
      variant >= MIXED_VARIANTS)
    return fail(GEON_ERR_INVALID, "bad kind, source or variant");
  g_variant[kind][source].store(variant);
  return GEON_OK;
}

int geon_get_mixed_variant(int kind, int source) {
  if (kind < GEON_MINKOWSKI || kind > GEON_MORRIS_THORNE || source < 0 || source > 1) return GEON_ERR_INVALID;
  return g_variant[kind][source].load();
}

// Autotuner: time every register-cap variant of the mixed kernel on calibration
// jobs of this metric and keep the fastest per ray source:
//  source 0 (camera rays; also used for ray arrays): n camera rays of a
//    60-degree view from the metric's usual observer, step 0.05;
//  source 1 (equatorial shadow rays, Schwarzschild only): n launch angles
//    spread over [10, 20] degrees from r = 20M, step 0.01.
// Every ray is capped at max_steps. rates_out[2*3] receives ray-steps/s per
// (source, variant); best_out[2] the chosen variant per source (-1: not tuned).
static int time_variants(const TraceLaunch& base, int src, int sink, int64_t n, const int64_t* d_steps,
                         cudaStream_t s, double* rates, int* best) {
  cudaEvent_t a, b;
  GEON_CUDA(cudaEventCreate(&a));
  GEON_CUDA(cudaEventCreate(&b));
  double best_rate = -1.0;
  *best = 0;
  std::vector<int64_t> st(n);
  for (int v = 0; v < MIXED_VARIANTS; ++v) {
    TraceLaunch L = base;
    L.variant = v;
    float best_ms = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      GEON_CUDA(cudaMemsetAsync(L.queue, 0, sizeof(unsigned long long) * 2, s));
      GEON_CUDA(cudaEventRecord(a, s));
      counted();
      GEON_CUDA(launch_trace_mixed(L, src, sink, s));
      GEON_CUDA(cudaEventRecord(b, s));
      GEON_CUDA(cudaEventSynchronize(b));
      float ms = 0.0f;
      GEON_CUDA(cudaEventElapsedTime(&ms, a, b));
      if (ms < best_ms) best_ms = ms;
    }
    GEON_CUDA(cudaMemcpy(st.data(), d_steps, sizeof(int64_t) * n, cudaMemcpyDeviceToHost));
    double total = 0.0;
    for (int64_t q = 0; q < n; ++q) total += (double)st[q];
    const double rate = total / (best_ms * 1e-3);
    rates[v] = rate;
    if (rate > best_rate) {
      best_rate = rate;
      *best = v;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return GEON_OK;
}

int geon_autotune_mixed(geon_metric_t m, int64_t n_rays, int64_t max_steps, double* rates_out, int* best_out) {
  if (int rc = check_metric(m)) return rc;
  if (n_rays <= 0 || max_steps <= 0) return fail(GEON_ERR_INVALID, "bad calibration size");
  const int kind = m->desc.kind;
  double rates[6] = {0, 0, 0, 0, 0, 0};
  int best[2] = {0, -1};
  cudaStream_t s = host_stream();
  geon_camera cam;
  std::memset(&cam, 0, sizeof cam);
  const double r0 = kind == GEON_SCHWARZSCHILD ? 30.0 * m->desc.p[0] : 10.0;
  cam.observer[1] = kind == GEON_ALCUBIERRE ? -r0 : r0;
  cam.observer[2] = (kind == GEON_SCHWARZSCHILD || kind == GEON_MORRIS_THORNE) ? 1.5707963267948966 : 0.0;
  cam.fov_y_deg = 60.0;
  cam.width = 256;
  cam.height = (n_rays + 255) / 256;
  cam.forward_sign = kind == GEON_ALCUBIERRE ? -1 : 1;
  CameraDesc c;
  if (int rc = make_camera(m, &cam, 1, c, s)) return rc;
  const int64_t n = cam.width * cam.height;
  DBuf dsrgb, dterm, dsteps, dres, ws, dalpha;
  GEON_CUDA(dsrgb.alloc(sizeof(float) * 3 * n, s));
  GEON_CUDA(dterm.alloc(sizeof(int32_t) * n, s));
  GEON_CUDA(dsteps.alloc(sizeof(int64_t) * n, s));
  GEON_CUDA(dres.alloc(sizeof(double) * n, s));
  GEON_CUDA(ws.alloc(sizeof(unsigned long long) * 2, s));
  TraceLaunch L = base_launch(m, 0.05, max_steps);
  L.cam = c;
  L.n = n;
  L.term = dterm.as<int32_t>();
  L.steps = dsteps.as<int64_t>();
  L.resid = dres.as<double>();
  L.srgb = dsrgb.as<float>();
  L.show_stars = 1;
  L.queue = ws.as<unsigned long long>();
  L.flags = reinterpret_cast<int*>(L.queue + 1);
  if (int rc = time_variants(L, SRC_CAMERA, SINK_RENDER, n, dsteps.as<int64_t>(), s, rates, &best[0])) return rc;
  g_variant[kind][0].store(best[0]);
  if (kind == GEON_SCHWARZSCHILD) {
    std::vector<double> alpha(n);
    for (int64_t i = 0; i < n; ++i) alpha[i] = (10.0 + 10.0 * ((double)((i * 7919) % n) + 0.5) / (double)n) * RADS_PER_DEG;
    GEON_CUDA(dalpha.alloc(sizeof(double) * n, s));
    GEON_CUDA(cudaMemcpyAsync(dalpha.p, alpha.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    TraceLaunch E = base_launch(m, 0.01, max_steps);
    E.n = n;
    E.alpha = dalpha.as<double>();
    E.r_obs = 20.0 * m->desc.p[0];
    E.term = dterm.as<int32_t>();
    E.steps = dsteps.as<int64_t>();
    E.queue = ws.as<unsigned long long>();
    E.flags = reinterpret_cast<int*>(E.queue + 1);
    if (int rc = time_variants(E, SRC_EQUATORIAL, SINK_SHADOW, n, dsteps.as<int64_t>(), s, rates + 3, &best[1]))
      return rc;
    g_variant[kind][1].store(best[1]);
  }
  if (rates_out) std::memcpy(rates_out, rates, sizeof rates);
  if (best_out) {
    best_out[0] = best[0];
    best_out[1] = best[1];
  }
  return GEON_OK;
}

}  // extern "C"
