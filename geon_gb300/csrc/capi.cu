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
  double* field = nullptr;  // device copy of a sampled metric's nodes (GEON_FIELD)
};

namespace {

thread_local std::string g_last_error;
std::atomic<int> g_show_stars{1};
// Mixed-precision options: FP64 band half-width per metric kind (in units of
// M, b0, s; 0 disables) and the null re-projection switch.
std::atomic<float> g_band[4] = {{0.0f}, {0.0f}, {0.0f}, {0.0f}};
std::atomic<int> g_reproject{0};
std::atomic<int> g_orbit{1};  // orbit-plane frame of the mixed path (default on)
std::atomic<int> g_nullfix{1};  // compensated null re-projection every 16 steps (planar steps; default on)
std::atomic<int> g_sweep_order{1};  // longest-first claim order of shadow sweeps
std::atomic<float> g_reserve{0.0f};
std::atomic<double> g_rtol{1e-10};  // GEON_ADAPTIVE error tolerances
std::atomic<double> g_atol{1e-12};
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
  L.mixed_flags = (g_reproject.load() ? MIXED_REPROJECT : 0) | (g_orbit.load() ? MIXED_ORBIT : 0) |
                  (g_nullfix.load() ? MIXED_NULLFIX : 0);
  L.reserve_per_sm = g_reserve.load();
  L.variant = g_variant[m->desc.kind][0].load();
  L.rtol = g_rtol.load();
  L.atol = g_atol.load();
  return L;
}

cudaError_t launch_trace(const TraceLaunch& L0, int precision, int src, int sink, cudaStream_t s) {
  if (L0.n > 0) counted();
  TraceLaunch L = L0;
  if (src == SRC_EQUATORIAL) L.variant = g_variant[L.M.kind][1].load();
  if (precision == GEON_MIXED) return launch_trace_mixed(L, src, sink, s);
  if (precision == GEON_ADAPTIVE) return launch_trace_adaptive(L, src, sink, s);
  if (precision == GEON_FP64_FAST) return launch_trace_fp64fast(L, src, sink, s);
  return launch_trace_fp64(L, src, sink, s);
}

bool valid_precision(int p) {
  return p == GEON_FP64 || p == GEON_MIXED || p == GEON_ADAPTIVE || p == GEON_FP64_FAST;
}

// The precision is known and has a stepper for this metric.
int check_precision(geon_metric_t m, int p) {
  if (!valid_precision(p)) return fail(GEON_ERR_INVALID, "unknown precision");
  if (p == GEON_MIXED && m->desc.kind == GEON_FIELD)
    return fail(GEON_ERR_UNSUPPORTED, "the mixed-precision path has no stepper for a sampled metric");
  return GEON_OK;
}

// Levels of the speculative bisection tree traced per round: as many as keep
// nb * (2^L - 1) launch angles within target_rays (at most 16).
int64_t bisect_levels_target(size_t nb, int64_t target_rays) {
  int L = 1;
  while (L < 16 && (int64_t)nb * ((1LL << (L + 1)) - 1) <= target_rays) ++L;
  return L;
}

constexpr int64_t BISECT_RAYS_DEFAULT = 16384;
std::atomic<int64_t> g_bisect_rays{BISECT_RAYS_DEFAULT};

int64_t bisect_levels(size_t nb) { return bisect_levels_target(nb, g_bisect_rays.load()); }

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
int bisect_levels_for(size_t nb) { return (int)bisect_levels_target(nb, BISECT_RAYS_DEFAULT); }
int camera_desc_for(geon_metric_t m, const geon_camera* cam, int64_t spa, CameraDesc& c, cudaStream_t s) {
  return make_camera(m, cam, spa, c, s);
}
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
void geon_set_mixed_orbit_plane(int on) { g_orbit.store(on ? 1 : 0); }
void geon_set_mixed_null_fix(int on) { g_nullfix.store(on ? 1 : 0); }
void geon_set_sweep_order(int on) { g_sweep_order.store(on ? 1 : 0); }
int geon_get_sweep_order(void) { return g_sweep_order.load(); }
int geon_get_mixed_null_fix(void) { return g_nullfix.load(); }
int geon_get_mixed_orbit_plane(void) { return g_orbit.load(); }

int geon_set_bisect_rays_per_round(int64_t rays) {
  if (rays < 1 || rays > ((int64_t)1 << 24)) return fail(GEON_ERR_INVALID, "rays per round out of range");
  g_bisect_rays.store(rays);
  return GEON_OK;
}

int64_t geon_get_bisect_rays_per_round(void) { return g_bisect_rays.load(); }

int geon_set_adaptive_tolerance(double rtol, double atol) {
  if (!(rtol >= 0.0) || !(atol >= 0.0) || (rtol == 0.0 && atol == 0.0) || !std::isfinite(rtol) ||
      !std::isfinite(atol))
    return fail(GEON_ERR_INVALID, "bad tolerances");
  g_rtol.store(rtol);
  g_atol.store(atol);
  return GEON_OK;
}

void geon_get_adaptive_tolerance(double* rtol, double* atol) {
  if (rtol) *rtol = g_rtol.load();
  if (atol) *atol = g_atol.load();
}

void geon_set_persistent_reserve(int blocks_per_sm) { geon_set_persistent_reserve_f((double)blocks_per_sm); }
void geon_set_persistent_reserve_f(double blocks_per_sm) {
  g_reserve.store(blocks_per_sm > 0.0 ? (float)blocks_per_sm : 0.0f);  // NaN and negatives: none
}

int geon_set_mixed_variant(int kind, int source, int variant) {
  if (kind < GEON_MINKOWSKI || kind > GEON_MORRIS_THORNE || source < 0 || source > 1 || variant < 0 ||
      variant >= (source == 1 ? MIXED_VARIANTS : MIXED_CAPS))
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
//  source 0 (camera rays, as the render's trace kernel steps them; also used
//    for ray arrays): n camera rays of a 60-degree view from the metric's usual
//    observer, step 0.05;
//  source 1 (equatorial shadow rays, Schwarzschild only): n launch angles
//    spread over [10, 20] degrees from r = 20M, step 0.01.
// Every ray is capped at max_steps. rates_out[3 + 9] receives ray-steps/s per
// (source, variant): 3 register caps for source 0, then 9 (cap + 3 x block size
// 128/64/256) for source 1; best_out[2] the chosen variant per source (-1: not
// tuned).
static int time_variants(const TraceLaunch& base, int src, int sink, int64_t n, const int64_t* d_steps,
                         cudaStream_t s, double* rates, int* best, int nvariants) {
  cudaEvent_t a, b;
  GEON_CUDA(cudaEventCreate(&a));
  GEON_CUDA(cudaEventCreate(&b));
  double best_rate = -1.0;
  *best = 0;
  std::vector<int64_t> st(n);
  for (int v = 0; v < nvariants; ++v) {
    TraceLaunch L = base;
    L.variant = v;
    float best_ms = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      GEON_CUDA(cudaMemsetAsync(L.queue, 0, sizeof(unsigned long long) * 2, s));
      if (src == SRC_STATE) {  // the states are traced in place: prepare them again, untimed
        counted();
        GEON_CUDA(launch_render_prepare(L, s));
      }
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
  if (m->desc.kind == GEON_FIELD) return fail(GEON_ERR_UNSUPPORTED, "no mixed-precision stepper for a sampled metric");
  if (n_rays < 0 || max_steps <= 0) return fail(GEON_ERR_INVALID, "bad calibration size");
  if (n_rays == 0) {
    // four rays per lane of the largest variant's grid: occupancy decides the
    // rate only when every lane has work for most of the launch
    int dev = 0, sms = 0;
    GEON_CUDA(cudaGetDevice(&dev));
    GEON_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    n_rays = (int64_t)sms * 6 * 128 * 4;  // 128 threads per trace block
  }
  const int kind = m->desc.kind;
  double rates[MIXED_CAPS + MIXED_VARIANTS] = {};
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
  DBuf dsrgb, dterm, dsteps, dres, ws, dalpha, dstate;
  GEON_CUDA(dsrgb.alloc(sizeof(float) * 3 * n, s));
  GEON_CUDA(dstate.alloc(sizeof(uint32_t) * 16 * n, s));
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
  L.ystate = dstate.as<uint32_t>();
  // the trace kernel of the three-kernel render (camera rays prepared, states out)
  if (int rc = time_variants(L, SRC_STATE, SINK_STATE, n, dsteps.as<int64_t>(), s, rates, &best[0], MIXED_CAPS))
    return rc;
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
    if (int rc = time_variants(E, SRC_EQUATORIAL, SINK_SHADOW, n, dsteps.as<int64_t>(), s, rates + MIXED_CAPS,
                               &best[1], MIXED_VARIANTS))
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


int geon_get_show_stars(void) { return g_show_stars.load(); }

int geon_metric_create(int kind, const double* params, int nparams, geon_metric_t* out) {
  if (!out) return fail(GEON_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (kind < GEON_MINKOWSKI || kind > GEON_MORRIS_THORNE) return fail(GEON_ERR_INVALID, "unknown metric kind");
  if (nparams < 0 || (nparams > 0 && !params)) return fail(GEON_ERR_INVALID, "bad params");
  MetricDesc d;
  std::memset(&d, 0, sizeof d);
  d.kind = kind;
  // Reference defaults: Schwarzschild::new (schwarzschild.rs:20-28), Alcubierre::default
  // (alcubierre.rs:21-30), MorrisThorne::default (morris_thorne.rs:15-18).
  static const double defaults[4][4] = {{0, 0, 0, 0}, {1.0, 1.001, 1000.0, 0}, {2.0, 0.5, 2.0, 0.0}, {1.0, 0, 0, 0}};
  static const int counts[4] = {0, 3, 4, 1};
  if (nparams > counts[kind]) return fail(GEON_ERR_INVALID, "too many params for this metric");
  for (int i = 0; i < 4; ++i) d.p[i] = i < nparams ? params[i] : defaults[kind][i];
  if (kind == GEON_SCHWARZSCHILD) {
    d.capture_r = d.p[1] * 2.0 * d.p[0];
    d.escape_r = d.p[2] * d.p[0];
  }
  if (kind == GEON_ALCUBIERRE) {
    cudaStream_t s = host_stream();
    DBuf b;
    GEON_CUDA(b.alloc(sizeof(MetricDesc), s));
    GEON_CUDA(cudaMemcpyAsync(b.p, &d, sizeof d, cudaMemcpyHostToDevice, s));
    counted();
  GEON_CUDA(launch_metric_init(b.as<MetricDesc>(), s));
    GEON_CUDA(cudaMemcpyAsync(&d, b.p, sizeof d, cudaMemcpyDeviceToHost, s));
    GEON_CUDA(cudaStreamSynchronize(s));
  }
  geon_metric* m = new (std::nothrow) geon_metric;
  if (!m) return fail(GEON_ERR_OOM, "out of host memory");
  m->desc = d;
  *out = m;
  return GEON_OK;
}

int geon_metric_create_field(const geon_grid* grid, const double* samples, int chart, geon_metric_t* out) {
  if (!out) return fail(GEON_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!grid || !samples) return fail(GEON_ERR_INVALID, "null grid or samples");
  if (chart != GEON_CHART_CARTESIAN && chart != GEON_CHART_SPHERICAL) return fail(GEON_ERR_INVALID, "unknown chart");
  MetricDesc d;
  std::memset(&d, 0, sizeof d);
  d.kind = GEON_FIELD;
  int64_t nodes = 1;
  for (int a = 0; a < 3; ++a) {
    if (grid->n[a] < 1 || grid->n[a] > (int64_t)1 << 30) return fail(GEON_ERR_INVALID, "bad grid size");
    if (!std::isfinite(grid->lo[a]) || !std::isfinite(grid->hi[a]) || (grid->n[a] > 1 && !(grid->hi[a] > grid->lo[a])))
      return fail(GEON_ERR_INVALID, "bad grid extent");
    d.f.lo[a] = grid->lo[a];
    d.f.hi[a] = grid->hi[a];
    d.f.n[a] = grid->n[a];
    d.f.inv_d[a] = grid->n[a] > 1 ? (double)(grid->n[a] - 1) / (grid->hi[a] - grid->lo[a]) : 0.0;
    nodes *= grid->n[a];
  }
  d.f.chart = chart;
  geon_metric* m = new (std::nothrow) geon_metric;
  if (!m) return fail(GEON_ERR_OOM, "out of host memory");
  const size_t bytes = sizeof(double) * 10 * (size_t)nodes;
  cudaError_t e = cudaMalloc(&m->field, bytes);
  if (e == cudaSuccess) e = cudaMemcpy(m->field, samples, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (m->field) cudaFree(m->field);
    delete m;
    return fail(e == cudaErrorMemoryAllocation ? GEON_ERR_OOM : GEON_ERR_CUDA, cudaGetErrorString(e));
  }
  d.f.c = m->field;
  m->desc = d;
  *out = m;
  return GEON_OK;
}

int geon_metric_destroy(geon_metric_t m) {
  if (m && m->field) cudaFree(m->field);
  delete m;
  return GEON_OK;
}

int geon_metric_kind(geon_metric_t m) { return m ? m->desc.kind : GEON_ERR_INVALID; }

const char* geon_metric_name(geon_metric_t m) {
  static const char* names[5] = {"minkowski", "schwarzschild", "alcubierre", "morris_thorne", "field"};
  return m ? names[m->desc.kind] : "";
}

static int pointwise(geon_metric_t m, int what, const double* in, size_t n, int in_width, double* out,
                     int out_width, int32_t* iout) {
  if (int rc = check_metric(m)) return rc;
  if (n == 0) return GEON_OK;
  if (!in || (!out && !iout)) return fail(GEON_ERR_INVALID, "null buffer");
  cudaStream_t s = host_stream();
  DBuf din, dout, dflags;
  GEON_CUDA(din.alloc(sizeof(double) * n * in_width, s));
  GEON_CUDA(dout.alloc(out ? sizeof(double) * n * out_width : sizeof(int32_t) * n, s));
  GEON_CUDA(dflags.alloc(sizeof(int), s));
  GEON_CUDA(cudaMemsetAsync(dflags.p, 0, sizeof(int), s));
  GEON_CUDA(cudaMemcpyAsync(din.p, in, sizeof(double) * n * in_width, cudaMemcpyHostToDevice, s));
  counted();
  GEON_CUDA(launch_pointwise(m->desc, what, din.as<double>(), (int64_t)n, out ? dout.as<double>() : nullptr,
                             out ? nullptr : dout.as<int32_t>(), dflags.as<int>(), s));
  if (out) GEON_CUDA(cudaMemcpyAsync(out, dout.p, sizeof(double) * n * out_width, cudaMemcpyDeviceToHost, s));
  else GEON_CUDA(cudaMemcpyAsync(iout, dout.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  int flags = 0;
  if (int rc = sync_and_flags(s, dflags.as<int>(), &flags)) return rc;
  return singular_status(flags);
}

int geon_metric_g(geon_metric_t m, const double* x, size_t n, double* out) { return pointwise(m, PW_G, x, n, 4, out, 16, nullptr); }
int geon_metric_dg(geon_metric_t m, const double* x, size_t n, double* out) { return pointwise(m, PW_DG, x, n, 4, out, 64, nullptr); }
int geon_metric_g_inv(geon_metric_t m, const double* x, size_t n, double* out) { return pointwise(m, PW_GINV, x, n, 4, out, 16, nullptr); }
int geon_metric_christoffel(geon_metric_t m, const double* x, size_t n, double* out) { return pointwise(m, PW_CHRISTOFFEL, x, n, 4, out, 64, nullptr); }
int geon_metric_terminate(geon_metric_t m, const double* x, size_t n, int32_t* out) { return pointwise(m, PW_TERMINATE, x, n, 4, nullptr, 0, out); }
int geon_metric_asymptotic_direction(geon_metric_t m, const double* st, size_t n, double* out) { return pointwise(m, PW_ASYM, st, n, 8, out, 3, nullptr); }

int geon_trace_dev(geon_metric_t m, const double* y0, size_t n, double step, int64_t max_steps, int precision,
                   int32_t* term, double* final_state, int64_t* steps_taken, double* null_residual,
                   void* stream) {
  if (int rc = check_metric(m)) return rc;
  if (int rc = check_precision(m, precision)) return rc;
  if (n == 0) return GEON_OK;
  if (!y0 || !term || !final_state || !steps_taken || !null_residual)
    return fail(GEON_ERR_INVALID, "geon_trace_dev needs every device buffer");
  if (max_steps < 0) return fail(GEON_ERR_INVALID, "max_steps < 0");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DBuf ws;
  GEON_CUDA(ws.alloc(sizeof(unsigned long long) + sizeof(int) * 2, s));
  GEON_CUDA(cudaMemsetAsync(ws.p, 0, sizeof(unsigned long long) + sizeof(int) * 2, s));
  TraceLaunch L = base_launch(m, step, max_steps);
  L.n = (int64_t)n;
  L.y0 = y0;
  L.term = term;
  L.yfinal = final_state;
  L.steps = steps_taken;
  L.resid = null_residual;
  L.queue = ws.as<unsigned long long>();
  L.flags = reinterpret_cast<int*>(L.queue + 1);
  GEON_CUDA(launch_trace(L, precision, SRC_ARRAY, SINK_TRACE, s));
  return GEON_OK;
}

int geon_trace(geon_metric_t m, const double* y0, size_t n, double step, int64_t max_steps, int precision,
               int32_t* term, double* final_state, int64_t* steps_taken, double* null_residual) {
  if (int rc = check_metric(m)) return rc;
  if (int rc = check_precision(m, precision)) return rc;
  if (n == 0) return GEON_OK;
  if (!y0 || !term) return fail(GEON_ERR_INVALID, "null buffer");
  if (max_steps < 0) return fail(GEON_ERR_INVALID, "max_steps < 0");
  cudaStream_t s = host_stream();
  DBuf dy0, dterm, dyf, dsteps, dres, ws;
  GEON_CUDA(dy0.alloc(sizeof(double) * 8 * n, s));
  GEON_CUDA(dterm.alloc(sizeof(int32_t) * n, s));
  GEON_CUDA(dyf.alloc(sizeof(double) * 8 * n, s));
  GEON_CUDA(dsteps.alloc(sizeof(int64_t) * n, s));
  GEON_CUDA(dres.alloc(sizeof(double) * n, s));
  GEON_CUDA(ws.alloc(sizeof(unsigned long long) + sizeof(int) * 2, s));
  GEON_CUDA(cudaMemsetAsync(ws.p, 0, sizeof(unsigned long long) + sizeof(int) * 2, s));
  GEON_CUDA(cudaMemcpyAsync(dy0.p, y0, sizeof(double) * 8 * n, cudaMemcpyHostToDevice, s));
  TraceLaunch L = base_launch(m, step, max_steps);
  L.n = (int64_t)n;
  L.y0 = dy0.as<double>();
  L.term = dterm.as<int32_t>();
  L.yfinal = dyf.as<double>();
  L.steps = dsteps.as<int64_t>();
  L.resid = dres.as<double>();
  L.queue = ws.as<unsigned long long>();
  L.flags = reinterpret_cast<int*>(L.queue + 1);
  GEON_CUDA(launch_trace(L, precision, SRC_ARRAY, SINK_TRACE, s));
  if (int rc = copy_out(term, dterm.p, sizeof(int32_t) * n, s)) return rc;
  if (int rc = copy_out(final_state, dyf.p, sizeof(double) * 8 * n, s)) return rc;
  if (int rc = copy_out(steps_taken, dsteps.p, sizeof(int64_t) * n, s)) return rc;
  if (int rc = copy_out(null_residual, dres.p, sizeof(double) * n, s)) return rc;
  int flags = 0;
  if (int rc = sync_and_flags(s, L.flags, &flags)) return rc;
  return singular_status(flags);
}

int geon_camera_tetrad(geon_metric_t m, const double observer[4], double out_tetrad[16]) {
  if (int rc = check_metric(m)) return rc;
  if (!observer || !out_tetrad) return fail(GEON_ERR_INVALID, "null buffer");
  geon_camera cam;
  std::memset(&cam, 0, sizeof cam);
  std::memcpy(cam.observer, observer, sizeof cam.observer);
  cam.fov_y_deg = 60.0;
  cam.width = cam.height = 1;
  cam.forward_sign = 1;
  CameraDesc c;
  if (int rc = make_camera(m, &cam, 1, c, host_stream())) return rc;
  std::memcpy(out_tetrad, c.tet, sizeof c.tet);
  return GEON_OK;
}

int geon_camera_ray_states(const geon_camera* cam, const double tetrad[16], double du, double dv,
                           double* out_states) {
  if (!cam || !tetrad || !out_states || cam->width <= 0 || cam->height <= 0)
    return fail(GEON_ERR_INVALID, "bad camera arguments");
  if (cam->forward_sign != 1 && cam->forward_sign != -1) return fail(GEON_ERR_INVALID, "forward_sign must be +1 or -1");
  CameraDesc c;
  std::memcpy(c.tet, tetrad, sizeof c.tet);
  std::memcpy(c.obs, cam->observer, sizeof c.obs);
  const double fov = cam->fov_y_deg * RADS_PER_DEG;
  const double aspect = (double)cam->width / (double)cam->height;
  c.h_img = std::tan(fov * 0.5);
  c.w_img = c.h_img * aspect;
  c.width_d = (double)cam->width;
  c.height_d = (double)cam->height;
  c.width = cam->width;
  c.height = cam->height;
  c.spa = 1;
  c.inv_spa = 1.0;
  c.forward_sign = cam->forward_sign;
  const size_t n = (size_t)(cam->width * cam->height);
  cudaStream_t s = host_stream();
  DBuf d;
  GEON_CUDA(d.alloc(sizeof(double) * 8 * n, s));
  counted();
  GEON_CUDA(launch_camera_rays(c, du, dv, d.as<double>(), s));
  GEON_CUDA(cudaMemcpyAsync(out_states, d.p, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost, s));
  GEON_CUDA(cudaStreamSynchronize(s));
  return GEON_OK;
}

// render() with its f32 image (rgb) and/or write_png's tonemapped bytes (rgb8).
static int render_any(geon_metric_t m, const geon_camera* cam, const geon_render_config* cfg, float* rgb,
                      uint8_t* rgb8, geon_render_stats* stats, int32_t* pixel_class, int64_t* pixel_steps) {
  if (int rc = check_metric(m)) return rc;
  if (!cfg || (!rgb && !rgb8)) return fail(GEON_ERR_INVALID, "null buffer");
  if (int rc = check_precision(m, cfg->precision)) return rc;
  if (cfg->max_steps < 0) return fail(GEON_ERR_INVALID, "max_steps < 0");
  cudaStream_t s = host_stream();
  const int64_t spa = cfg->samples_per_axis < 1 ? 1 : cfg->samples_per_axis;
  CameraDesc c;
  if (int rc = make_camera(m, cam, spa, c, s)) return rc;
  const int64_t npix = cam->width * cam->height;
  const int64_t nsamp = npix * spa * spa;
  DBuf dsrgb, dterm, dsteps, dres, drgb, dcls, dpst, ws, dstate;
  GEON_CUDA(dsrgb.alloc(sizeof(float) * 3 * nsamp, s));
  GEON_CUDA(dterm.alloc(sizeof(int32_t) * nsamp, s));
  GEON_CUDA(dsteps.alloc(sizeof(int64_t) * nsamp, s));
  GEON_CUDA(dres.alloc(sizeof(double) * nsamp, s));
  GEON_CUDA(drgb.alloc(sizeof(float) * 3 * npix, s));
  GEON_CUDA(dcls.alloc(sizeof(int32_t) * npix + (rgb8 ? 3 * npix : 0), s));  // + the bytes of rgb8
  GEON_CUDA(dpst.alloc(sizeof(int64_t) * npix, s));
  const size_t ws_bytes = sizeof(unsigned long long) * 8;
  GEON_CUDA(ws.alloc(ws_bytes, s));
  GEON_CUDA(cudaMemsetAsync(ws.p, 0, ws_bytes, s));
  TraceLaunch L = base_launch(m, cfg->step, cfg->max_steps);
  L.cam = c;
  L.n = nsamp;
  L.term = dterm.as<int32_t>();
  L.steps = dsteps.as<int64_t>();
  L.resid = dres.as<double>();
  L.srgb = dsrgb.as<float>();
  L.show_stars = cfg->show_stars < 0 ? g_show_stars.load() : (cfg->show_stars != 0);
  for (int q = 0; q < 3; ++q) {
    L.captured_rgb[q] = cfg->captured_rgb[q];
    L.diverged_rgb[q] = cfg->diverged_rgb[q];
  }
  unsigned long long* wsu = ws.as<unsigned long long>();
  L.queue = wsu;
  L.flags = reinterpret_cast<int*>(wsu + 1);
  unsigned long long* dstats = wsu + 2;  // 6 counters
  if (cfg->precision == GEON_MIXED) {
    // prepare / trace / shade (launch_render_mixed): 16 words of state per sample
    GEON_CUDA(dstate.alloc(sizeof(uint32_t) * 16 * nsamp, s));
    L.ystate = dstate.as<uint32_t>();
    counted(3);
    GEON_CUDA(launch_render_mixed(L, s));
  } else {
    GEON_CUDA(launch_trace(L, cfg->precision, SRC_CAMERA, SINK_RENDER, s));
  }
  counted();
  uint8_t* d8 = rgb8 ? reinterpret_cast<uint8_t*>(dcls.as<int32_t>() + npix) : nullptr;
  GEON_CUDA(launch_render_reduce(dsrgb.as<float>(), dterm.as<int32_t>(), dsteps.as<int64_t>(),
                                 dres.as<double>(), npix, spa, rgb ? drgb.as<float>() : nullptr,
                                 dcls.as<int32_t>(), dpst.as<int64_t>(), dstats, s, d8));
  unsigned long long hst[6];
  if (rgb) GEON_CUDA(cudaMemcpyAsync(rgb, drgb.p, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost, s));
  if (rgb8) GEON_CUDA(cudaMemcpyAsync(rgb8, d8, 3 * npix, cudaMemcpyDeviceToHost, s));
  if (int rc = copy_out(pixel_class, dcls.p, sizeof(int32_t) * npix, s)) return rc;
  if (int rc = copy_out(pixel_steps, dpst.p, sizeof(int64_t) * npix, s)) return rc;
  GEON_CUDA(cudaMemcpyAsync(hst, dstats, sizeof hst, cudaMemcpyDeviceToHost, s));
  int flags = 0;
  if (int rc = sync_and_flags(s, L.flags, &flags)) return rc;
  if (stats) {
    stats->captured = (int64_t)hst[0];
    stats->escaped = (int64_t)hst[1];
    stats->diverged = (int64_t)hst[2];
    double mr;
    std::memcpy(&mr, &hst[4], sizeof mr);
    stats->max_null_residual = mr;
    stats->avg_steps = (double)(int64_t)hst[3] / (double)npix;
    stats->total_steps = (int64_t)hst[5];
  }
  return singular_status(flags);
}

int geon_render_ex(geon_metric_t m, const geon_camera* cam, const geon_render_config* cfg, float* rgb,
                   geon_render_stats* stats, int32_t* pixel_class, int64_t* pixel_steps) {
  if (!rgb) return fail(GEON_ERR_INVALID, "null buffer");
  return render_any(m, cam, cfg, rgb, nullptr, stats, pixel_class, pixel_steps);
}

int geon_render(geon_metric_t m, const geon_camera* cam, const geon_render_config* cfg, float* rgb,
                geon_render_stats* stats) {
  return geon_render_ex(m, cam, cfg, rgb, stats, nullptr, nullptr);
}

int geon_render_u8(geon_metric_t m, const geon_camera* cam, const geon_render_config* cfg, uint8_t* rgb8,
                   float* rgb, geon_render_stats* stats) {
  if (!rgb8) return fail(GEON_ERR_INVALID, "null buffer");
  return render_any(m, cam, cfg, rgb, rgb8, stats, nullptr, nullptr);
}

int geon_render_batch(const geon_render_item* items, size_t n) {
  if (n == 0) return GEON_OK;
  if (!items || n > (size_t)MULTI_MAX_JOBS) return fail(GEON_ERR_INVALID, "geon_render_batch takes 1 to 8 items");
  const int precision = items[0].render.precision;
  if (precision != GEON_FP64 && precision != GEON_MIXED)
    return fail(GEON_ERR_INVALID, "geon_render_batch runs GEON_FP64 or GEON_MIXED");
  for (size_t j = 0; j < n; ++j) {
    const geon_render_item& it = items[j];
    if (int rc = check_metric(it.metric)) return rc;
    if (it.render.precision != precision) return fail(GEON_ERR_INVALID, "every item of a batch needs one precision");
    if (it.metric->desc.kind == GEON_FIELD) return fail(GEON_ERR_UNSUPPORTED, "geon_render_batch: no sampled metrics");
    if (!it.rgb) return fail(GEON_ERR_INVALID, "null buffer");
    if (it.render.max_steps < 0) return fail(GEON_ERR_INVALID, "max_steps < 0");
  }
  cudaStream_t s = host_stream();
  if (precision == GEON_MIXED && (g_reproject.load() || g_band[GEON_SCHWARZSCHILD].load() > 0.0f ||
                                  g_band[GEON_ALCUBIERRE].load() > 0.0f || g_band[GEON_MORRIS_THORNE].load() > 0.0f))
    return fail(GEON_ERR_UNSUPPORTED, "geon_render_batch runs the default mixed step (no FP64 band, no re-projection)");
  struct Bufs {
    DBuf srgb, term, steps, res, rgb, cls, pst, state;
    int64_t npix = 0, spa = 1;
  };
  std::vector<Bufs> B(n);
  std::vector<TraceLaunch> jobs(n);
  MultiDesc D;
  std::memset(&D, 0, sizeof D);
  D.njobs = (int)n;
  DBuf ws, djobs;
  const size_t ws_bytes = sizeof(unsigned long long) * (2 + 6 * n);
  GEON_CUDA(ws.alloc(ws_bytes, s));
  GEON_CUDA(cudaMemsetAsync(ws.p, 0, ws_bytes, s));
  unsigned long long* wsu = ws.as<unsigned long long>();
  for (size_t j = 0; j < n; ++j) {
    const geon_render_item& it = items[j];
    Bufs& b = B[j];
    b.spa = it.render.samples_per_axis < 1 ? 1 : it.render.samples_per_axis;
    CameraDesc c;
    if (int rc = make_camera(it.metric, &it.camera, b.spa, c, s)) return rc;
    b.npix = it.camera.width * it.camera.height;
    const int64_t nsamp = b.npix * b.spa * b.spa;
    GEON_CUDA(b.srgb.alloc(sizeof(float) * 3 * nsamp, s));
    GEON_CUDA(b.term.alloc(sizeof(int32_t) * nsamp, s));
    GEON_CUDA(b.steps.alloc(sizeof(int64_t) * nsamp, s));
    GEON_CUDA(b.res.alloc(sizeof(double) * nsamp, s));
    GEON_CUDA(b.rgb.alloc(sizeof(float) * 3 * b.npix, s));
    GEON_CUDA(b.cls.alloc(sizeof(int32_t) * b.npix, s));
    GEON_CUDA(b.pst.alloc(sizeof(int64_t) * b.npix, s));
    TraceLaunch L = base_launch(it.metric, it.render.step, it.render.max_steps);
    L.cam = c;
    L.n = nsamp;
    L.term = b.term.as<int32_t>();
    L.steps = b.steps.as<int64_t>();
    L.resid = b.res.as<double>();
    L.srgb = b.srgb.as<float>();
    L.show_stars = it.render.show_stars < 0 ? g_show_stars.load() : (it.render.show_stars != 0);
    for (int q = 0; q < 3; ++q) {
      L.captured_rgb[q] = it.render.captured_rgb[q];
      L.diverged_rgb[q] = it.render.diverged_rgb[q];
    }
    L.queue = wsu;
    L.flags = reinterpret_cast<int*>(wsu + 1);
    if (precision == GEON_MIXED) {
      GEON_CUDA(b.state.alloc(sizeof(uint32_t) * 16 * nsamp, s));
      L.ystate = b.state.as<uint32_t>();
      counted();
      GEON_CUDA(launch_render_prepare(L, s));
    }
    jobs[j] = L;
    D.start[j + 1] = D.start[j] + nsamp;
    D.kind_mask |= 1 << L.M.kind;
  }
  D.queue = wsu;
  GEON_CUDA(djobs.alloc(sizeof(TraceLaunch) * n, s));
  GEON_CUDA(cudaMemcpyAsync(djobs.p, jobs.data(), sizeof(TraceLaunch) * n, cudaMemcpyHostToDevice, s));
  counted();
  if (precision == GEON_MIXED) GEON_CUDA(launch_trace_multi_mixed(djobs.as<TraceLaunch>(), D, g_reserve.load(), s));
  else GEON_CUDA(launch_trace_multi_fp64(djobs.as<TraceLaunch>(), D, g_reserve.load(), s));
  std::vector<unsigned long long> hst(6 * n);
  for (size_t j = 0; j < n; ++j) {
    const geon_render_item& it = items[j];
    Bufs& b = B[j];
    unsigned long long* dstats = wsu + 2 + 6 * j;
    if (precision == GEON_MIXED) {
      counted();
      GEON_CUDA(launch_render_shade(jobs[j], s));
    }
    counted();
    GEON_CUDA(launch_render_reduce(b.srgb.as<float>(), b.term.as<int32_t>(), b.steps.as<int64_t>(),
                                   b.res.as<double>(), b.npix, b.spa, b.rgb.as<float>(), b.cls.as<int32_t>(),
                                   b.pst.as<int64_t>(), dstats, s));
    GEON_CUDA(cudaMemcpyAsync(it.rgb, b.rgb.p, sizeof(float) * 3 * b.npix, cudaMemcpyDeviceToHost, s));
    if (int rc = copy_out(it.pixel_class, b.cls.p, sizeof(int32_t) * b.npix, s)) return rc;
    if (int rc = copy_out(it.pixel_steps, b.pst.p, sizeof(int64_t) * b.npix, s)) return rc;
    GEON_CUDA(cudaMemcpyAsync(&hst[6 * j], dstats, sizeof(unsigned long long) * 6, cudaMemcpyDeviceToHost, s));
  }
  int flags = 0;
  if (int rc = sync_and_flags(s, reinterpret_cast<int*>(wsu + 1), &flags)) return rc;
  for (size_t j = 0; j < n; ++j) {
    geon_render_stats* st = items[j].stats;
    if (!st) continue;
    const unsigned long long* h = &hst[6 * j];
    st->captured = (int64_t)h[0];
    st->escaped = (int64_t)h[1];
    st->diverged = (int64_t)h[2];
    double mr;
    std::memcpy(&mr, &h[4], sizeof mr);
    st->max_null_residual = mr;
    st->avg_steps = (double)(int64_t)h[3] / (double)B[j].npix;
    st->total_steps = (int64_t)h[5];
  }
  return singular_status(flags);
}

int geon_tonemap_u8_dev(const float* rgb, size_t n, uint8_t* out, void* stream) {
  if (n == 0) return GEON_OK;
  if (!rgb || !out) return fail(GEON_ERR_INVALID, "null buffer");
  counted();
  GEON_CUDA(launch_tonemap(rgb, (int64_t)n, out, static_cast<cudaStream_t>(stream)));
  return GEON_OK;
}

int geon_tonemap_u8(const float* rgb, size_t n, uint8_t* out) {
  if (n == 0) return GEON_OK;
  if (!rgb || !out) return fail(GEON_ERR_INVALID, "null buffer");
  cudaStream_t s = host_stream();
  DBuf d;
  GEON_CUDA(d.alloc(sizeof(float) * n + n, s));
  uint8_t* d8 = reinterpret_cast<uint8_t*>(d.as<float>() + n);
  GEON_CUDA(cudaMemcpyAsync(d.p, rgb, sizeof(float) * n, cudaMemcpyHostToDevice, s));
  counted();
  GEON_CUDA(launch_tonemap(d.as<float>(), (int64_t)n, d8, s));
  GEON_CUDA(cudaMemcpyAsync(out, d8, n, cudaMemcpyDeviceToHost, s));
  GEON_CUDA(cudaStreamSynchronize(s));
  return GEON_OK;
}

int geon_sky_sample(const double* dir, size_t n, int show_stars, float* rgb) {
  if (n == 0) return GEON_OK;
  if (!dir || !rgb) return fail(GEON_ERR_INVALID, "null buffer");
  cudaStream_t s = host_stream();
  DBuf dd, dr;
  GEON_CUDA(dd.alloc(sizeof(double) * 3 * n, s));
  GEON_CUDA(dr.alloc(sizeof(float) * 3 * n, s));
  GEON_CUDA(cudaMemcpyAsync(dd.p, dir, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  counted();
  GEON_CUDA(launch_sky(dd.as<double>(), (int64_t)n, show_stars, dr.as<float>(), s));
  GEON_CUDA(cudaMemcpyAsync(rgb, dr.p, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s));
  GEON_CUDA(cudaStreamSynchronize(s));
  return GEON_OK;
}

static int curvature_call(geon_metric_t m, int what, const double* x, size_t n, const double* k, size_t nk,
                          int k_shared, double* out, int out_width) {
  if (int rc = check_metric(m)) return rc;
  if (n == 0) return GEON_OK;
  if (!x || !out) return fail(GEON_ERR_INVALID, "null buffer");
  cudaStream_t s = host_stream();
  DBuf dx, dk, dout, dflags;
  const size_t kcount = what == 5 ? (k_shared ? nk : nk * n) : 0;
  GEON_CUDA(dx.alloc(sizeof(double) * 4 * n, s));
  GEON_CUDA(dk.alloc(sizeof(double) * 4 * kcount, s));
  GEON_CUDA(dout.alloc(sizeof(double) * n * out_width, s));
  GEON_CUDA(dflags.alloc(sizeof(int), s));
  GEON_CUDA(cudaMemsetAsync(dflags.p, 0, sizeof(int), s));
  GEON_CUDA(cudaMemcpyAsync(dx.p, x, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, s));
  if (kcount) GEON_CUDA(cudaMemcpyAsync(dk.p, k, sizeof(double) * 4 * kcount, cudaMemcpyHostToDevice, s));
  counted();
  GEON_CUDA(launch_curvature(m->desc, what, dx.as<double>(), (int64_t)n, dk.as<double>(), (int64_t)nk,
                             k_shared, dout.as<double>(), dflags.as<int>(), s));
  GEON_CUDA(cudaMemcpyAsync(out, dout.p, sizeof(double) * n * out_width, cudaMemcpyDeviceToHost, s));
  int flags = 0;
  if (int rc = sync_and_flags(s, dflags.as<int>(), &flags)) return rc;
  return singular_status(flags);
}

int geon_riemann(geon_metric_t m, const double* x, size_t n, double* out) { return curvature_call(m, 0, x, n, nullptr, 0, 1, out, 256); }
int geon_ricci(geon_metric_t m, const double* x, size_t n, double* out) { return curvature_call(m, 1, x, n, nullptr, 0, 1, out, 16); }
int geon_ricci_scalar(geon_metric_t m, const double* x, size_t n, double* out) { return curvature_call(m, 2, x, n, nullptr, 0, 1, out, 1); }
int geon_einstein(geon_metric_t m, const double* x, size_t n, double* out) { return curvature_call(m, 3, x, n, nullptr, 0, 1, out, 16); }
int geon_stress_energy(geon_metric_t m, const double* x, size_t n, double* out) { return curvature_call(m, 4, x, n, nullptr, 0, 1, out, 16); }

int geon_nec_contraction(geon_metric_t m, const double* x, size_t n, const double* k, size_t nk, int k_shared,
                         double* out) {
  if (nk == 0 || n == 0) return GEON_OK;
  if (!k) return fail(GEON_ERR_INVALID, "null k");
  return curvature_call(m, 5, x, n, k, nk, k_shared, out, (int)nk);
}

int geon_wec_contraction(geon_metric_t m, const double* x, size_t n, const double* u, size_t nu, int u_shared,
                         double* out) {
  return geon_nec_contraction(m, x, n, u, nu, u_shared, out);
}

int geon_equatorial_rays(geon_metric_t m, double r_obs, const double* alpha, size_t n, double* out_states) {
  if (int rc = check_metric(m)) return rc;
  if (m->desc.kind != GEON_SCHWARZSCHILD) return fail(GEON_ERR_INVALID, "equatorial rays need a Schwarzschild metric");
  if (n == 0) return GEON_OK;
  if (!alpha || !out_states) return fail(GEON_ERR_INVALID, "null buffer");
  cudaStream_t s = host_stream();
  DBuf da, dout;
  GEON_CUDA(da.alloc(sizeof(double) * n, s));
  GEON_CUDA(dout.alloc(sizeof(double) * 8 * n, s));
  GEON_CUDA(cudaMemcpyAsync(da.p, alpha, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  counted();
  GEON_CUDA(launch_equatorial_rays(m->desc.p[0], r_obs, da.as<double>(), (int64_t)n, dout.as<double>(), s));
  GEON_CUDA(cudaMemcpyAsync(out_states, dout.p, sizeof(double) * 8 * n, cudaMemcpyDeviceToHost, s));
  GEON_CUDA(cudaStreamSynchronize(s));
  return GEON_OK;
}

// Classify rays launched at the given angles on stream s (device buffers).
// Sweeps of at least SHADOW_ORDER_MIN rays (and fewer than 2^31) are claimed
// longest first (launch_shadow_order); smaller ones in index order.
constexpr int64_t SHADOW_ORDER_MIN = 65536;

static int classify_dev(geon_metric_t m, double r_obs, const double* d_alpha, int64_t n, double step,
                        int64_t max_steps, int precision, int32_t* d_term, int64_t* d_steps,
                        cudaStream_t s) {
  DBuf ws, dorder;
  GEON_CUDA(ws.alloc(sizeof(unsigned long long) * 4, s));
  GEON_CUDA(cudaMemsetAsync(ws.p, 0, sizeof(unsigned long long) * 4, s));
  const int32_t* order = nullptr;
  if (g_sweep_order.load() && n >= SHADOW_ORDER_MIN && n < ((int64_t)1 << 31)) {
    GEON_CUDA(dorder.alloc(sizeof(int32_t) * n, s));
    counted();
    GEON_CUDA(launch_shadow_order(m->desc.p[0], r_obs, d_alpha, n, dorder.as<int32_t>(),
                                  ws.as<unsigned long long>() + 2, s));
    order = dorder.as<int32_t>();
  }
  TraceLaunch L = base_launch(m, step, max_steps);
  L.order = order;
  L.n = n;
  L.alpha = d_alpha;
  L.r_obs = r_obs;
  L.term = d_term;
  L.steps = d_steps;
  L.queue = ws.as<unsigned long long>();
  L.flags = reinterpret_cast<int*>(L.queue + 1);
  GEON_CUDA(launch_trace(L, precision, SRC_EQUATORIAL, SINK_SHADOW, s));
  return GEON_OK;
}

int geon_shadow_classify(geon_metric_t m, double r_obs, const double* alpha, size_t n, double step,
                         int64_t max_steps, int precision, int32_t* term, int64_t* steps) {
  if (int rc = check_metric(m)) return rc;
  if (m->desc.kind != GEON_SCHWARZSCHILD) return fail(GEON_ERR_INVALID, "shadow classification needs a Schwarzschild metric");
  if (!valid_precision(precision)) return fail(GEON_ERR_INVALID, "unknown precision");
  if (n == 0) return GEON_OK;
  if (!alpha || !term) return fail(GEON_ERR_INVALID, "null buffer");
  cudaStream_t s = host_stream();
  DBuf da, dt, dst;
  GEON_CUDA(da.alloc(sizeof(double) * n, s));
  GEON_CUDA(dt.alloc(sizeof(int32_t) * n, s));
  GEON_CUDA(dst.alloc(sizeof(int64_t) * n, s));
  GEON_CUDA(cudaMemcpyAsync(da.p, alpha, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  if (int rc = classify_dev(m, r_obs, da.as<double>(), (int64_t)n, step, max_steps, precision,
                            dt.as<int32_t>(), dst.as<int64_t>(), s))
    return rc;
  GEON_CUDA(cudaMemcpyAsync(term, dt.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  if (int rc = copy_out(steps, dst.p, sizeof(int64_t) * n, s)) return rc;
  GEON_CUDA(cudaStreamSynchronize(s));
  return GEON_OK;
}

int geon_shadow_trace(geon_metric_t m, double r_obs, const double* alpha, size_t n, double step,
                      int64_t max_steps, int precision, int32_t* term, double* final_state, int64_t* steps,
                      double* null_residual) {
  if (int rc = check_metric(m)) return rc;
  if (m->desc.kind != GEON_SCHWARZSCHILD) return fail(GEON_ERR_INVALID, "equatorial rays need a Schwarzschild metric");
  if (!valid_precision(precision)) return fail(GEON_ERR_INVALID, "unknown precision");
  if (n == 0) return GEON_OK;
  if (!alpha || !term) return fail(GEON_ERR_INVALID, "null buffer");
  cudaStream_t s = host_stream();
  DBuf da, dt, dy, dst, dr, ws;
  GEON_CUDA(da.alloc(sizeof(double) * n, s));
  GEON_CUDA(dt.alloc(sizeof(int32_t) * n, s));
  GEON_CUDA(dy.alloc(sizeof(double) * 8 * n, s));
  GEON_CUDA(dst.alloc(sizeof(int64_t) * n, s));
  GEON_CUDA(dr.alloc(sizeof(double) * n, s));
  GEON_CUDA(ws.alloc(sizeof(unsigned long long) * 2, s));
  GEON_CUDA(cudaMemcpyAsync(da.p, alpha, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  GEON_CUDA(cudaMemsetAsync(ws.p, 0, sizeof(unsigned long long) * 2, s));
  TraceLaunch L = base_launch(m, step, max_steps);
  L.n = (int64_t)n;
  L.alpha = da.as<double>();
  L.r_obs = r_obs;
  L.term = dt.as<int32_t>();
  L.yfinal = dy.as<double>();
  L.steps = dst.as<int64_t>();
  L.resid = dr.as<double>();
  L.queue = ws.as<unsigned long long>();
  L.flags = reinterpret_cast<int*>(L.queue + 1);
  GEON_CUDA(launch_trace(L, precision, SRC_EQUATORIAL, SINK_TRACE, s));
  GEON_CUDA(cudaMemcpyAsync(term, dt.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  if (int rc = copy_out(final_state, dy.p, sizeof(double) * 8 * n, s)) return rc;
  if (int rc = copy_out(steps, dst.p, sizeof(int64_t) * n, s)) return rc;
  if (int rc = copy_out(null_residual, dr.p, sizeof(double) * n, s)) return rc;
  GEON_CUDA(cudaStreamSynchronize(s));
  return GEON_OK;
}

// Bisection of bin/validate_shadow.rs:70-79, evaluated L levels at a time: for
// each bracket every midpoint the next L sequential halvings could visit (a
// complete binary tree of 2^L - 1 launch angles, built on the device with the
// same 0.5*(lo+hi) arithmetic) is traced in one launch, then a walk kernel
// replays the sequential path through the tree. The result equals the
// sequential loop bit for bit, with ceil(iters / L) dependent rounds instead of
// iters, and no host round trip between rounds (3 launches per round).

int geon_shadow_bisect_dev(geon_metric_t m, double r_obs, const double* lo, const double* hi, size_t nb,
                           int iters, double step, int64_t max_steps, int precision, double* alpha_c,
                           double* lo_out, double* hi_out, int64_t* steps_out, void* stream) {
  if (int rc = check_metric(m)) return rc;
  if (m->desc.kind != GEON_SCHWARZSCHILD) return fail(GEON_ERR_INVALID, "shadow bisection needs a Schwarzschild metric");
  if (!valid_precision(precision)) return fail(GEON_ERR_INVALID, "unknown precision");
  if (nb == 0) return GEON_OK;
  if (!lo || !hi || !alpha_c || iters < 0 || max_steps < 0) return fail(GEON_ERR_INVALID, "bad bisection arguments");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int Lmax = (int)bisect_levels(nb);
  const int64_t cap = (int64_t)nb * ((1LL << Lmax) - 1);
  DBuf work, tree, tterm, tsteps, ws;
  GEON_CUDA(work.alloc(sizeof(double) * 2 * nb + sizeof(int64_t) * nb, s));
  GEON_CUDA(tree.alloc(sizeof(double) * cap, s));
  GEON_CUDA(tterm.alloc(sizeof(int32_t) * cap, s));
  GEON_CUDA(tsteps.alloc(sizeof(int64_t) * cap, s));
  GEON_CUDA(ws.alloc(sizeof(unsigned long long) * 2, s));
  double* wlo = work.as<double>();
  double* whi = wlo + nb;
  int64_t* wst = reinterpret_cast<int64_t*>(whi + nb);
  GEON_CUDA(cudaMemcpyAsync(wlo, lo, sizeof(double) * nb, cudaMemcpyDefault, s));
  GEON_CUDA(cudaMemcpyAsync(whi, hi, sizeof(double) * nb, cudaMemcpyDefault, s));
  GEON_CUDA(cudaMemsetAsync(wst, 0, sizeof(int64_t) * nb, s));
  int remaining = iters;
  while (remaining > 0) {
    const int L = remaining < Lmax ? remaining : Lmax;
    const int64_t per = (1LL << L) - 1;
    const int64_t nr = (int64_t)nb * per;
    counted();
    GEON_CUDA(launch_bisect_build((int64_t)nb, per, wlo, whi, tree.as<double>(), s));
    GEON_CUDA(cudaMemsetAsync(ws.p, 0, sizeof(unsigned long long) * 2, s));
    TraceLaunch T = base_launch(m, step, max_steps);
    T.n = nr;
    T.alpha = tree.as<double>();
    T.r_obs = r_obs;
    T.term = tterm.as<int32_t>();
    T.steps = tsteps.as<int64_t>();
    T.queue = ws.as<unsigned long long>();
    T.flags = reinterpret_cast<int*>(T.queue + 1);
    T.decide = 1;  // only each ray's class matters to the walk
    GEON_CUDA(launch_trace(T, precision, SRC_EQUATORIAL, SINK_SHADOW, s));
    counted();
    GEON_CUDA(launch_bisect_walk((int64_t)nb, per, L, tree.as<double>(), tterm.as<int32_t>(),
                                 tsteps.as<int64_t>(), wlo, whi, wst, s));
    remaining -= L;
  }
  counted();
  GEON_CUDA(launch_bisect_finish((int64_t)nb, wlo, whi, alpha_c, s));
  if (lo_out) GEON_CUDA(cudaMemcpyAsync(lo_out, wlo, sizeof(double) * nb, cudaMemcpyDefault, s));
  if (hi_out) GEON_CUDA(cudaMemcpyAsync(hi_out, whi, sizeof(double) * nb, cudaMemcpyDefault, s));
  if (steps_out) GEON_CUDA(cudaMemcpyAsync(steps_out, wst, sizeof(int64_t) * nb, cudaMemcpyDefault, s));
  return GEON_OK;
}

int geon_shadow_bisect(geon_metric_t m, double r_obs, const double* lo, const double* hi, size_t nb, int iters,
                       double step, int64_t max_steps, int precision, double* alpha_c, double* lo_out,
                       double* hi_out, int64_t* steps_out) {
  if (int rc = check_metric(m)) return rc;
  if (nb == 0) return GEON_OK;
  if (!lo || !hi || !alpha_c) return fail(GEON_ERR_INVALID, "bad bisection arguments");
  cudaStream_t s = host_stream();
  DBuf io;
  GEON_CUDA(io.alloc(sizeof(double) * 5 * nb + sizeof(int64_t) * nb, s));
  double* d_lo = io.as<double>();
  double* d_hi = d_lo + nb;
  double* d_ac = d_hi + nb;
  double* d_lo_o = d_ac + nb;
  double* d_hi_o = d_lo_o + nb;
  int64_t* d_st = reinterpret_cast<int64_t*>(d_hi_o + nb);
  GEON_CUDA(cudaMemcpyAsync(d_lo, lo, sizeof(double) * nb, cudaMemcpyHostToDevice, s));
  GEON_CUDA(cudaMemcpyAsync(d_hi, hi, sizeof(double) * nb, cudaMemcpyHostToDevice, s));
  if (int rc = geon_shadow_bisect_dev(m, r_obs, d_lo, d_hi, nb, iters, step, max_steps, precision, d_ac, d_lo_o,
                                      d_hi_o, d_st, s))
    return rc;
  GEON_CUDA(cudaMemcpyAsync(alpha_c, d_ac, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
  if (int rc = copy_out(lo_out, d_lo_o, sizeof(double) * nb, s)) return rc;
  if (int rc = copy_out(hi_out, d_hi_o, sizeof(double) * nb, s)) return rc;
  if (int rc = copy_out(steps_out, d_st, sizeof(int64_t) * nb, s)) return rc;
  GEON_CUDA(cudaStreamSynchronize(s));
  return GEON_OK;
}

int geon_shadow_classify_dev(geon_metric_t m, double r_obs, const double* alpha, size_t n, double step,
                             int64_t max_steps, int precision, int32_t* term, int64_t* steps, void* stream) {
  if (int rc = check_metric(m)) return rc;
  if (m->desc.kind != GEON_SCHWARZSCHILD) return fail(GEON_ERR_INVALID, "shadow classification needs a Schwarzschild metric");
  if (!valid_precision(precision)) return fail(GEON_ERR_INVALID, "unknown precision");
  if (n == 0) return GEON_OK;
  if (!alpha || !term) return fail(GEON_ERR_INVALID, "null buffer");
  return classify_dev(m, r_obs, alpha, (int64_t)n, step, max_steps, precision, term, steps,
                      static_cast<cudaStream_t>(stream));
}

unsigned long long geon_launch_count(void) { return g_launches.load(); }


int geon_probe_fma_peak(int fp64, double* tflops) {
  if (!tflops) return fail(GEON_ERR_INVALID, "null output");
  int dev = 0, sms = 0;
  GEON_CUDA(cudaGetDevice(&dev));
  GEON_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256;
  const int iters = fp64 ? 4096 : 65536;
  cudaStream_t s = host_stream();
  DBuf out;
  GEON_CUDA(out.alloc((size_t)blocks * threads * 8, s));
  cudaEvent_t a, b;
  GEON_CUDA(cudaEventCreate(&a));
  GEON_CUDA(cudaEventCreate(&b));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    GEON_CUDA(cudaEventRecord(a, s));
    counted();
    GEON_CUDA(launch_fma_probe(fp64, out.p, blocks, threads, iters, s));
    GEON_CUDA(cudaEventRecord(b, s));
    GEON_CUDA(cudaEventSynchronize(b));
    float ms = 0.0f;
    GEON_CUDA(cudaEventElapsedTime(&ms, a, b));
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return GEON_OK;
}


static int grid_desc(const geon_grid* g, GridDesc& d, int64_t& n) {
  if (!g || g->n[0] < 1 || g->n[1] < 1 || g->n[2] < 1) return fail(GEON_ERR_INVALID, "bad grid");
  std::memcpy(d.lo, g->lo, sizeof d.lo);
  std::memcpy(d.hi, g->hi, sizeof d.hi);
  std::memcpy(d.n, g->n, sizeof d.n);
  d.t = g->t;
  n = g->n[0] * g->n[1] * g->n[2];
  return GEON_OK;
}

int geon_curvature_grid_dev(geon_metric_t m, const geon_grid* grid, size_t nk, uint64_t seed, double* einstein,
                            double* nec, double* k_out, void* stream) {
  if (int rc = check_metric(m)) return rc;
  GridDesc d;
  int64_t n = 0;
  if (int rc = grid_desc(grid, d, n)) return rc;
  if (nk > 0 && !nec) return fail(GEON_ERR_INVALID, "nec output needed when nk > 0");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DBuf dflags;
  GEON_CUDA(dflags.alloc(sizeof(int), s));
  GEON_CUDA(cudaMemsetAsync(dflags.p, 0, sizeof(int), s));
  counted();
  GEON_CUDA(launch_curvature_grid(m->desc, d, (int64_t)nk, seed, einstein, nec, k_out, dflags.as<int>(), s));
  return GEON_OK;
}

int geon_curvature_grid(geon_metric_t m, const geon_grid* grid, size_t nk, uint64_t seed, double* einstein,
                        double* nec, double* k_out) {
  if (int rc = check_metric(m)) return rc;
  GridDesc d;
  int64_t n = 0;
  if (int rc = grid_desc(grid, d, n)) return rc;
  if (nk > 0 && !nec) return fail(GEON_ERR_INVALID, "nec output needed when nk > 0");
  cudaStream_t s = host_stream();
  DBuf de, dn, dk, dflags;
  if (einstein) GEON_CUDA(de.alloc(sizeof(double) * 16 * n, s));
  if (nk) GEON_CUDA(dn.alloc(sizeof(double) * nk * n, s));
  if (k_out && nk) GEON_CUDA(dk.alloc(sizeof(double) * 4 * nk * n, s));
  GEON_CUDA(dflags.alloc(sizeof(int), s));
  GEON_CUDA(cudaMemsetAsync(dflags.p, 0, sizeof(int), s));
  counted();
  GEON_CUDA(launch_curvature_grid(m->desc, d, (int64_t)nk, seed, einstein ? de.as<double>() : nullptr,
                                  nk ? dn.as<double>() : nullptr, (k_out && nk) ? dk.as<double>() : nullptr,
                                  dflags.as<int>(), s));
  if (int rc = copy_out(einstein, de.p, sizeof(double) * 16 * n, s)) return rc;
  if (nk) {
    if (int rc = copy_out(nec, dn.p, sizeof(double) * nk * n, s)) return rc;
    if (int rc = copy_out(k_out, dk.p, sizeof(double) * 4 * nk * n, s)) return rc;
  }
  int flags = 0;
  if (int rc = sync_and_flags(s, dflags.as<int>(), &flags)) return rc;
  return singular_status(flags);
}

}  // extern "C"
