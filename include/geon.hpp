/*
 * geon.hpp: the geon crate's API (metric/mod.rs, camera.rs, geodesic.rs,
 * render.rs, curvature.rs) in C++17 over the C ABI of geon_gpu.h, for hosts
 * written in C++ and for the C++ ports of the reference's executables. Header
 * only; link with -lgeon_gpu.
 *
 * Mapping (Rust -> C++): `trait Metric` -> class geon::Metric (handle to the
 * device functor); Minkowski / Schwarzschild::new(m) / Alcubierre::default() /
 * MorrisThorne::default() -> factory functions of the same names; Vec4, Mat4,
 * State, Christoffel -> std::array of the same shapes; Option<Termination> ->
 * std::optional<Termination>; `panic!` -> geon::Panic (thrown with the
 * reference's message); render() -> std::pair<std::vector<float>, RenderStats>.
 * Every call runs on the GPU; there is no CPU fallback.
 */
#ifndef GEON_HPP
#define GEON_HPP

#include <array>
#include <cmath>
#include <cstdint>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "geon_gpu.h"

namespace geon {

using Scalar = double;
using Vec4 = std::array<double, 4>;
using Mat4 = std::array<std::array<double, 4>, 4>;
using State = std::array<double, 8>;
using Christoffel = std::array<std::array<std::array<double, 4>, 4>, 4>;

// types.rs: Termination (mod.rs:112-120)
enum class Termination { Diverged = GEON_DIVERGED, Captured = GEON_CAPTURED, Escaped = GEON_ESCAPED };

// A reference panic, or a library error (CUDA, out of memory, bad argument).
struct Panic : std::runtime_error {
  int status;
  Panic(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(int rc) {
  if (rc == GEON_OK) return;
  switch (rc) {  // the reference's panic messages (types.rs:39, camera.rs:53, camera.rs:85-88)
    case GEON_ERR_SINGULAR_METRIC: throw Panic(rc, "metric became singular — coordinate chart broke down");
    case GEON_ERR_NOT_TIMELIKE: throw Panic(rc, "observer is not in a timelike region (g_tt >= 0)");
    case GEON_ERR_GRAM_SCHMIDT:
      throw Panic(rc, "Gram–Schmidt produced non-spacelike vector — chart broken at this point");
    default: throw Panic(rc, std::string("geon_gpu: ") + geon_last_error());
  }
}

// trait Metric (metric/mod.rs:19-109): an immutable device functor.
class Metric {
 public:
  Metric(int kind, std::vector<double> params) : kind_(kind), params_(std::move(params)) {
    check(geon_metric_create(kind, params_.empty() ? nullptr : params_.data(), (int)params_.size(), &h_));
  }
  Metric(const Metric& o) : Metric(o.kind_, o.params_) {}
  Metric& operator=(const Metric&) = delete;
  ~Metric() { geon_metric_destroy(h_); }

  geon_metric_t handle() const { return h_; }
  int kind() const { return kind_; }
  std::string name() const { return geon_metric_name(h_); }  // Metric::name (mod.rs:84)
  Vec4 fd_step() const { return {1e-5, 1e-5, 1e-5, 1e-5}; }  // Metric::fd_step (mod.rs:73-75)

  Mat4 g(const Vec4& x) const { return one<Mat4>(geon_metric_g, x); }                  // mod.rs:21
  std::array<Mat4, 4> dg(const Vec4& x) const { return one<std::array<Mat4, 4>>(geon_metric_dg, x); }  // mod.rs:25-43
  Mat4 g_inv(const Vec4& x) const { return one<Mat4>(geon_metric_g_inv, x); }          // mod.rs:46-48
  Christoffel christoffel(const Vec4& x) const { return one<Christoffel>(geon_metric_christoffel, x); }  // mod.rs:51-69
  // Metric::terminate (mod.rs:78)
  std::optional<Termination> terminate(const Vec4& x) const {
    int32_t t = -1;
    check(geon_metric_terminate(h_, x.data(), 1, &t));
    if (t < 0) return std::nullopt;
    return static_cast<Termination>(t);
  }
  // Metric::asymptotic_direction (mod.rs:91-108)
  std::array<double, 3> asymptotic_direction(const Vec4& x, const Vec4& p) const {
    const State s{x[0], x[1], x[2], x[3], p[0], p[1], p[2], p[3]};
    std::array<double, 3> d{};
    check(geon_metric_asymptotic_direction(h_, s.data(), 1, d.data()));
    return d;
  }
  // Batched forms: one device launch for all points.
  std::vector<Christoffel> christoffel(const std::vector<Vec4>& xs) const {
    std::vector<Christoffel> out(xs.size());
    check(geon_metric_christoffel(h_, xs.front().data(), xs.size(), out.front()[0][0].data()));
    return out;
  }

 private:
  template <class Out, class Fn>
  Out one(Fn fn, const Vec4& x) const {
    Out o{};
    check(fn(h_, x.data(), 1, reinterpret_cast<double*>(&o)));
    return o;
  }
  int kind_;
  std::vector<double> params_;
  geon_metric_t h_ = nullptr;
};

// The four implementations with the reference's constructors and defaults.
inline Metric Minkowski() { return Metric(GEON_MINKOWSKI, {}); }
// Schwarzschild::new(mass): horizon_pad 1.001, escape_radius 1000 (schwarzschild.rs:20-28)
inline Metric Schwarzschild(double mass, double horizon_pad = 1.001, double escape_radius = 1000.0) {
  return Metric(GEON_SCHWARZSCHILD, {mass, horizon_pad, escape_radius});
}
// Alcubierre { bubble_radius, bubble_thickness, ship_velocity, ship_x }; default 2, 0.5, 2, 0 (alcubierre.rs:21-30)
inline Metric Alcubierre(double bubble_radius = 2.0, double bubble_thickness = 0.5, double ship_velocity = 2.0,
                         double ship_x = 0.0) {
  return Metric(GEON_ALCUBIERRE, {bubble_radius, bubble_thickness, ship_velocity, ship_x});
}
// MorrisThorne { throat_radius }; default 1 (morris_thorne.rs:15-18)
inline Metric MorrisThorne(double throat_radius = 1.0) { return Metric(GEON_MORRIS_THORNE, {throat_radius}); }

// geodesic.rs:18-25
struct TraceResult {
  Termination termination;
  State final_state;
  size_t steps_taken;
  double null_residual;
};

// geodesic::trace (geodesic.rs:62-117); precision GEON_FP64 reproduces the reference.
inline std::vector<TraceResult> trace_many(const Metric& m, const std::vector<State>& y0, Scalar step,
                                           size_t max_steps, int precision = GEON_FP64) {
  const size_t n = y0.size();
  std::vector<int32_t> t(n);
  std::vector<State> yf(n);
  std::vector<int64_t> st(n);
  std::vector<double> r(n);
  if (n) check(geon_trace(m.handle(), y0.front().data(), n, step, (int64_t)max_steps, precision, t.data(),
                          yf.front().data(), st.data(), r.data()));
  std::vector<TraceResult> out(n);
  for (size_t i = 0; i < n; ++i) out[i] = {static_cast<Termination>(t[i]), yf[i], (size_t)st[i], r[i]};
  return out;
}
inline TraceResult trace(const Metric& m, const State& y0, Scalar step, size_t max_steps,
                         int precision = GEON_FP64) {
  return trace_many(m, {y0}, step, max_steps, precision)[0];
}

// camera.rs:21-160
struct Camera {
  Vec4 observer;
  Scalar fov_y_rad;
  size_t width, height;
  int forward_sign = 1;  // +1 the reference camera; -1 looks along +e1 (an extension)

  static Camera new_(const Vec4& observer, Scalar fov_y_deg, size_t width, size_t height) {
    return Camera{observer, fov_y_deg * (3.141592653589793 / 180.0), width, height, 1};
  }
  geon_camera c() const {
    geon_camera g{};
    for (int i = 0; i < 4; ++i) g.observer[i] = observer[i];
    g.fov_y_deg = fov_y_rad * (180.0 / 3.141592653589793);
    g.width = (int64_t)width;
    g.height = (int64_t)height;
    g.forward_sign = forward_sign;
    return g;
  }
  // Camera::tetrad (camera.rs:47-97): rows e_(a)^mu
  Mat4 tetrad(const Metric& m) const {
    Mat4 t{};
    check(geon_camera_tetrad(m.handle(), observer.data(), t[0].data()));
    return t;
  }
  // Camera::ray_state_sub for every pixel (row-major)
  std::vector<State> ray_states(const Mat4& tet, Scalar du = 0.5, Scalar dv = 0.5) const {
    const geon_camera g = c();
    std::vector<State> s(width * height);
    check(geon_camera_ray_states(&g, tet[0].data(), du, dv, s.front().data()));
    return s;
  }
  State ray_state_sub(const Mat4& tet, size_t i, size_t j, Scalar du, Scalar dv) const {
    return ray_states(tet, du, dv)[j * width + i];
  }
  State ray_state(const Mat4& tet, size_t i, size_t j) const { return ray_state_sub(tet, i, j, 0.5, 0.5); }
};

// render.rs:17-53
struct RenderConfig {
  Scalar step = 0.05;
  size_t max_steps = 20000;
  std::array<float, 3> captured_rgb{0.0f, 0.0f, 0.0f};
  std::array<float, 3> diverged_rgb{1.0f, 0.0f, 1.0f};
  size_t samples_per_axis = 1;
  int show_stars = -1;  // -1: the process-wide flag (sky.rs:23, set_show_stars)
  int precision = GEON_FP64;

  static RenderConfig default_() { return RenderConfig{}; }
  geon_render_config c() const {
    geon_render_config g{};
    g.step = step;
    g.max_steps = (int64_t)max_steps;
    for (int i = 0; i < 3; ++i) {
      g.captured_rgb[i] = captured_rgb[i];
      g.diverged_rgb[i] = diverged_rgb[i];
    }
    g.samples_per_axis = (int64_t)samples_per_axis;
    g.show_stars = show_stars;
    g.precision = precision;
    return g;
  }
};

struct RenderStats {
  size_t captured = 0, escaped = 0, diverged = 0;
  Scalar max_null_residual = 0.0, avg_steps = 0.0;
  uint64_t total_steps = 0;  // an addition: the ray-steps of the image
};

inline RenderStats stats_of(const geon_render_stats& s) {
  return RenderStats{(size_t)s.captured, (size_t)s.escaped, (size_t)s.diverged, s.max_null_residual, s.avg_steps,
                     (uint64_t)s.total_steps};
}

// sky::SHOW_STARS (sky.rs:23)
inline void set_show_stars(bool on) { geon_set_show_stars(on ? 1 : 0); }

// render::render (render.rs:55-166): pixels W*H*3 row-major (the Vec<f32>)
inline std::pair<std::vector<float>, RenderStats> render(const Metric& m, const Camera& cam, const RenderConfig& cfg) {
  const geon_camera c = cam.c();
  const geon_render_config r = cfg.c();
  std::vector<float> px(cam.width * cam.height * 3);
  geon_render_stats s{};
  check(geon_render(m.handle(), &c, &r, px.data(), &s));
  return {std::move(px), stats_of(s)};
}

// render() + write_png's tonemap (render.rs:169-183) on the device: the bytes
// write_png hands to the PNG encoder.
inline std::pair<std::vector<uint8_t>, RenderStats> render_u8(const Metric& m, const Camera& cam,
                                                              const RenderConfig& cfg) {
  const geon_camera c = cam.c();
  const geon_render_config r = cfg.c();
  std::vector<uint8_t> px(cam.width * cam.height * 3);
  geon_render_stats s{};
  check(geon_render_u8(m.handle(), &c, &r, px.data(), nullptr, &s));
  return {std::move(px), stats_of(s)};
}

// curvature.rs:48-141 (each a batched launch when given many points)
namespace curvature {
inline std::array<Mat4, 16> riemann(const Metric& m, const Vec4& x) {  // [rho][sigma][mu][nu] as 16 Mat4
  std::array<Mat4, 16> out{};
  check(geon_riemann(m.handle(), x.data(), 1, out[0][0].data()));
  return out;
}
inline Mat4 ricci(const Metric& m, const Vec4& x) {
  Mat4 o{};
  check(geon_ricci(m.handle(), x.data(), 1, o[0].data()));
  return o;
}
inline Scalar ricci_scalar(const Metric& m, const Vec4& x) {
  double r = 0.0;
  check(geon_ricci_scalar(m.handle(), x.data(), 1, &r));
  return r;
}
inline Mat4 einstein(const Metric& m, const Vec4& x) {
  Mat4 o{};
  check(geon_einstein(m.handle(), x.data(), 1, o[0].data()));
  return o;
}
inline Mat4 stress_energy(const Metric& m, const Vec4& x) {
  Mat4 o{};
  check(geon_stress_energy(m.handle(), x.data(), 1, o[0].data()));
  return o;
}
inline Scalar nec_contraction(const Metric& m, const Vec4& x, const Vec4& k) {
  double v = 0.0;
  check(geon_nec_contraction(m.handle(), x.data(), 1, k.data(), 1, 1, &v));
  return v;
}
inline std::vector<double> nec_contraction(const Metric& m, const std::vector<Vec4>& xs, const Vec4& k) {
  std::vector<double> v(xs.size());
  if (!xs.empty()) check(geon_nec_contraction(m.handle(), xs.front().data(), xs.size(), k.data(), 1, 1, v.data()));
  return v;
}
inline Scalar wec_contraction(const Metric& m, const Vec4& x, const Vec4& u) { return nec_contraction(m, x, u); }
}  // namespace curvature

// bin/validate_shadow.rs:20-35: the equatorial ray at launch angle alpha
inline State equatorial_ray(const Metric& schwarzschild, Scalar r_obs, Scalar alpha) {
  State s{};
  check(geon_equatorial_rays(schwarzschild.handle(), r_obs, &alpha, 1, s.data()));
  return s;
}

// The 60-halving bisection of bin/validate_shadow.rs:70-79, bit for bit, as
// one batched device job (lo, hi updated in place; returns alpha_c).
inline Scalar shadow_bisect(const Metric& schwarzschild, Scalar r_obs, Scalar& lo, Scalar& hi, int iters,
                            Scalar step = 0.01, size_t max_steps = 200000, int precision = GEON_FP64) {
  double ac = 0.0, lo_o = 0.0, hi_o = 0.0;
  int64_t st = 0;
  check(geon_shadow_bisect(schwarzschild.handle(), r_obs, &lo, &hi, 1, iters, step, (int64_t)max_steps, precision,
                           &ac, &lo_o, &hi_o, &st));
  lo = lo_o;
  hi = hi_o;
  return ac;
}

}  // namespace geon

#endif  // GEON_HPP
