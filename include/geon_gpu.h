/*
 * geon_gpu.h: C ABI of the GB300 geodesic ray-tracing and curvature library.
 *
 * A drop-in for the hot path of the geon crate (Rust): the Metric trait's
 * functors with their finite-difference fallbacks, geodesic::trace, the Camera
 * tetrad, render(), the shadow bisection of bin/validate_shadow.rs and the
 * curvature.rs chain. A Rust host binds these with `extern "C"` declarations;
 * every array layout below is the memory layout
 * of the corresponding Rust type, so slices pass through without copies:
 *   Vec4 = [f64; 4], Mat4 = [[f64; 4]; 4] (row-major), Christoffel =
 *   [[[f64; 4]; 4]; 4] indexed [mu][alpha][beta], State = [f64; 8] =
 *   (x^0..x^3, p^0..p^3), Riemann = [[[[f64; 4]; 4]; 4]; 4] indexed
 *   [rho][sigma][mu][nu].
 *
 * Conventions
 *  - Every function returns GEON_OK (0) or a negative GEON_ERR_* status; where
 *    the reference panics (singular metric, non-timelike observer, failed
 *    Gram-Schmidt) the call returns the matching status and the host shim
 *    raises the reference's panic message. geon_last_error() gives a message.
 *  - Plain entry points take HOST pointers, copy in, run, copy out and return
 *    when the results are in the caller's buffers. `_dev` variants take DEVICE
 *    pointers and a cudaStream_t (as void*) and are stream-ordered.
 *  - Handles are immutable after creation; calls are thread-safe.
 *  - Termination codes: GEON_DIVERGED 0, GEON_CAPTURED 1, GEON_ESCAPED 2 (the
 *    encoding of the reference's cuda/schwarzschild_render.cu:93); -1 = None.
 *  - precision: GEON_FP64 reproduces the reference's FP64 arithmetic (the same
 *    bits as the reference for the same sin/cos/tanh values); GEON_MIXED runs
 *    the FP32 bulk integrator with FP64 kept where stability needs it.
 */
#ifndef GEON_GPU_H
#define GEON_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GEON_ABI_VERSION 1

/* status codes */
#define GEON_OK 0
#define GEON_ERR_INVALID (-1)          /* bad argument */
#define GEON_ERR_SINGULAR_METRIC (-2)  /* types.rs:39 panic: g not invertible */
#define GEON_ERR_NOT_TIMELIKE (-3)     /* camera.rs:53 panic: g_tt >= 0 at the observer */
#define GEON_ERR_GRAM_SCHMIDT (-4)     /* camera.rs:85-88 panic: n^2 <= 0 */
#define GEON_ERR_CUDA (-5)             /* CUDA runtime error */
#define GEON_ERR_OOM (-6)              /* device allocation failed */
#define GEON_ERR_ADMISSION (-7)        /* job larger than the server's memory budget */
#define GEON_ERR_TIMEOUT (-8)          /* wait deadline passed */
#define GEON_ERR_NOT_FOUND (-9)        /* unknown job id */
#define GEON_ERR_CANCELLED (-10)       /* job cancelled */
#define GEON_ERR_UNSUPPORTED (-11)     /* combination not provided */

enum geon_metric_kind {
  GEON_MINKOWSKI = 0,     /* metric/minkowski.rs */
  GEON_SCHWARZSCHILD = 1, /* metric/schwarzschild.rs */
  GEON_ALCUBIERRE = 2,    /* metric/alcubierre.rs */
  GEON_MORRIS_THORNE = 3, /* metric/morris_thorne.rs */
  GEON_FIELD = 4          /* a sampled metric (geon_metric_create_field); an extension */
};
/* chart of a sampled metric: how asymptotic_direction reads (x1, x2, x3) */
enum geon_chart { GEON_CHART_CARTESIAN = 0, GEON_CHART_SPHERICAL = 1 };
enum geon_termination { GEON_DIVERGED = 0, GEON_CAPTURED = 1, GEON_ESCAPED = 2 };
/* GEON_ADAPTIVE (an extension; the reference lists it as a TODO at
 * integrator.rs:5-7): FP64 Dormand-Prince 5(4) with error control instead of
 * the fixed-step RK4; `step` is the first trial step, max_steps caps accepted
 * steps, tolerances from geon_set_adaptive_tolerance. Not for the server. */
/* GEON_FP64_FAST (an extension): FP64 fixed-step RK4 in the same chart, with the
 * same stage points, termination tests, NaN guard and step cap as GEON_FP64,
 * held to the reference CUDA kernel's tolerance (cuda/schwarzschild_render.cu:3-5,
 * equal "up to associativity") instead of to the reference's bits: fused
 * multiply-adds, one reciprocal per right-hand side, sin/cos of the polar angle
 * once per step. Schwarzschild only; other metrics run the GEON_FP64 stepper.
 * Not for the server. */
enum geon_precision { GEON_FP64 = 0, GEON_MIXED = 1, GEON_ADAPTIVE = 2, GEON_FP64_FAST = 3 };

typedef struct geon_metric* geon_metric_t;

/* Camera (camera.rs:21-36). forward_sign = +1 is the reference camera (image
 * forward = -e1, right = +e3, up = -e2); -1 looks along +e1 with right = -e3,
 * an extension for poses the reference camera cannot express. */
typedef struct {
  double observer[4];
  double fov_y_deg;
  int64_t width;
  int64_t height;
  int32_t forward_sign;
  int32_t reserved;
} geon_camera;

/* RenderConfig (render.rs:17-43) plus the sky flag and precision. */
typedef struct {
  double step;              /* default 0.05 */
  int64_t max_steps;        /* default 20000 */
  float captured_rgb[3];    /* default (0, 0, 0) */
  float diverged_rgb[3];    /* default (1, 0, 1) */
  int64_t samples_per_axis; /* default 1 */
  int32_t show_stars;       /* 1/0, or -1 to use the process-wide flag (sky.rs:23) */
  int32_t precision;        /* GEON_FP64 or GEON_MIXED */
} geon_render_config;

/* RenderStats (render.rs:45-53) plus the total ray-step count. */
typedef struct {
  int64_t captured;
  int64_t escaped;
  int64_t diverged;
  double max_null_residual;
  double avg_steps;
  int64_t total_steps; /* sum of steps_taken over every traced sample */
} geon_render_stats;

/* A regular grid over the three spatial chart coordinates: n[a] points from
 * lo[a] to hi[a] inclusive (x fastest), at time t. */
typedef struct {
  double lo[3];
  double hi[3];
  int64_t n[3];
  double t;
} geon_grid;

const char* geon_version(void);
/* Message of the last failed call on this thread. */
const char* geon_last_error(void);
/* Fill cfg with RenderConfig::default() (render.rs:32-43). */
void geon_render_config_default(geon_render_config* cfg);

/* --- Metric handles (trait Metric, metric/mod.rs:19; the four `impl Metric` blocks) --
 * params, by kind (the reference struct's fields in declaration order):
 *   MINKOWSKI      none
 *   SCHWARZSCHILD  {mass, horizon_pad, escape_radius}  (Schwarzschild::new(m): pad 1.001, escape 1000)
 *   ALCUBIERRE     {bubble_radius, bubble_thickness, ship_velocity, ship_x}
 *   MORRIS_THORNE  {throat_radius}
 * Missing trailing params take the reference's defaults. */
int geon_metric_create(int kind, const double* params, int nparams, geon_metric_t* out);
/* A sampled (tensor-field) metric: the phase-4 idea of g from a sampled or
 * neural field (phase4/ARCHITECTURE.md:33-58) feeding the same finite-difference
 * Christoffel and curvature chain as the reference's fallback metrics.
 * samples: grid->n[0]*n[1]*n[2] nodes x 10 doubles, the unique components
 * (g00 g01 g02 g03 g11 g12 g13 g22 g23 g33) of a static g at the nodes
 * (x1, x2, x3) = lo + (i, j, k) * (hi - lo) / (n - 1) (grid->t ignored), node
 * (i, j, k) at index i + n0 * (j + n1 * k). The samples are the control points of
 * a uniform cubic B-spline, so g is C2 (its curvature is meaningful) and
 * reproduces affine fields exactly (smoother fields to O(spacing^2)); an axis
 * with one node is constant. Trace termination: leaving the grid box escapes
 * (on a spherical chart, falling below the inner radius is a capture); a
 * non-finite position diverges. The samples are copied to the device; FP64 and
 * adaptive paths (the mixed path answers GEON_ERR_UNSUPPORTED). */
int geon_metric_create_field(const geon_grid* grid, const double* samples, int chart, geon_metric_t* out);
int geon_metric_destroy(geon_metric_t m);
int geon_metric_kind(geon_metric_t m);
/* Metric::name (metric/mod.rs:84) */
const char* geon_metric_name(geon_metric_t m);

/* Point-wise functors over n points. x: n Vec4. */
int geon_metric_g(geon_metric_t m, const double* x, size_t n, double* out_mat4);          /* Metric::g, mod.rs:21 (n*16) */
int geon_metric_dg(geon_metric_t m, const double* x, size_t n, double* out_dg);           /* Metric::dg, mod.rs:25-43, [alpha][mu][nu] (n*64) */
int geon_metric_g_inv(geon_metric_t m, const double* x, size_t n, double* out_mat4);      /* Metric::g_inv, mod.rs:46-48 (n*16) */
int geon_metric_christoffel(geon_metric_t m, const double* x, size_t n, double* out_chr); /* Metric::christoffel, mod.rs:51-69 (n*64) */
int geon_metric_terminate(geon_metric_t m, const double* x, size_t n, int32_t* out_term); /* Metric::terminate, mod.rs:78, -1 = None */
/* Metric::asymptotic_direction (mod.rs:91-108) over n States: n*3 out. */
int geon_metric_asymptotic_direction(geon_metric_t m, const double* states, size_t n, double* out_dir);

/* --- geodesic::trace (geodesic.rs:62-117) over n rays ----------------------
 * y0: n States. Outputs (each may be NULL except term): termination, final
 * State, steps_taken, null_residual. precision: GEON_FP64 or GEON_MIXED. */
int geon_trace(geon_metric_t m, const double* y0, size_t n, double step, int64_t max_steps,
               int precision, int32_t* term, double* final_state, int64_t* steps_taken,
               double* null_residual);
int geon_trace_dev(geon_metric_t m, const double* y0, size_t n, double step, int64_t max_steps,
                   int precision, int32_t* term, double* final_state, int64_t* steps_taken,
                   double* null_residual, void* stream);

/* --- Camera (camera.rs:47-160) --------------------------------------------- */
/* Camera::tetrad (camera.rs:47-97): rows e_(a)^mu, out 16 doubles. */
int geon_camera_tetrad(geon_metric_t m, const double observer[4], double out_tetrad[16]);
/* Camera::ray_state_sub (camera.rs:113-160) for every pixel at sub-pixel (du, dv):
 * out width*height States, row-major (pixel (i, j) at j*width + i). */
int geon_camera_ray_states(const geon_camera* cam, const double tetrad[16], double du, double dv,
                           double* out_states);

/* --- render() (render.rs:55-166) ------------------------------------------- */
/* rgb: width*height*3 floats, row-major, top-left origin (the Vec<f32>). */
int geon_render(geon_metric_t m, const geon_camera* cam, const geon_render_config* cfg, float* rgb,
                geon_render_stats* stats);
/* As geon_render, also returning per-pixel classification (render.rs:129-135)
 * and per-pixel mean steps; either may be NULL. */
int geon_render_ex(geon_metric_t m, const geon_camera* cam, const geon_render_config* cfg,
                   float* rgb, geon_render_stats* stats, int32_t* pixel_class,
                   int64_t* pixel_steps);
/* render() followed by write_png's tonemap (render.rs:169-183) on the device:
 * rgb8 receives width*height*3 bytes, the buffer write_png hands to the PNG
 * encoder (clamp to [0, 1], ^(1/2.2) in f32, *255, round, saturating cast).
 * rgb (the f32 image) may be NULL. */
int geon_render_u8(geon_metric_t m, const geon_camera* cam, const geon_render_config* cfg,
                   uint8_t* rgb8, float* rgb, geon_render_stats* stats);
/* Several renders traced together by ONE persistent kernel launch: the rays of
 * every item share one device work queue, and a lane that finishes a ray takes
 * the next one of any item (any metric kind), so images of uneven path length
 * keep the GPU full until the last ray. Each item's outputs equal what
 * geon_render_ex gives for it alone, bit for bit. 1 to 8 items, one precision
 * for all (GEON_FP64 or GEON_MIXED); sampled metrics are not supported. An
 * extension: the reference renders one image per call (render.rs:55-166). */
typedef struct {
  geon_metric_t metric;
  geon_camera camera;
  geon_render_config render;
  float* rgb;                 /* out: width*height*3 */
  geon_render_stats* stats;   /* out, may be NULL */
  int32_t* pixel_class;       /* out, may be NULL */
  int64_t* pixel_steps;       /* out, may be NULL */
} geon_render_item;
int geon_render_batch(const geon_render_item* items, size_t n);
/* write_png's tonemap (render.rs:174-178) alone, over n floats. */
int geon_tonemap_u8(const float* rgb, size_t n, uint8_t* out);
int geon_tonemap_u8_dev(const float* rgb, size_t n, uint8_t* out, void* stream);
/* sky::sample (sky.rs:107-120) over n unit directions (n*3 in, n*3 out). */
int geon_sky_sample(const double* dir, size_t n, int show_stars, float* rgb);
/* sky::SHOW_STARS (sky.rs:23; set by bin/render.rs:71-73). */
void geon_set_show_stars(int on);
int geon_get_show_stars(void);

/* --- mixed-precision options (no counterpart in the reference, which is FP64 only) ---
 * FP64 band half-width for GEON_MIXED, per metric kind, in the metric's own
 * scale: Schwarzschild r < band*M, Morris-Thorne |l| < band*b0, Alcubierre
 * |r_s - R| < band*s; 0 (the default) disables the band: with the compensated
 * FP32 state the band is not needed for accuracy and costs warp divergence.
 * geon_set_mixed_reproject(1) re-imposes g(p, p) = 0 on p^t after every FP32 step. */
int geon_set_mixed_band(int kind, double band);
double geon_get_mixed_band(int kind);
void geon_set_mixed_reproject(int on);
/* Default on: GEON_MIXED traces of the spherically symmetric metrics
 * (Schwarzschild, Morris-Thorne), camera rays and ray arrays, step each ray in
 * the frame of its own orbit plane, on the equator with no trigonometry in the
 * step, and turn its final state back into the chart; every geodesic of these
 * metrics lies in a plane through the centre, so the frame is exact geometry
 * and keeps the rays away from the chart's polar axis, where the reference's
 * (theta, phi) step flings rays off their geodesic. The final state is the same
 * point of the geodesic with theta in [0, pi] and phi in (-pi, pi] (the frame
 * does not count turns of phi). Served camera rays use it too. Off (0): the
 * rays step in the chart (the FP64 band and null re-projection options step
 * in the chart whatever this says). No counterpart in the reference. */
void geon_set_mixed_orbit_plane(int on);
int geon_get_mixed_orbit_plane(void);
/* Compensated null re-projection for GEON_MIXED null rays on their plane
 * (shadow rays; Schwarzschild and Morris-Thorne rays in their orbit-plane
 * frame): after every 16 steps of a ray, g(p, p) is formed in float-float
 * from the compensated state and one Newton step on g(p, p) = 0 in p^t is
 * added to p^t with its rounding error kept (null drift ~1e-13, the FP64
 * path's, at ~3 % of the step's cost). Camera and equatorial rays are null by
 * construction; a ray of a geon_trace array is null if g(p, p) at its initial
 * state cancels to 1e-8 of its largest term (FP64), and a timelike or
 * spacelike ray keeps the invariant its integration gives it, as in the
 * reference. Default on (1); served requests always use it. No counterpart
 * in the reference. */
void geon_set_mixed_null_fix(int on);
int geon_get_mixed_null_fix(void);
/* Error tolerances of GEON_ADAPTIVE: a step is accepted when
 * sqrt(mean_i((e_i / (atol + rtol * max(|y_i|, |y_new_i|)))^2)) <= 1.
 * Defaults rtol 1e-10, atol 1e-12. Calls made after this use them. */
int geon_set_adaptive_tolerance(double rtol, double atol);
/* Width of the speculative bisection (geon_shadow_bisect*): each round traces
 * every midpoint the next L halvings can visit, with the largest L that keeps
 * nb * (2^L - 1) <= rays launch angles (default 16384). A wider round takes
 * fewer dependent rounds and more rays; results do not change. The no-alloc
 * variant keeps the default. */
int geon_set_bisect_rays_per_round(int64_t rays);
int64_t geon_get_bisect_rays_per_round(void);
void geon_get_adaptive_tolerance(double* rtol, double* atol);
/* Trace kernels are persistent (one grid fills every SM and pulls rays from a
 * device work queue). To let another job run beside one (e.g. bisections next
 * to a sweep), calls made after this keep `blocks_per_sm` resident slots per SM
 * free. Default 0. */
void geon_set_persistent_reserve(int blocks_per_sm);
/* The same with a fractional count: the grid keeps floor(SMs x (occupancy -
 * blocks_per_sm)) blocks, so e.g. 4.5 leaves 4 slots on half of the SMs and 5
 * on the others. No counterpart in the reference (no persistent kernels). */
void geon_set_persistent_reserve_f(double blocks_per_sm);
/* Launch variant of the mixed kernel per metric kind and ray source (source 0:
 * camera rays and ray arrays, 1: equatorial shadow rays). Register cap c: 0 =
 * none, 1 = at most 64 registers per thread, 2 = at most 51. Source 0 takes
 * variant = c (blocks of 128 threads); source 1 takes variant = c + 3 b with
 * block size b: 0 = 128, 1 = 64, 2 = 256 threads. geon_autotune_mixed times
 * every variant on calibration jobs of this metric (n_rays rays - 0 picks four
 * per lane of the widest grid - at most max_steps each; the equatorial job only
 * for Schwarzschild), selects the fastest per source and writes ray-steps/s to
 * rates_out[12] (3 for source 0, then 9 for source 1) and the choices to
 * best_out[2] (-1 = source not tuned); either may be NULL. The persistent
 * reserve (geon_set_persistent_reserve) counts slots of 128 threads whatever
 * the block size. */
int geon_set_mixed_variant(int kind, int source, int variant);
int geon_get_mixed_variant(int kind, int source);
int geon_autotune_mixed(geon_metric_t m, int64_t n_rays, int64_t max_steps, double* rates_out,
                        int* best_out);

/* --- curvature.rs ------------------------------------------------------------ */
int geon_riemann(geon_metric_t m, const double* x, size_t n, double* out);       /* curvature.rs:48, n*256 */
int geon_ricci(geon_metric_t m, const double* x, size_t n, double* out);         /* curvature.rs:72, n*16 */
int geon_ricci_scalar(geon_metric_t m, const double* x, size_t n, double* out);  /* curvature.rs:87, n */
int geon_einstein(geon_metric_t m, const double* x, size_t n, double* out);      /* curvature.rs:99, n*16 */
int geon_stress_energy(geon_metric_t m, const double* x, size_t n, double* out); /* curvature.rs:112, n*16 */
/* nec_contraction (curvature.rs:127-136) at n points for nk vectors each: k is nk Vec4 shared by all
 * points when k_shared != 0, else n*nk Vec4 (point-major). out: n*nk. */
int geon_nec_contraction(geon_metric_t m, const double* x, size_t n, const double* k, size_t nk,
                         int k_shared, double* out);
/* Curvature over a regular grid (a batch form of curvature.rs with no
 * counterpart in the reference, which evaluates point by point in
 * bin/energy_conditions.rs:86-117). Point index p = (iz*ny + iy)*nx + ix at
 * x = (t, lo[0] + ix*(hi[0]-lo[0])/(nx-1), ...), endpoints included. For each
 * point: einstein (16 doubles, may be NULL) and nk values of T(k, k) for null
 * vectors k = e0 + n1 e1 + n2 e2 + n3 e3 in the point's static-observer
 * Gram-Schmidt tetrad, n uniform on the sphere drawn from the counter-based
 * stream splitmix64(seed ^ (p*nk + q)); k_out (n*nk*4, may be NULL) returns
 * the vectors used. */
int geon_curvature_grid(geon_metric_t m, const geon_grid* grid, size_t nk, uint64_t seed, double* einstein,
                        double* nec, double* k_out);
int geon_curvature_grid_dev(geon_metric_t m, const geon_grid* grid, size_t nk, uint64_t seed,
                            double* einstein, double* nec, double* k_out, void* stream);
/* wec_contraction is nec_contraction with a timelike vector (curvature.rs:139-141). */
int geon_wec_contraction(geon_metric_t m, const double* x, size_t n, const double* u, size_t nu,
                         int u_shared, double* out);

/* --- bin/energy_conditions.rs (energy_conditions.rs:37-156) as one batched job --
 * The 99 numbers the bin prints, in its order: Minkowski T(k,k), R; for
 * Schwarzschild r = 5, 10, 30: T(k,k), R; Alcubierre (R 2, thickness 0.5, v 2):
 * T(k,k) at the 41 scan points x = -4 + 0.2 n, the minimum, its x, the
 * negative-part integral over x = -5 .. 5 (dx 0.05, the bin's accumulated
 * positions); Morris-Thorne (b0 1): T(k,k) at the 41 points l = -4 + 0.2 n,
 * the minimum, its l, then T^mu_nu[i][i] at the throat for i = 0..3. */
#define GEON_ENERGY_CONDITIONS_N 99
int geon_energy_conditions(double* out);

/* --- shadow validation (bin/validate_shadow.rs:20-94) ------------------------ */
/* equatorial_ray (validate_shadow.rs:20-35): n launch angles -> n States. */
int geon_equatorial_rays(geon_metric_t schwarzschild, double r_obs, const double* alpha, size_t n,
                         double* out_states);
/* is_captured (validate_shadow.rs:37-41) for n launch angles: term (n), steps (n, may be NULL). */
int geon_shadow_classify(geon_metric_t schwarzschild, double r_obs, const double* alpha, size_t n,
                         double step, int64_t max_steps, int precision, int32_t* term,
                         int64_t* steps);
/* geodesic::trace (geodesic.rs:62-117) of the equatorial rays of n launch angles
 * (validate_shadow.rs:20-35), with the stepper geon_shadow_classify uses for
 * them (the mixed path steps them on their invariant plane). Outputs as
 * geon_trace; final_state, steps and null_residual may be NULL. An extension:
 * the reference traces these rays only inside is_captured. */
int geon_shadow_trace(geon_metric_t schwarzschild, double r_obs, const double* alpha, size_t n,
                      double step, int64_t max_steps, int precision, int32_t* term,
                      double* final_state, int64_t* steps, double* null_residual);
/* nb independent bisections of `iters` halvings each on [lo[i], hi[i]]
 * (bin/validate_shadow.rs:70-79). Outputs alpha_c = 0.5*(lo+hi) after the loop;
 * lo_out/hi_out/steps_out (ray-steps spent) may be NULL. With GEON_FP64 the
 * result equals the sequential bisection bit for bit. */
int geon_shadow_bisect(geon_metric_t schwarzschild, double r_obs, const double* lo, const double* hi,
                       size_t nb, int iters, double step, int64_t max_steps, int precision,
                       double* alpha_c, double* lo_out, double* hi_out, int64_t* steps_out);

/* Claim order of geon_shadow_classify(_dev) over 65536 rays or more: 1 (the
 * default) claims the rays whose impact parameter is at least 0.998 of the
 * critical one (escaping or orbiting near the photon sphere: the long paths)
 * first, so the short ones fill the end of the sweep when lanes run out of
 * work; 0 claims them in index order. Results do not change. */
void geon_set_sweep_order(int on);
int geon_get_sweep_order(void);
/* Device-pointer, stream-ordered forms of the two calls above (alpha, lo, hi and
 * every output are device addresses; the call returns once the work is queued).
 * The bisection keeps its rounds on the device: no host round trip per round. */
int geon_shadow_classify_dev(geon_metric_t schwarzschild, double r_obs, const double* alpha, size_t n,
                             double step, int64_t max_steps, int precision, int32_t* term,
                             int64_t* steps, void* stream);
int geon_shadow_bisect_dev(geon_metric_t schwarzschild, double r_obs, const double* lo, const double* hi,
                           size_t nb, int iters, double step, int64_t max_steps, int precision,
                           double* alpha_c, double* lo_out, double* hi_out, int64_t* steps_out,
                           void* stream);

/* geon_shadow_bisect_dev without any device allocation. No counterpart in the
 * reference: it exists for callers that may not let a library allocate GPU
 * memory while they run (a host that owns all device memory through its own
 * pool, a real-time loop with no room for an allocator call, code that must not
 * fail with "out of memory" mid-way). Its working memory is one fixed 512 KiB
 * array compiled into the library; at most 4096 brackets per call (larger:
 * GEON_ERR_INVALID). Every call looks up the array's device address on the
 * current device. With CUDA's lazy module loading, the array and the kernels'
 * code are placed on a device at their first use there, so the first call on
 * each device takes that memory (once; it is held until exit): make the first
 * call before the caller reserves the rest of the device memory, and before any
 * stream capture. Calls share the array: calls that overlap on the GPU race
 * with each other, so order them on one stream. The speculative width is the
 * default one (geon_set_bisect_rays_per_round does not apply). Same arguments
 * and results as geon_shadow_bisect_dev. */
int geon_shadow_bisect_dev_noalloc(geon_metric_t schwarzschild, double r_obs, const double* lo,
                                   const double* hi, size_t nb, int iters, double step,
                                   int64_t max_steps, int precision, double* alpha_c,
                                   double* lo_out, double* hi_out, int64_t* steps_out, void* stream);

/* --- serving engine (no counterpart in the reference) ---------------------------
 * The reference renders one image per process (bin/render.rs:69-143), bisects in
 * one loop (bin/validate_shadow.rs:70-77) and evaluates curvature point by point
 * (curvature.rs:16-141). A server runs all three kinds of request for many
 * callers at once on one GPU: requests are admitted while their buffers fit in a
 * device memory budget fixed at creation, rays of every admitted request share
 * persistent kernels that refill finished lanes from a device work queue, and
 * a request that arrives while others run joins at the next kernel launch.
 * Each result is the one the matching single-call entry point gives
 * (geon_render_ex, geon_shadow_bisect with one bracket, geon_curvature_grid),
 * bit for bit, whatever else runs beside it. Mixed-precision requests run the
 * default mixed step (camera rays of Schwarzschild and Morris-Thorne in their
 * orbit plane); geon_set_mixed_band, geon_set_mixed_reproject and
 * geon_set_mixed_orbit_plane(0) are not applied to served requests. */
typedef struct geon_server* geon_server_t;
enum geon_job_type { GEON_JOB_RENDER = 0, GEON_JOB_BISECT = 1, GEON_JOB_CURVATURE = 2 };

typedef struct {
  int32_t type;             /* geon_job_type */
  int32_t metric_kind;      /* geon_metric_kind */
  double metric_params[4];  /* as geon_metric_create */
  int32_t nparams;
  int32_t precision;        /* GEON_FP64 or GEON_MIXED (ray requests) */
  double deadline_s;        /* > 0: give up after this many seconds (GEON_ERR_TIMEOUT) */
  /* GEON_JOB_RENDER: geon_render_ex's arguments (render.precision is ignored) */
  geon_camera camera;
  geon_render_config render;
  float* rgb;                     /* out: width*height*3 (may be NULL when rgb8 is set) */
  geon_render_stats* render_stats;/* out, may be NULL */
  int32_t* pixel_class;           /* out, may be NULL */
  int64_t* pixel_steps;           /* out, may be NULL */
  uint8_t* rgb8;                  /* out, may be NULL: the tonemapped bytes (geon_render_u8) */
  /* GEON_JOB_BISECT: one bracket of geon_shadow_bisect (Schwarzschild only) */
  double r_obs, lo, hi, step;
  int64_t max_steps;
  int32_t iters;            /* halvings */
  int32_t rays_per_round;   /* 2^L - 1 speculative midpoints per round (L = 1..12; default 31) */
  double* alpha_c;          /* out */
  double* lo_out;           /* out, may be NULL */
  double* hi_out;           /* out, may be NULL */
  int64_t* steps_out;       /* out, may be NULL: steps of the rays on the bisection path */
  /* GEON_JOB_CURVATURE: geon_curvature_grid's arguments */
  geon_grid grid;
  int64_t nk;
  uint64_t seed;
  double* einstein;         /* out, may be NULL */
  double* nec;              /* out, may be NULL */
} geon_job;

typedef struct {
  int64_t submitted, completed, failed, queued, running;
  int64_t completed_by_type[3];
  double p50_ms, p99_ms, mean_ms;           /* submission to completion, every type */
  double p50_ms_by_type[3], p99_ms_by_type[3];
  double ray_steps;                         /* ray-steps integrated for completed requests */
  double grid_points;                       /* curvature points of completed requests */
  double wall_s;                            /* first submission to last completion */
  int64_t epochs;                           /* persistent-kernel launches */
  double ray_steps_unfinished;              /* ray-steps of the rays that finished in requests
                                               that were cancelled or timed out */
} geon_server_stats;

/* budget_bytes: device memory for request buffers (a request larger than it is
 * refused with GEON_ERR_ADMISSION at submission). */
int geon_server_create(size_t budget_bytes, geon_server_t* out);
/* Queue a request; output pointers must stay valid until it completes. */
int geon_server_submit(geon_server_t s, const geon_job* job, uint64_t* id);
/* 0 queued, 1 running, 2 done; a negative status if it failed. */
int geon_server_poll(geon_server_t s, uint64_t id);
/* Block until the request is done (timeout_s < 0: no limit); returns its status. */
int geon_server_wait(geon_server_t s, uint64_t id, double timeout_s);
int geon_server_wait_all(geon_server_t s, double timeout_s);
/* A queued request is dropped; a running one stops at the next launch
 * boundary. Its status becomes GEON_ERR_CANCELLED. */
int geon_server_cancel(geon_server_t s, uint64_t id);
int geon_server_stats_get(geon_server_t s, geon_server_stats* out);
/* Steps per launch of the persistent serving kernels of one precision
 * (GEON_FP64 or GEON_MIXED): each launch runs at most this many RK4 steps per
 * lane before the host admits arrivals and finishes jobs (rounded up to a
 * multiple of 16: a lane takes 16 steps between refills). Defaults 128 (FP64)
 * and 4096 (mixed). Larger: fewer host round trips; smaller: finer admission
 * and completion granularity. */
int geon_server_set_steps_per_launch(geon_server_t s, int precision, int steps);
int geon_server_get_steps_per_launch(geon_server_t s, int precision);
/* The steps-per-launch autotuner: on an idle server, times a calibration render
 * (Schwarzschild, r_obs 30, fov 60, h 0.05, cap 20000, escape 1000M; 320^2 FP64,
 * 512^2 mixed) through the server at 32..512 (FP64) and 1024..16384 (mixed)
 * steps per launch, keeps for each precision the smallest value within 2 % of
 * the fastest, and returns ray-steps/s in rates_out[2][5] (FP64 row first) and
 * the choices in best_out[2]. */
int geon_server_autotune(geon_server_t s, double* rates_out, int* best_out);
/* Stops the server after the work in flight; queued requests are cancelled. */
int geon_server_destroy(geon_server_t s);

/* --- measurement helpers (no counterpart in the reference) --------------------- */
/* Kernels this library has launched since it was loaded. */
unsigned long long geon_launch_count(void);
/* Sustained FMA throughput of this GPU (independent chains on every SM), in
 * TFLOP/s: fp64 != 0 measures DFMA, else FFMA. The roofline denominator. */
int geon_probe_fma_peak(int fp64, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* GEON_GPU_H */
