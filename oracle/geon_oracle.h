/*
 * geon oracle: CPU FP64 restatement of the geon reference's ray-tracing and
 * curvature path. TEST INFRASTRUCTURE ONLY: it is the checker for the GPU
 * library, never part of the product path. Only tests/, the smoke check and
 * bench.py's CPU-baseline leg load it.
 *
 * Every function follows the reference's operation order (left-associated
 * sums, no FMA contraction, dense loops) so that with the same transcendental
 * results it reproduces the Rust code bit for bit. Parity anchors: the
 * reference's own printed known answers (docs/energy_conditions.txt:1-49,
 * README.md:43-50), checked by tests/test_oracle_kat.py.
 *
 * Math mode (`math` argument everywhere):
 *   ORC_MATH_LIBM = 0  sin/cos/tanh from the C library (glibc), which is what
 *                      Rust's f64::{sin,cos,tanh} call on linux-gnu. This is the
 *                      reference-faithful mode.
 *   ORC_MATH_GEON = 1  the deterministic sin/cos/tanh defined in this file
 *                      (Cody-Waite reduction + Taylor kernels evaluated with
 *                      explicit fma). The GPU library implements the same
 *                      method; device results must equal this mode bit for bit.
 *   ORC_MATH_NUDGE = 2 libm with each sin/cos/tanh result moved one ulp up: the
 *                      sensitivity of every output to a 1-ulp change in libm.
 *
 * Termination codes follow cuda/schwarzschild_render.cu:93 of the reference:
 *   0 = Diverged, 1 = Captured, 2 = Escaped.
 * Metric kinds: 0 Minkowski, 1 Schwarzschild, 2 Alcubierre, 3 Morris-Thorne.
 * Metric params (double[4]):
 *   Minkowski      unused
 *   Schwarzschild  {mass, horizon_pad, escape_radius}
 *   Alcubierre     {bubble_radius, bubble_thickness, ship_velocity, ship_x}
 *   Morris-Thorne  {throat_radius}
 */
#ifndef GEON_ORACLE_H
#define GEON_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_MATH_LIBM = 0, ORC_MATH_GEON = 1, ORC_MATH_NUDGE = 2 };

typedef struct {
  int64_t captured, escaped, diverged;
  double max_null_residual;
  double avg_steps;
  int64_t total_steps; /* sum over every traced sample (the ray-step count) */
} orc_render_stats;

/* deterministic math, exported so tests can compare it with libm and the GPU */
void orc_geon_sincos(const double* x, int64_t n, double* s, double* c);
void orc_geon_tanh(const double* x, int64_t n, double* out);
void orc_geon_expm1(const double* x, int64_t n, double* out);
/* 4x4 inverse used in place of nalgebra's try_inverse; returns 0 if singular */
int orc_inv4(const double* m16, double* out16);

/* point-wise metric functors over n points (AoS: x is n*4) */
int orc_metric_g(int kind, const double* params, int math, const double* x, int64_t n, double* out16);
int orc_metric_dg(int kind, const double* params, int math, const double* x, int64_t n, double* out64);
int orc_metric_g_inv(int kind, const double* params, int math, const double* x, int64_t n, double* out16);
int orc_metric_christoffel(int kind, const double* params, int math, const double* x, int64_t n, double* out64);
/* term: -1 = None, else a termination code */
int orc_metric_terminate(int kind, const double* params, int math, const double* x, int64_t n, int32_t* term);
int orc_asymptotic_direction(int kind, const double* params, int math, const double* xp8, int64_t n, double* out3);

/* geodesic::trace over n rays (y0: n*8 AoS). nthreads <= 0 means all cores. */
int orc_trace(int kind, const double* params, int math, const double* y0, int64_t n, double step,
              int64_t max_steps, int nthreads, int32_t* term, double* yfinal, int64_t* steps,
              double* resid);

/* Camera::tetrad; returns 0 ok, -3 not timelike, -4 Gram-Schmidt failure */
int orc_camera_tetrad(int kind, const double* params, int math, const double* observer, double* out16);
/* Camera::ray_state_sub for every pixel of rows [row0, row0+nrows) with sub-sample (du, dv).
   fov_y_deg is converted with to_radians. forward_sign=+1 is the reference camera. */
int orc_camera_rays(const double* tetrad16, const double* observer, double fov_y_deg, int64_t width,
                    int64_t height, int64_t row0, int64_t nrows, double du, double dv,
                    int forward_sign, double* y0_out);
/* sky::sample over n directions */
void orc_sky_sample(const double* dir3, int64_t n, int show_stars, float* rgb_out);

/* render::render restricted to rows [row0, row0+nrows) (nrows = height for the whole image).
   rgb_out: nrows*width*3, pclass_out (optional): nrows*width, psteps_out (optional) */
int orc_render(int kind, const double* params, int math, const double* observer, double fov_y_deg,
               int64_t width, int64_t height, int64_t row0, int64_t nrows, double step,
               int64_t max_steps, int64_t samples_per_axis, int show_stars, int forward_sign,
               int nthreads, float* rgb_out, int32_t* pclass_out, int64_t* psteps_out,
               orc_render_stats* stats);

/* Register the sampled metric used for kind 4 (the GPU's GEON_FIELD): grid
   lo/hi/n per spatial axis, chart 0 Cartesian / 1 spherical, samples n0*n1*n2 x
   10 unique components (00 01 02 03 11 12 13 22 23 33), x fastest. */
int orc_field_set(const double* lo3, const double* hi3, const int64_t* n3, int chart, const double* samples);

/* The GPU's GEON_ADAPTIVE trace (Dormand-Prince 5(4), trace_adaptive.cu), restated. */
int orc_trace_adaptive(int kind, const double* params, int math, const double* y0, int64_t n, double h0,
                       int64_t max_steps, double rtol, double atol, int nthreads, int32_t* term, double* yfinal,
                       int64_t* steps, double* resid);

/* write_png's tonemap (render.rs:174-178): clamp, f32 powf(v, 1/2.2) from libm,
   *255, round, saturating cast to u8 (NaN -> 0). */
void orc_tonemap_u8(const float* rgb, int64_t n, uint8_t* out);

/* curvature.rs. what: 0 riemann(256) 1 ricci(16) 2 ricci_scalar(1) 3 einstein(16)
   4 stress_energy(16). faithful=1 evaluates exactly the reference's call graph
   (Riemann recomputed inside ricci_scalar); 0 computes it once (bit-identical). */
int orc_curvature(int kind, const double* params, int math, const double* x, int64_t n, int what,
                  int faithful, int nthreads, double* out);
/* nec_contraction at n points with nk null vectors per point (k: n*nk*4, or nk*4 shared
   when k_shared=1). out: n*nk. */
int orc_nec(int kind, const double* params, int math, const double* x, int64_t n, const double* k,
            int64_t nk, int k_shared, int faithful, int nthreads, double* out);

/* bin/validate_shadow.rs */
void orc_equatorial_ray(double mass, double r_obs, int math, const double* alpha, int64_t n,
                        double* y0_out);
/* is_captured for n launch angles; captured_out[i] = 1/0, steps_out optional */
int orc_shadow_classify(const double* schw_params, double r_obs, int math, const double* alpha,
                        int64_t n, double step, int64_t max_steps, int nthreads,
                        int32_t* term_out, int64_t* steps_out);
/* nb independent bisections on [lo, hi], iters halvings each (bin/validate_shadow.rs:70-79).
   alpha_c_out = 0.5*(lo+hi) after the loop; lo_out/hi_out optional; steps_out optional (sum). */
int orc_shadow_bisect(const double* schw_params, double r_obs, int math, const double* lo,
                      const double* hi, int64_t nb, int iters, double step, int64_t max_steps,
                      int nthreads, double* alpha_c_out, double* lo_out, double* hi_out,
                      int64_t* steps_out);

/* bin/energy_conditions.rs main: fills a flat array of every printed value, in print order:
   [0] mink nec, [1] mink R, [2..7] schw (nec,R) at r=5,10,30,
   [8..48] alcubierre nec at x=-4+0.2n (41), [49] alc min, [50] alc min x, [51] alc integral,
   [52..92] MT nec at l=-4+0.2n (41), [93] MT min, [94] MT min l, [95..98] MT T diag at throat.
   returns the count written (99). */
int orc_energy_conditions(int math, double* out);

int orc_hardware_threads(void);

#ifdef __cplusplus
}
#endif
#endif
