// Mixed-precision ray tracing: the RK4 right-hand sides run in FP32, the ray
// state is carried as FP32 (high, low) pairs with a compensated (two-sum)
// update, and FP64 is used only inside a band around the photon sphere /
// horizon / throat / bubble wall, where a ray's fate is decided.
//
// Why pairs for the whole state: a plain FP32 position at r = 1000 has an ulp
// of 6e-5, coarser than a 0.01 step's increment allows, and a plain FP32
// momentum random-walks to ~1e-6 relative over the 2000 steps before the
// photon sphere, which would move the critical impact parameter past 1e-6. With
// (hi, lo) pairs (48-bit significand) the state keeps FP64-class accuracy and
// only the FP32 evaluation error of each increment (~1e-7 of h*k) remains.
//
// The persistent loop and the sources/sinks are shared with the FP64 path
// (trace_common.cuh); this unit is compiled with --fmad=false too, so every
// fused multiply-add in the FP32 code is written out explicitly.
#include <cuda_runtime.h>

#include <type_traits>

#include "internal.h"
#include "metric_analytic.cuh"
#include "orbit_frame.cuh"
#include "serve_common.cuh"
#include "trace_common.cuh"

namespace geon {

// (hi, lo) += inc, compensated: the low word is folded into the increment and
// the rounding error of hi + (inc + lo) becomes the new low word (TwoSum,
// Knuth; or Fast2Sum, Dekker, when |hi| >= |inc + lo| is known). hi stays the
// FP32 number nearest to hi + lo (|lo| <= ulp(hi)/2), so the stages, which
// are evaluated at the high words, see the state to FP32 precision, and no
// separate renormalisation is needed; the value lost per step is the rounding
// of inc + lo, 2^-24 of the increment, below the FP32 evaluation error of the
// increment itself.
__device__ __forceinline__ void two_sum_update(float& hi, float& lo, float inc) {
  const float t = inc + lo;
  const float s = hi + t;
  const float bb = s - hi;
  lo = (hi - (s - bb)) + (t - bb);
  hi = s;
}

__device__ __forceinline__ void fast_two_sum_update(float& hi, float& lo, float inc) {
  const float t = inc + lo;
  const float s = hi + t;
  lo = (hi - s) + t;
  hi = s;
}

// Float-float (hi, lo) products and sums for the compensated null
// re-projection: the exact rounding error of a product from one fused
// multiply-add, of a sum from TwoSum; the results are not renormalised (their
// low words stay far below the high words' ulp for the few operations chained).
struct FF {
  float h, l;
};
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = a.h * b.h;
  const float e = __fmaf_rn(a.h, b.h, -p);
  return {p, __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.h + b.h;
  const float bb = s - a.h;
  const float e = (a.h - (s - bb)) + (b.h - bb);
  return {s, e + (a.l + b.l)};
}
// 1 / (hi + lo): the correctly rounded reciprocal of hi and one Newton
// correction carried in the low word.
__device__ __forceinline__ FF ff_rcp(FF a) {
  const float q = __frcp_rn(a.h);
  const float e = __fmaf_rn(-q, a.h, 1.0f) - q * a.l;  // 1 - q (hi + lo), its leading part exact
  return {q, q * e};
}

// (hi + lo) > t for a threshold held as a (hi, lo) pair.
__device__ __forceinline__ bool ff_gt(float hi, float lo, float thi, float tlo) {
  return (hi - thi) + (lo - tlo) > 0.0f;
}

// Optional parts of the mixed step, compiled in only when a caller enables
// them: the FP64 band and the per-step null re-projection. The default kernels
// leave both out, which keeps their register demand (and code) small.
// FEAT_PLANAR: every ray is an equatorial Schwarzschild ray (theta = pi/2,
// p^theta = 0, bin/validate_shadow.rs:20-35); FEAT_PLANAR_DYN: a per-ray flag
// says so (the serving kernel, whose lanes take rays of any job). FEAT_ORBIT
// (the default, MIXED_ORBIT): rays of a spherically symmetric metric
// (Schwarzschild, Morris-Thorne) are turned into the frame of their own orbit
// plane at load, stepped there on the equator, and turned back at the end;
// FEAT_ORBIT_DYN: a per-ray flag says so (the serving kernel: camera rays).
// FEAT_DECIDE: every ray is a bisection ray whose class settles early
// (decided_k); FEAT_DECIDE_DYN: a per-ray flag says so (the serving kernel).
enum : int { FEAT_BAND = 1, FEAT_REPROJECT = 2, FEAT_PLANAR = 4, FEAT_PLANAR_DYN = 8, FEAT_ORBIT = 16,
             FEAT_ORBIT_DYN = 32, FEAT_DECIDE = 64, FEAT_DECIDE_DYN = 128 };

// Right-hand side on the equatorial plane: rhs_stage at sin theta = 1,
// cos theta = 0, p^theta = 0, where its theta terms vanish (Gamma^th_phph =
// -sin cos, Gamma^ph_thph p^th, p^th p^th) and what remains is evaluated with
// the same operations. The plane is invariant under the geodesic equation, so
// a ray that starts in it stays in it. Schwarzschild (r) and Morris-Thorne (l).
template <int K>
__device__ __forceinline__ void rhs_planar(const AConsts<float>& C, float r, float p0, float p1, float p3,
                                           float* k4, float* k5, float* k7) {
  using Mt = AMath<float>;
  const float u = -2.0f * p1;  // shared by the Gamma^t_tr and Gamma^ph_rph terms
  if (K == KIND_MORRIS_THORNE) {
    const float q = Mt::div(r, Mt::fma(r, r, C.b0sq));  // Gamma^ph_lph = l / (b0^2 + l^2)
    *k4 = 0.0f;
    *k5 = r * (p3 * p3);
    *k7 = (u * q) * p3;
    return;
  }
  // One reciprocal, of D = r (r - 2M): Gamma^t_tr = M / (r^2 f) = M / D,
  // 1/r = (r - 2M) / D, f = (r - 2M) / r, and Gamma^r_tt = M f / r^2 =
  // Gamma^t_tr f^2, so the p^t^2 and p^r^2 terms share the factor Gamma^t_tr.
  const float rm = r - C.two_m;
  const float iD = Mt::rcp(r * rm);
  const float gtr = C.m * iD;
  const float ir = rm * iD;
  const float E = (rm * ir) * p0;  // f p^t
  *k4 = (u * gtr) * p0;
  *k5 = Mt::fma(gtr, Mt::fma(-E, E, p1 * p1), rm * (p3 * p3));
  *k7 = (u * ir) * p3;
}

template <int FEAT>
struct MixedCore {
  float hi[8], lo[8];
  AConsts<float> C;
  float cap_hi, cap_lo, esc_hi, esc_lo;
  float cap_far, esc_far;  // cap_hi (1 + 2^-10), esc_hi (1 - 2^-10)
  float r_near;             // 3M (1.5 * 2M): inside it the horizon rules can apply
  float h, hh, sixth;
  unsigned nsteps = 0;  // steps this ray has taken (counted where the early decision needs it)
  bool ready = false;
  bool planar = (FEAT & FEAT_PLANAR) != 0;
  bool orbit = (FEAT & FEAT_ORBIT) != 0;
  bool decide = (FEAT & FEAT_DECIDE) != 0;
  bool nullray = true;  // the loaded state is null: the null re-projections apply
  float cap_steps;  // the step cap (max_steps), for the early decision's budget test
  float oe1[3], oe2[3];  // orbit-plane frame (FEAT_ORBIT, FEAT_ORBIT_DYN)
  // rays of metric kind K can step in their orbit-plane frame
  template <int K>
  static constexpr bool any_orbit() {
    return (K == KIND_SCHWARZSCHILD || K == KIND_MORRIS_THORNE) && (FEAT & (FEAT_ORBIT | FEAT_ORBIT_DYN)) != 0;
  }

  // Serving: the source of the ray about to be loaded or resumed (equatorial
  // rays step on their plane, camera rays in their orbit plane).
  __device__ __forceinline__ void set_source(int src) {
    if (FEAT & FEAT_PLANAR_DYN) planar = src == SRC_EQUATORIAL;
    if (FEAT & FEAT_ORBIT_DYN) orbit = src == SRC_CAMERA;
    if (FEAT & FEAT_DECIDE_DYN) decide = src == SRC_EQUATORIAL;  // served bisection rays
  }
  // Serving: a resumed camera ray gets its orbit-plane frame back from its
  // initial state (the frame is a function of it, so it is the one the ray
  // was loaded with).
  template <int K>
  __device__ __forceinline__ void resume_frame_k(const TraceLaunch& L, int64_t ray) {
    if constexpr (any_orbit<K>()) {
      if (orbit) {
        double y0[8], yr[8];
        camera_ray(L.cam, ray, y0);
        orbit_in(y0, yr, oe1, oe2);
      }
    }
  }

  __device__ __forceinline__ void setup(const TraceLaunch& L) {
    C.init(L.M);
    cap_hi = __double2float_rn(L.M.capture_r);
    cap_lo = __double2float_rn(L.M.capture_r - (double)cap_hi);
    esc_hi = __double2float_rn(L.M.escape_r);
    esc_lo = __double2float_rn(L.M.escape_r - (double)esc_hi);
    cap_far = cap_hi * (1.0f + 0x1p-10f);
    r_near = 1.5f * C.two_m;
    esc_far = esc_hi * (1.0f - 0x1p-10f);
    h = (float)L.step;
    hh = (float)L.half_step;
    sixth = (float)L.sixth;
    cap_steps = (float)L.max_steps;
    ready = true;
  }

  __device__ __forceinline__ void load_state(const double y[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      hi[i] = __double2float_rn(y[i]);
      lo[i] = __double2float_rn(y[i] - (double)hi[i]);
    }
  }

  template <int K>
  __device__ __forceinline__ void load_k(const TraceLaunch& L, const double y0[8]) {
    if (!ready) setup(L);
    nsteps = 0;
    if constexpr (any_orbit<K>()) {
      if (orbit) {
        double yr[8];
        orbit_in(y0, yr, oe1, oe2);
        load_state(yr);
        return;
      }
    }
    load_state(y0);
  }

  template <int K>
  __device__ __forceinline__ void to_double_k(double out[8]) const {
    double y[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = (double)hi[i] + (double)lo[i];
    if constexpr (any_orbit<K>()) {
      if (orbit) {
        orbit_out(y, oe1, oe2, out);
        return;
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = y[i];
  }

  // Early decision for bisection rays (validate_shadow.rs:37-41 needs only
  // whether a ray is captured). In Schwarzschild a null geodesic has at most one
  // turning point, outside the photon sphere r = 3M: a ray moving outward
  // beyond it (here r > 3.3M, p^r > 0) has passed its turning point and reaches
  // the escape radius, and p^r only grows on the way, so it gets there within
  // (r_esc - r) / p^r of affine parameter; if that fits in the steps left
  // before the cap (2 % margin) the ray is reported Escaped now. A ray moving
  // inward inside the photon sphere (r < 2.9M, p^r < 0) has no turning point
  // left and is reported Captured now. The class is the one the full trace
  // would end with; steps_taken counts the steps actually taken.
  template <int K>
  __device__ __forceinline__ int decided_k() const {
    if (K == KIND_SCHWARZSCHILD) {
      if (hi[5] > 0.0f) {
        if (hi[1] > 3.3f * C.m && (esc_hi - hi[1]) * 1.02f < (cap_steps - (float)nsteps - 2.0f) * h * hi[5])
          return TERM_ESCAPED;
      } else if (hi[1] < 2.9f * C.m) {
        return TERM_CAPTURED;
      }
    }
    return TERM_NONE;
  }

  // The step count of the ray, kept only where the early decision reads it.
  __device__ __forceinline__ void count_step() {
    if constexpr ((FEAT & (FEAT_DECIDE | FEAT_DECIDE_DYN)) != 0) ++nsteps;
  }

  // A ray of an input array is null if g(p, p) at its initial state (FP64,
  // the metric functor of the FP64 path) cancels to 1e-8 of its largest
  // term; camera and equatorial rays are null by construction. The null
  // re-projections hold g(p, p) at 0, so they apply to null rays only: a
  // timelike or spacelike geodesic keeps the invariant the integration gives
  // it, as in the reference.
  template <int K>
  __device__ __forceinline__ void check_null_k(const TraceLaunch& L, const double y0[8]) {
    double g[16];
    metric_g<K>(L.M, y0, g);
    double sum = 0.0, mag = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const double t = g[4 * i + j] * y0[4 + i] * y0[4 + j];
        sum += t;
        mag += fabs(t);
      }
    }
    nullray = fabs(sum) <= 1e-8 * mag;  // false for a non-finite state
  }

  // After every group of 16 steps a ray survives (rays start at a warp refill
  // and refills come every 16 steps, so this is the same step of every lane of
  // the warp, and every 16th step of each ray): the compensated null
  // re-projection of a null ray stepping on its plane.
  template <int K>
  __device__ __forceinline__ void group_end_k(const TraceLaunch& L) {
    if (!(L.mixed_flags & MIXED_NULLFIX) || !nullray) return;
    const bool on_plane = (any_orbit<K>() && orbit) ||
                          (K == KIND_SCHWARZSCHILD && (FEAT & (FEAT_PLANAR | FEAT_PLANAR_DYN)) != 0 &&
                           ((FEAT & FEAT_PLANAR) != 0 || planar));
    if (on_plane) null_fix_planar<K>();
  }

  // Termination tests of the reference, evaluated on the compensated state.
  template <int K>
  __device__ __forceinline__ int terminate_k(const TraceLaunch&) const {
    if (K == KIND_SCHWARZSCHILD) {
      // Far from both radii the high word decides: |lo| <= ulp(hi)/2 = 2^-24
      // of hi, far inside the 2^-10 margins. (A non-finite r fails this test.)
      if (hi[1] > cap_far && hi[1] < esc_far) {
        if constexpr ((FEAT & (FEAT_DECIDE | FEAT_DECIDE_DYN)) != 0) {
          if (decide) return decided_k<K>();
        }
        return TERM_NONE;
      }
      if (!isfinite(hi[1])) return TERM_DIVERGED;
      if (ff_gt(cap_hi, cap_lo, hi[1], lo[1])) return TERM_CAPTURED;
      if (ff_gt(hi[1], lo[1], esc_hi, esc_lo)) return TERM_ESCAPED;
      return TERM_NONE;
    } else if (K == KIND_MORRIS_THORNE) {
      if (!isfinite(hi[1])) return TERM_DIVERGED;
      const float a = fabsf(hi[1]);
      const float al = hi[1] < 0.0f ? -lo[1] : lo[1];
      return ff_gt(a, al, 1000.0f, 0.0f) ? TERM_ESCAPED : TERM_NONE;
    } else {
      const float r2 = __fmaf_rn(hi[1], hi[1], __fmaf_rn(hi[2], hi[2], hi[3] * hi[3]));
      if (K == KIND_ALCUBIERRE && !isfinite(r2)) return TERM_DIVERGED;
      return r2 > 1e6f ? TERM_ESCAPED : TERM_NONE;
    }
  }

  // Null re-projection of p^t for a ray on its plane (Schwarzschild: equatorial
  // rays and rays in their orbit-plane frame; Morris-Thorne in its frame): the
  // residual R = g(p, p) is formed in float-float from the compensated state
  // (its terms are O(1) and cancel to ~1e-8, below FP32's own precision), and
  // one Newton step on g(p, p) = 0 in p^t, delta = R / (2 (-g_tt) p^t), is
  // added to (hi, lo) of p^t by TwoSum. Schwarzschild, theta = pi/2:
  //   f R = -(f p^t)^2 + (p^r)^2 + f (r p^phi)^2,  f = 1 - 2M/r;
  // Morris-Thorne: R = -(p^t)^2 + (p^l)^2 + (b0^2 + l^2) (p^phi)^2.
  template <int K>
  __device__ __forceinline__ void null_fix_planar() {
    const FF r = {hi[1], lo[1]}, pt = {hi[4], lo[4]}, pr = {hi[5], lo[5]}, pp = {hi[7], lo[7]};
    if (K == KIND_SCHWARZSCHILD) {
      const FF ir = ff_rcp(r);
      const FF u = ff_mul({C.two_m, 0.0f}, ir);  // 2M / r
      const FF f = ff_add({1.0f, 0.0f}, {-u.h, -u.l});
      const FF E = ff_mul(f, pt);
      const FF w = ff_mul(r, pp);
      const FF fw2 = ff_mul(f, ff_mul(w, w));
      const FF E2 = ff_mul(E, E);
      const FF fR = ff_add(ff_add(ff_mul(pr, pr), fw2), {-E2.h, -E2.l});
      const float d = (fR.h + fR.l) / (2.0f * f.h * E.h);
      if (isfinite(d)) two_sum_update(hi[4], lo[4], d);
    } else if (K == KIND_MORRIS_THORNE) {
      const FF r2 = ff_add({C.b0sq, 0.0f}, ff_mul(r, r));
      const FF pt2 = ff_mul(pt, pt);
      const FF R = ff_add(ff_add(ff_mul(pr, pr), ff_mul(r2, ff_mul(pp, pp))), {-pt2.h, -pt2.l});
      const float d = (R.h + R.l) / (2.0f * pt.h);
      if (isfinite(d)) two_sum_update(hi[4], lo[4], d);
    }
  }

  // A Schwarzschild ray moving inward inside the photon sphere (r < 3M, p^r < 0)
  // has no turning point left: it falls through the horizon. Near the horizon
  // p^t = E/f grows without bound and the fixed step stops resolving it; a step
  // whose p^t increment is a quarter of p^t or more (or not finite) is such a
  // step, and its result would fling the ray off its geodesic (the reference
  // then reports it Escaped at r ~ 1e30 or Diverged). The ray is reported
  // Captured there instead. Elsewhere |increment / p^t| = 2 M h |p^r| / (r^2 f)
  // stays far below a quarter at any sensible step.
  __device__ __forceinline__ bool unresolved_infall(float inc_pt) const {
    return hi[5] < 0.0f && hi[1] < r_near && !(fabsf(inc_pt) < 0.25f * hi[4]);
  }

  // Returns STEP_OK, STEP_NONFINITE (state unchanged) or STEP_HORIZON: an RK4
  // stage of a Schwarzschild ray reached r <= 2M, where f = 1 - 2M/r changes
  // sign and the fixed step has no meaning; the ray has crossed the horizon and
  // is reported Captured. (The FP64 path keeps the reference's behaviour: such a
  // step overflows or throws the ray to r ~ 1e30, reported Diverged or Escaped.)
  template <int K>
  __device__ __forceinline__ int step_fp32_k(const TraceLaunch& L) {
    float s0 = 0.0f, c0 = 1.0f;
    if (K == KIND_SCHWARZSCHILD || K == KIND_MORRIS_THORNE) sincosf(hi[2], &s0, &c0);
    float k[8], acc[8], p[4];
    // stage 1 at the state (high words; the polar angle with its low word)
#pragma unroll
    for (int i = 0; i < 4; ++i) p[i] = hi[4 + i];
    rhs_stage<K, float>(C, hi[1], hi[2], hi[3], hi[2], lo[2], p, s0, c0, k);
#pragma unroll
    for (int i = 0; i < 8; ++i) acc[i] = k[i];
    // stages 2-4 at y + c h k
    float rmin = 0.0f;  // lowest stage radius (Schwarzschild horizon rule)
#pragma unroll
    for (int st = 0; st < 3; ++st) {
      const float c = st < 2 ? hh : h;
#pragma unroll
      for (int i = 0; i < 4; ++i) p[i] = __fmaf_rn(c, k[4 + i], hi[4 + i]);
      const float x1 = __fmaf_rn(c, k[1], hi[1]);
      const float x2 = __fmaf_rn(c, k[2], hi[2]);
      const float x3 = __fmaf_rn(c, k[3], hi[3]);
      const float dth = __fmaf_rn(c, k[2], lo[2]);
      rmin = st == 0 ? x1 : fminf(rmin, x1);
      rhs_stage<K, float>(C, x1, x2, x3, hi[2], dth, p, s0, c0, k);
      if (st < 2) {
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i] = __fmaf_rn(2.0f, k[i], acc[i]);
      }
    }
    if (K == KIND_SCHWARZSCHILD && !(rmin > C.two_m)) return STEP_HORIZON;
    bool finite = true;
    float inc[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      inc[i] = sixth * (acc[i] + k[i]);
      finite &= isfinite(inc[i]);
    }
    if (K == KIND_SCHWARZSCHILD && unresolved_infall(inc[4])) return STEP_HORIZON;
    if (!finite) return STEP_NONFINITE;
    // Positions move monotonically in t and phi and stay far from 0 in r and
    // theta relative to one step, so Fast2Sum is exact for them (and for t = 0 or
    // phi = 0 exactly); momenta cross zero (p^r at periapsis), so TwoSum.
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (K == KIND_ALCUBIERRE || K == KIND_MINKOWSKI) two_sum_update(hi[i], lo[i], inc[i]);
      else fast_two_sum_update(hi[i], lo[i], inc[i]);
    }
#pragma unroll
    for (int i = 4; i < 8; ++i) two_sum_update(hi[i], lo[i], inc[i]);
    count_step();
    if ((FEAT & FEAT_REPROJECT) && (L.mixed_flags & MIXED_REPROJECT) && nullray) {
      float s = 0.0f;
      if (K == KIND_SCHWARZSCHILD || K == KIND_MORRIS_THORNE) s = sinf(hi[2]);
      const float x[4] = {hi[0], hi[1], hi[2], hi[3]};
      const float p[4] = {hi[4], hi[5], hi[6], hi[7]};
      const float pt = null_pt<K, float>(C, x, p, s, hi[4]);
      if (isfinite(pt)) {
        two_sum_update(hi[4], lo[4], (pt - hi[4]) - lo[4]);
      }
    }
    return STEP_OK;
  }

  // step_fp32 for a ray on the equator (Schwarzschild: equatorial rays, or any
  // ray in its orbit-plane frame; Morris-Thorne in its orbit-plane frame): the
  // six components that move (t, r or l, phi and their momenta), theta and
  // p^theta held at their loaded values (pi/2 and 0). Same stage points,
  // horizon rule and compensated update as step_fp32.
  template <int K>
  __device__ __forceinline__ int step_fp32_planar_k(const TraceLaunch& L) {
    float k1, k4, k5, k7;
    float p0 = hi[4], p1 = hi[5], p3 = hi[7];
    rhs_planar<K>(C, hi[1], p0, p1, p3, &k4, &k5, &k7);
    k1 = p1;
    float a0 = p0, a1 = p1, a3 = p3, a4 = k4, a5 = k5, a7 = k7;
    float k0 = p0, k3 = p3;
    float rmin = 0.0f;
#pragma unroll
    for (int st = 0; st < 3; ++st) {
      const float c = st < 2 ? hh : h;
      p0 = __fmaf_rn(c, k4, hi[4]);
      p1 = __fmaf_rn(c, k5, hi[5]);
      p3 = __fmaf_rn(c, k7, hi[7]);
      const float r = __fmaf_rn(c, k1, hi[1]);
      rmin = st == 0 ? r : fminf(rmin, r);
      rhs_planar<K>(C, r, p0, p1, p3, &k4, &k5, &k7);
      k0 = p0; k1 = p1; k3 = p3;
      if (st < 2) {
        a0 = __fmaf_rn(2.0f, k0, a0);
        a1 = __fmaf_rn(2.0f, k1, a1);
        a3 = __fmaf_rn(2.0f, k3, a3);
        a4 = __fmaf_rn(2.0f, k4, a4);
        a5 = __fmaf_rn(2.0f, k5, a5);
        a7 = __fmaf_rn(2.0f, k7, a7);
      }
    }
    const float i0 = sixth * (a0 + k0), i1 = sixth * (a1 + k1), i3 = sixth * (a3 + k3);
    const float i4 = sixth * (a4 + k4), i5 = sixth * (a5 + k5), i7 = sixth * (a7 + k7);
    // The horizon rules (a stage at or inside 2M; an unresolved infall, which
    // needs r < 3M) apply only when a stage or the ray is within 3M (or a
    // stage radius is not a number), and the NaN guard on the momenta only
    // when an increment is not finite: one branch per step covers all three,
    // tested in their order inside it. (Every stage value of p^t, p^r, p^phi
    // enters k4, k5, k7 and so the momentum increments, so a non-finite t, r
    // or phi increment, a sum of those stage values, implies a non-finite
    // momentum increment; positions that nothing reads, t and phi for the
    // shadow sink, are then left out by the compiler.)
    const bool finite = isfinite(i4) && isfinite(i5) && isfinite(i7);
    const bool near = K == KIND_SCHWARZSCHILD && (!(rmin > r_near) || hi[1] < r_near);
    if (near || !finite) {
      if (K == KIND_SCHWARZSCHILD && !(rmin > C.two_m)) return STEP_HORIZON;
      if (K == KIND_SCHWARZSCHILD && near && unresolved_infall(i4)) return STEP_HORIZON;
      if (!finite) return STEP_NONFINITE;
    }
    fast_two_sum_update(hi[0], lo[0], i0);
    fast_two_sum_update(hi[1], lo[1], i1);
    fast_two_sum_update(hi[3], lo[3], i3);
    // p^t = E/f and p^phi = L/r^2 keep their sign and change by a small
    // fraction per step (|inc/p^phi| = 2h|p^r|/r; |inc/p^t| = 2h m |p^r|/(r^2 f),
    // below 0.1 down to r = 2.1M and below 1 down to ~2.01M, one or two steps
    // before the capture radius), so Fast2Sum is exact for them wherever the
    // ray's class is still open; p^r crosses zero at periapsis and keeps TwoSum.
    fast_two_sum_update(hi[4], lo[4], i4);
    two_sum_update(hi[5], lo[5], i5);
    fast_two_sum_update(hi[7], lo[7], i7);
    count_step();
    if ((FEAT & FEAT_REPROJECT) && (L.mixed_flags & MIXED_REPROJECT) && nullray) {
      const float x[4] = {hi[0], hi[1], hi[2], hi[3]};
      const float p[4] = {hi[4], hi[5], 0.0f, hi[7]};
      const float pt = null_pt<K, float>(C, x, p, 1.0f, hi[4]);
      if (isfinite(pt)) two_sum_update(hi[4], lo[4], (pt - hi[4]) - lo[4]);
    }
    return STEP_OK;
  }

  // FP64 RK4 with the closed-form right-hand side (band steps).
  template <int K>
  __device__ __forceinline__ int step_fp64_k(const TraceLaunch& L) {
    AConsts<double> Cd;
    Cd.init(L.M);
    double y[8];
    to_double_k<K>(y);
    double s0 = 0.0, c0 = 1.0;
    if (K == KIND_SCHWARZSCHILD || K == KIND_MORRIS_THORNE) ::sincos(y[2], &s0, &c0);
    const double zero[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double k[8], acc[8], d[8];
    rhs_analytic<K, double>(Cd, y, zero, s0, c0, k);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      acc[i] = k[i];
      d[i] = L.half_step * k[i];
    }
    double rmin = d[1];
    rhs_analytic<K, double>(Cd, y, d, s0, c0, k);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      acc[i] = ::fma(2.0, k[i], acc[i]);
      d[i] = L.half_step * k[i];
    }
    rmin = fmin(rmin, d[1]);
    rhs_analytic<K, double>(Cd, y, d, s0, c0, k);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      acc[i] = ::fma(2.0, k[i], acc[i]);
      d[i] = L.step * k[i];
    }
    rmin = fmin(rmin, d[1]);
    rhs_analytic<K, double>(Cd, y, d, s0, c0, k);
    if (K == KIND_SCHWARZSCHILD && !(y[1] + rmin > Cd.two_m)) return STEP_HORIZON;
    double yn[8];
    bool finite = true;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      yn[i] = ::fma(L.sixth, acc[i] + k[i], y[i]);
      finite &= isfinite(yn[i]);
    }
    if (!finite) return STEP_NONFINITE;
    load_state(yn);
    count_step();
    return STEP_OK;
  }

  template <int K>
  __device__ __forceinline__ int step_k(const TraceLaunch& L) {
    if ((FEAT & FEAT_BAND) && K != KIND_MINKOWSKI && L.band > 0.0f && in_band<K>(L.M, hi[1], hi[2], hi[3], L.band))
      return step_fp64_k<K>(L);
    if (any_orbit<K>() && orbit) return step_fp32_planar_k<K>(L);
    if (K == KIND_SCHWARZSCHILD && (FEAT & (FEAT_PLANAR | FEAT_PLANAR_DYN)) && ((FEAT & FEAT_PLANAR) || planar))
      return step_fp32_planar_k<K>(L);
    return step_fp32_k<K>(L);
  }

  __device__ __forceinline__ void finish(const TraceLaunch&) {}
  // Serving: rays of different jobs pass through one lane, so the per-job
  // constants are rebuilt when a lane takes a ray of another job.
  __device__ __forceinline__ void rebind(const TraceLaunch& L) { setup(L); }
  __device__ __forceinline__ void save(uint32_t w[16]) const {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      w[i] = __float_as_uint(hi[i]);
      w[8 + i] = __float_as_uint(lo[i]);
    }
  }
  __device__ __forceinline__ void restore(const TraceLaunch& L, const uint32_t w[16], int64_t n) {
    setup(L);
    nsteps = (unsigned)n;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      hi[i] = __uint_as_float(w[i]);
      lo[i] = __uint_as_float(w[8 + i]);
    }
  }
};


// The stepper of one metric kind K (every ray of the launch has that kind).
template <int K, int FEAT = 0>
struct MixedStepper : MixedCore<FEAT> {
  __device__ __forceinline__ void resume_frame(const TraceLaunch& L, int64_t ray) {
    this->template resume_frame_k<K>(L, ray);
  }
  __device__ __forceinline__ void load(const TraceLaunch& L, const double y0[8]) { this->template load_k<K>(L, y0); }
  __device__ __forceinline__ void to_double(double out[8]) const { this->template to_double_k<K>(out); }
  __device__ __forceinline__ int terminate(const TraceLaunch& L) const { return this->template terminate_k<K>(L); }
  __device__ __forceinline__ int step(const TraceLaunch& L) { return this->template step_k<K>(L); }
  __device__ __forceinline__ void group_end(const TraceLaunch& L) { this->template group_end_k<K>(L); }
  __device__ __forceinline__ void check_null(const TraceLaunch& L, const double y0[8]) {
    this->template check_null_k<K>(L, y0);
  }
};

// The stepper of a launch whose rays have different metric kinds (several
// renders traced by one persistent kernel): each lane keeps the kind of the
// ray it holds and branches on it; lanes of a warp mostly hold rays of one job,
// claimed together, so the branch is mostly uniform. KMASK (bit K for metric
// kind K) lists the kinds the launch holds: only their steps are compiled in,
// which keeps the kernel's registers near those of the largest single step.
template <int FEAT, int KMASK = 15>
struct MixedStepperAny : MixedCore<FEAT> {
  int kind = KIND_MINKOWSKI;
  // f(std::integral_constant<int, K>) for the lane's kind K among KMASK's
  template <class F>
  __device__ __forceinline__ auto on_kind(F&& f) const {
    using S = std::integral_constant<int, KIND_SCHWARZSCHILD>;
    using T = std::integral_constant<int, KIND_MORRIS_THORNE>;
    using A = std::integral_constant<int, KIND_ALCUBIERRE>;
    using M = std::integral_constant<int, KIND_MINKOWSKI>;
    if constexpr ((KMASK >> KIND_SCHWARZSCHILD) & 1) {
      if (kind == KIND_SCHWARZSCHILD || KMASK == (1 << KIND_SCHWARZSCHILD)) return f(S{});
    }
    if constexpr ((KMASK >> KIND_MORRIS_THORNE) & 1) {
      if (kind == KIND_MORRIS_THORNE || (KMASK & ~((1 << KIND_SCHWARZSCHILD) | (1 << KIND_MORRIS_THORNE))) == 0)
        return f(T{});
    }
    if constexpr ((KMASK >> KIND_ALCUBIERRE) & 1) {
      if (kind == KIND_ALCUBIERRE || (KMASK >> KIND_MINKOWSKI & 1) == 0) return f(A{});
    }
    return f(M{});
  }
  // A lane takes a ray of job L: its metric constants and kind.
  __device__ __forceinline__ void bind(const TraceLaunch& L, int src) {
    this->setup(L);
    kind = L.M.kind;
    this->orbit = (FEAT & FEAT_ORBIT_DYN) && src == SRC_CAMERA && (L.mixed_flags & MIXED_ORBIT) &&
                  (kind == KIND_SCHWARZSCHILD || kind == KIND_MORRIS_THORNE);
  }
  __device__ __forceinline__ void load(const TraceLaunch& L, const double y0[8]) {
    on_kind([&](auto k) { this->template load_k<decltype(k)::value>(L, y0); });
  }
  __device__ __forceinline__ void to_double(double out[8]) const {
    on_kind([&](auto k) { this->template to_double_k<decltype(k)::value>(out); });
  }
  __device__ __forceinline__ int terminate(const TraceLaunch& L) const {
    return on_kind([&](auto k) { return this->template terminate_k<decltype(k)::value>(L); });
  }
  __device__ __forceinline__ int step(const TraceLaunch& L) {
    return on_kind([&](auto k) { return this->template step_k<decltype(k)::value>(L); });
  }
  __device__ __forceinline__ void group_end(const TraceLaunch& L) {
    on_kind([&](auto k) { this->template group_end_k<decltype(k)::value>(L); });
  }
  __device__ __forceinline__ void check_null(const TraceLaunch& L, const double y0[8]) {
    on_kind([&](auto k) { this->template check_null_k<decltype(k)::value>(L, y0); });
  }
};

// MINB is the register cap chosen by the autotuner: __launch_bounds__(BLOCK,
// MINB) asks the compiler to fit MINB blocks per SM (1: no cap, 63 registers
// and 8 blocks of 128 for the planar equatorial step, 72 and 7 for the camera
// step; 8 blocks of 128: <= 64 registers; 10: <= 51), trading registers (and
// spills) for resident warps. BLOCK is the block size (128 except for the
// equatorial shadow kernel, whose autotuner also tries 64 and 256).
template <int K, int SRC, int SINK, int MINB, int FEAT, int BLOCK = TRACE_BLOCK>
__global__ void __launch_bounds__(BLOCK, MINB) trace_mixed_kernel(const TraceLaunch L) {
  constexpr int PL = (SRC == SRC_EQUATORIAL && K == KIND_SCHWARZSCHILD) ? FEAT_PLANAR : 0;
  trace_loop<MixedStepper<K, FEAT | PL>, K, SRC, SINK>(L);
}

template <int K, int SRC, int SINK, int MINB, int FEAT, int BLOCK = TRACE_BLOCK>
static cudaError_t launch_mst_v(const TraceLaunch& L, cudaStream_t s) {
  static int sms = 0, per_sm = 0;
  if (sms == 0) {
    int dev = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, trace_mixed_kernel<K, SRC, SINK, MINB, FEAT, BLOCK>, BLOCK,
                                                  0);
    per_sm = occ < 1 ? 1 : occ;
  }
  // persistent grid: every resident slot, minus what the caller keeps free for
  // a concurrent job (counted in slots of TRACE_BLOCK threads)
  const int64_t slots = persistent_slots(sms, per_sm, L.reserve_per_sm * (float)TRACE_BLOCK / (float)BLOCK);
  const int64_t need = (L.n + BLOCK - 1) / BLOCK;
  int grid = (int)(need < slots ? need : slots);
  if (grid < 1) grid = 1;
  trace_mixed_kernel<K, SRC, SINK, MINB, FEAT, BLOCK><<<grid, BLOCK, 0, s>>>(L);
  return cudaGetLastError();
}

template <int K, int SRC, int SINK>
static cudaError_t launch_mst(const TraceLaunch& L, cudaStream_t s) {
  const int feat = ((K != KIND_MINKOWSKI && L.band > 0.0f) ? FEAT_BAND : 0) |
                   ((L.mixed_flags & MIXED_REPROJECT) ? FEAT_REPROJECT : 0);
  if constexpr ((K == KIND_SCHWARZSCHILD || K == KIND_MORRIS_THORNE) && SRC != SRC_EQUATORIAL) {
    // orbit-plane frame (the default for camera rays and ray arrays of the
    // spherically symmetric metrics; equatorial rays already step on their plane)
    if (feat == 0 && (L.mixed_flags & MIXED_ORBIT)) {
      switch (L.variant % 3) {
        case 1: return launch_mst_v<K, SRC, SINK, 8, FEAT_ORBIT>(L, s);
        case 2: return launch_mst_v<K, SRC, SINK, 10, FEAT_ORBIT>(L, s);
        default: return launch_mst_v<K, SRC, SINK, 1, FEAT_ORBIT>(L, s);
      }
    }
  }
  switch (feat) {  // the optional parts run without a register cap
    case FEAT_BAND: return launch_mst_v<K, SRC, SINK, 1, FEAT_BAND>(L, s);
    case FEAT_REPROJECT: return launch_mst_v<K, SRC, SINK, 1, FEAT_REPROJECT>(L, s);
    case FEAT_BAND | FEAT_REPROJECT: return launch_mst_v<K, SRC, SINK, 1, FEAT_BAND | FEAT_REPROJECT>(L, s);
  }
  if constexpr (SRC == SRC_EQUATORIAL && SINK == SINK_SHADOW) {
    if (L.decide) return launch_mst_v<K, SRC, SINK, 1, FEAT_DECIDE>(L, s);  // bisection rounds
    // variant = register cap + 3 * block size (128, 64, 256); the same caps in
    // registers per thread (64, 51) at every block size
    switch (L.variant) {
      case 1: return launch_mst_v<K, SRC, SINK, 8, 0>(L, s);
      case 2: return launch_mst_v<K, SRC, SINK, 10, 0>(L, s);
      case 3: return launch_mst_v<K, SRC, SINK, 1, 0, 64>(L, s);
      case 4: return launch_mst_v<K, SRC, SINK, 16, 0, 64>(L, s);
      case 5: return launch_mst_v<K, SRC, SINK, 20, 0, 64>(L, s);
      case 6: return launch_mst_v<K, SRC, SINK, 1, 0, 256>(L, s);
      case 7: return launch_mst_v<K, SRC, SINK, 4, 0, 256>(L, s);
      case 8: return launch_mst_v<K, SRC, SINK, 5, 0, 256>(L, s);
      default: return launch_mst_v<K, SRC, SINK, 1, 0>(L, s);
    }
  } else {
    switch (L.variant % 3) {
      case 1: return launch_mst_v<K, SRC, SINK, 8, 0>(L, s);
      case 2: return launch_mst_v<K, SRC, SINK, 10, 0>(L, s);
      default: return launch_mst_v<K, SRC, SINK, 1, 0>(L, s);
    }
  }
}

// One persistent kernel over the rays of several renders (any metric kinds):
// the default mixed step per ray, camera rays of the spherically symmetric
// metrics in their orbit plane when the orbit-plane option is on (as in the
// single-render kernels, so each image equals its single render). The rays'
// states are prepared and shaded per render by the three-kernel render's
// prepare and shade kernels.
template <int KMASK>
__global__ void __launch_bounds__(TRACE_BLOCK) trace_multi_mixed_kernel(const TraceLaunch* jobs, const MultiDesc D) {
  trace_loop_multi<MixedStepperAny<FEAT_ORBIT_DYN, KMASK>, SRC_STATE, SINK_STATE>(jobs, D);
}

template <int KMASK>
static cudaError_t launch_multi_mixed_k(const TraceLaunch* jobs, const MultiDesc& D, float reserve, cudaStream_t s) {
  static int sms = 0, per_sm = 0;
  if (sms == 0) {
    int dev = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, trace_multi_mixed_kernel<KMASK>, TRACE_BLOCK, 0);
    per_sm = occ < 1 ? 1 : occ;
  }
  const int64_t n = D.start[D.njobs];
  if (n <= 0) return cudaSuccess;
  const int64_t slots = persistent_slots(sms, per_sm, reserve);
  const int64_t need = (n + TRACE_BLOCK - 1) / TRACE_BLOCK;
  const int grid = (int)(need < slots ? need : slots);
  trace_multi_mixed_kernel<KMASK><<<grid < 1 ? 1 : grid, TRACE_BLOCK, 0, s>>>(jobs, D);
  return cudaGetLastError();
}

// One kernel per set of metric kinds a batch can hold that is worth its own
// code: one kind, Alcubierre with Morris-Thorne (the exotic pair), and any.
cudaError_t launch_trace_multi_mixed(const TraceLaunch* jobs, const MultiDesc& D, float reserve, cudaStream_t s) {
  constexpr int S = 1 << KIND_SCHWARZSCHILD, T = 1 << KIND_MORRIS_THORNE, A = 1 << KIND_ALCUBIERRE,
                M = 1 << KIND_MINKOWSKI;
  switch (D.kind_mask) {
    case S: return launch_multi_mixed_k<S>(jobs, D, reserve, s);
    case T: return launch_multi_mixed_k<T>(jobs, D, reserve, s);
    case A: return launch_multi_mixed_k<A>(jobs, D, reserve, s);
    case M: return launch_multi_mixed_k<M>(jobs, D, reserve, s);
    case A | T: return launch_multi_mixed_k<A | T>(jobs, D, reserve, s);
    default: return launch_multi_mixed_k<S | T | A | M>(jobs, D, reserve, s);
  }
}

// Serving engine kernel for the mixed-precision classes (serve_common.cuh),
// no register cap. The server runs the default mixed step (no FP64 band, no
// re-projection; camera rays of the spherically symmetric metrics in their
// orbit plane, equatorial rays on theirs), as the single calls do by default.
template <int K>
__global__ void __launch_bounds__(TRACE_BLOCK, 7) serve_mixed_kernel(const ServeJob* jobs, ServeCounters cnt,
                                                                     ServeClass* cl, const unsigned* epoch, int budget) {
  constexpr int F = K == KIND_SCHWARZSCHILD ? (FEAT_PLANAR_DYN | FEAT_ORBIT_DYN | FEAT_DECIDE_DYN)
                    : K == KIND_MORRIS_THORNE ? FEAT_ORBIT_DYN : 0;
  serve_loop<MixedStepper<K, F>, K>(jobs, cnt, cl, epoch, budget);
}

int serve_mixed_blocks_per_sm(int kind) {
  int occ = 0;
  switch (kind) {
    case KIND_MINKOWSKI: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_mixed_kernel<KIND_MINKOWSKI>, TRACE_BLOCK, 0); break;
    case KIND_SCHWARZSCHILD: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_mixed_kernel<KIND_SCHWARZSCHILD>, TRACE_BLOCK, 0); break;
    case KIND_ALCUBIERRE: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_mixed_kernel<KIND_ALCUBIERRE>, TRACE_BLOCK, 0); break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_mixed_kernel<KIND_MORRIS_THORNE>, TRACE_BLOCK, 0); break;
  }
  return occ < 1 ? 1 : occ;
}

cudaError_t launch_serve_mixed(int kind, const ServeJob* jobs, ServeCounters cnt, ServeClass* cl,
                               const unsigned* epoch, int budget, int blocks, cudaStream_t s) {
  switch (kind) {
    case KIND_MINKOWSKI: serve_mixed_kernel<KIND_MINKOWSKI><<<blocks, TRACE_BLOCK, 0, s>>>(jobs, cnt, cl, epoch, budget); break;
    case KIND_SCHWARZSCHILD: serve_mixed_kernel<KIND_SCHWARZSCHILD><<<blocks, TRACE_BLOCK, 0, s>>>(jobs, cnt, cl, epoch, budget); break;
    case KIND_ALCUBIERRE: serve_mixed_kernel<KIND_ALCUBIERRE><<<blocks, TRACE_BLOCK, 0, s>>>(jobs, cnt, cl, epoch, budget); break;
    case KIND_MORRIS_THORNE: serve_mixed_kernel<KIND_MORRIS_THORNE><<<blocks, TRACE_BLOCK, 0, s>>>(jobs, cnt, cl, epoch, budget); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <int K>
static cudaError_t launch_mk(const TraceLaunch& L, int src, int sink, cudaStream_t s) {
  if (src == SRC_ARRAY && sink == SINK_TRACE) return launch_mst<K, SRC_ARRAY, SINK_TRACE>(L, s);
  if (src == SRC_CAMERA && sink == SINK_RENDER) return launch_mst<K, SRC_CAMERA, SINK_RENDER>(L, s);
  if (src == SRC_STATE && sink == SINK_STATE) return launch_mst<K, SRC_STATE, SINK_STATE>(L, s);
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Mixed renders in three kernels. The trace kernel of a render spends almost
// all its time in the FP32 step, but its FP64 set-up and sink code (the camera
// ray, the orbit-plane frame, the null residual, the escape direction, the sky)
// sets its register count and so its occupancy. Here the set-up runs in a
// prepare kernel (camera ray -> the stepper's (hi, lo) state, 16 words per ray
// in L.ystate), the trace kernel steps those states and writes the final ones
// back in place, and a shade kernel turns them into the render sink's outputs.
// Every value is computed by the same stepper code as in the one-kernel
// render, so the results are the same bits.
// ---------------------------------------------------------------------------
template <int K, int FEAT>
__global__ void __launch_bounds__(128) render_prepare_kernel(const TraceLaunch L) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n) return;
  double y0[8];
  camera_ray(L.cam, i, y0);
  MixedStepper<K, FEAT> st;
  st.load(L, y0);
  uint32_t w[16];
  st.save(w);
  store_words(L, i, w);
}

template <int K, int FEAT>
__global__ void __launch_bounds__(128) render_shade_kernel(const TraceLaunch L) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L.n) return;
  uint32_t w[16];
  load_words(L, i, w);
  const int64_t steps = L.steps[i];
  MixedStepper<K, FEAT> st;
  st.restore(L, w, steps);
  st.resume_frame(L, i);
  double y[8];
  st.to_double(y);
  store_ray<K, SINK_RENDER>(L, i, L.term[i], y, steps);
}

// the orbit-plane frame applies to this render's rays (as in launch_mst)
static bool render_orbit(const TraceLaunch& L) {
  return (L.M.kind == KIND_SCHWARZSCHILD || L.M.kind == KIND_MORRIS_THORNE) && (L.mixed_flags & MIXED_ORBIT) &&
         !(L.band > 0.0f) && !(L.mixed_flags & MIXED_REPROJECT);
}

template <int K, int FEAT>
static cudaError_t launch_prepare_shade(const TraceLaunch& L, bool prepare, cudaStream_t s) {
  const unsigned grid = (unsigned)((L.n + 127) / 128);
  if (prepare) render_prepare_kernel<K, FEAT><<<grid, 128, 0, s>>>(L);
  else render_shade_kernel<K, FEAT><<<grid, 128, 0, s>>>(L);
  return cudaGetLastError();
}

static cudaError_t prepare_or_shade(const TraceLaunch& L, bool prepare, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  const bool orbit = render_orbit(L);
  switch (L.M.kind) {
    case KIND_MINKOWSKI: return launch_prepare_shade<KIND_MINKOWSKI, 0>(L, prepare, s);
    case KIND_SCHWARZSCHILD:
      return orbit ? launch_prepare_shade<KIND_SCHWARZSCHILD, FEAT_ORBIT>(L, prepare, s)
                   : launch_prepare_shade<KIND_SCHWARZSCHILD, 0>(L, prepare, s);
    case KIND_ALCUBIERRE: return launch_prepare_shade<KIND_ALCUBIERRE, 0>(L, prepare, s);
    case KIND_MORRIS_THORNE:
      return orbit ? launch_prepare_shade<KIND_MORRIS_THORNE, FEAT_ORBIT>(L, prepare, s)
                   : launch_prepare_shade<KIND_MORRIS_THORNE, 0>(L, prepare, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_render_prepare(const TraceLaunch& L, cudaStream_t s) { return prepare_or_shade(L, true, s); }
cudaError_t launch_render_shade(const TraceLaunch& L, cudaStream_t s) { return prepare_or_shade(L, false, s); }

cudaError_t launch_render_mixed(const TraceLaunch& L, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  if (L.band > 0.0f || (L.mixed_flags & MIXED_REPROJECT))  // the chart options keep the one-kernel render
    return launch_trace_mixed(L, SRC_CAMERA, SINK_RENDER, s);
  cudaError_t e = launch_render_prepare(L, s);
  if (e == cudaSuccess) e = launch_trace_mixed(L, SRC_STATE, SINK_STATE, s);
  if (e == cudaSuccess) e = launch_render_shade(L, s);
  return e;
}

cudaError_t launch_trace_mixed(const TraceLaunch& L, int src, int sink, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  if (src == SRC_EQUATORIAL) {
    if (L.M.kind != KIND_SCHWARZSCHILD) return cudaErrorInvalidValue;
    if (sink == SINK_SHADOW) return launch_mst<KIND_SCHWARZSCHILD, SRC_EQUATORIAL, SINK_SHADOW>(L, s);
    if (sink == SINK_TRACE) return launch_mst<KIND_SCHWARZSCHILD, SRC_EQUATORIAL, SINK_TRACE>(L, s);
    return cudaErrorInvalidValue;
  }
  switch (L.M.kind) {
    case KIND_MINKOWSKI: return launch_mk<KIND_MINKOWSKI>(L, src, sink, s);
    case KIND_SCHWARZSCHILD: return launch_mk<KIND_SCHWARZSCHILD>(L, src, sink, s);
    case KIND_ALCUBIERRE: return launch_mk<KIND_ALCUBIERRE>(L, src, sink, s);
    case KIND_MORRIS_THORNE: return launch_mk<KIND_MORRIS_THORNE>(L, src, sink, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace geon
