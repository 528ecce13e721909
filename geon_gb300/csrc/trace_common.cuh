// Ray sources, result sinks and the persistent work-queue loop shared by the
// FP64 and mixed-precision steppers.
//
// One thread owns one ray at a time; the ray state stays in registers for its
// whole life. Each warp pulls ray indices from a device work queue with one
// atomic per refill (ballot + popc + shuffle), so a lane whose ray is captured
// or escapes picks up a fresh ray at the next step instead of idling until the
// slowest ray of its warp finishes.
#pragma once
#include "internal.h"
#include "metric_fp64.cuh"
#include "sky.cuh"

namespace geon {

// ---------------------------------------------------------------------------
// Sources of initial states
// ---------------------------------------------------------------------------
// camera.rs:113-160 (ray_state_sub), with forward_sign = +1 the reference.
__device__ __forceinline__ void camera_ray(const CameraDesc& c, int64_t ray, double y[8]) {
  const int64_t spa2 = c.spa * c.spa;
  const int64_t pix = ray / spa2;
  const int64_t sub = ray - pix * spa2;
  const int64_t sj = sub / c.spa, si = sub - sj * c.spa;
  const int64_t j = pix / c.width, i = pix - j * c.width;
  const double du = ((double)si + 0.5) * c.inv_spa;
  const double dv = ((double)sj + 0.5) * c.inv_spa;
  const double u = (2.0 * ((double)i + du) / c.width_d - 1.0) * c.w_img;
  const double v = -(2.0 * ((double)j + dv) / c.height_d - 1.0) * c.h_img;
  const double fs = (double)c.forward_sign;
  const double dx = -fs;
  const double dy = -v;
  const double dz = c.forward_sign == 1 ? u : fs * u;
  const double norm = sqrt(dx * dx + dy * dy + dz * dz);
  const double n1 = dx / norm, n2 = dy / norm, n3 = dz / norm;
#pragma unroll
  for (int mu = 0; mu < 4; ++mu) y[mu] = c.obs[mu];
#pragma unroll
  for (int mu = 0; mu < 4; ++mu)
    y[4 + mu] = c.tet[0][mu] + n1 * c.tet[1][mu] + n2 * c.tet[2][mu] + n3 * c.tet[3][mu];
}

// bin/validate_shadow.rs:20-35
__device__ __forceinline__ void equatorial_ray(double m, double r_obs, double alpha, double y[8]) {
  const double f = 1.0 - 2.0 * m / r_obs;
  double sin_a, cos_a;
  dm::sincos_det(alpha, &sin_a, &cos_a);
  const double sf = sqrt(f);
  y[0] = 0.0;
  y[1] = r_obs;
  y[2] = 1.5707963267948966;  // FRAC_PI_2
  y[3] = 0.0;
  y[4] = 1.0 / sf;
  y[5] = -cos_a * sf;
  y[6] = 0.0;
  y[7] = sin_a / r_obs;
}

template <int SRC>
__device__ __forceinline__ void load_ray(const TraceLaunch& L, int64_t ray, double y[8]) {
  if (SRC == SRC_ARRAY) {
    const double2* p = reinterpret_cast<const double2*>(L.y0 + 8 * ray);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double2 v = p[q];
      y[2 * q] = v.x;
      y[2 * q + 1] = v.y;
    }
  } else if (SRC == SRC_CAMERA) {
    camera_ray(L.cam, ray, y);
  } else {
    equatorial_ray(L.M.p[0], L.r_obs, L.alpha[ray], y);
  }
}

// A ray's prepared or final stepper state: 16 words, four 16-byte accesses.
__device__ __forceinline__ void load_words(const TraceLaunch& L, int64_t ray, uint32_t w[16]) {
  const uint4* p = reinterpret_cast<const uint4*>(L.ystate + 16 * ray);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint4 v = p[q];
    w[4 * q] = v.x; w[4 * q + 1] = v.y; w[4 * q + 2] = v.z; w[4 * q + 3] = v.w;
  }
}
__device__ __forceinline__ void store_words(const TraceLaunch& L, int64_t ray, const uint32_t w[16]) {
  uint4* p = reinterpret_cast<uint4*>(L.ystate + 16 * ray);
#pragma unroll
  for (int q = 0; q < 4; ++q) p[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
}

template <int K, int SINK>
__device__ __forceinline__ void store_ray(const TraceLaunch& L, int64_t ray, int term,
                                          const double y[8], int64_t steps) {
  if (SINK == SINK_SHADOW) {
    L.term[ray] = term;
    if (L.steps) L.steps[ray] = steps;
    return;
  }
  const double resid = null_residual<K>(L.M, y);
  if (SINK == SINK_TRACE) {
    L.term[ray] = term;
    double2* o = reinterpret_cast<double2*>(L.yfinal + 8 * ray);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = make_double2(y[2 * q], y[2 * q + 1]);
    L.steps[ray] = steps;
    L.resid[ray] = resid;
  } else {  // SINK_RENDER (render.rs:77-101)
    float rgb[3];
    if (term == TERM_CAPTURED) {
      rgb[0] = L.captured_rgb[0]; rgb[1] = L.captured_rgb[1]; rgb[2] = L.captured_rgb[2];
    } else if (term == TERM_DIVERGED) {
      rgb[0] = L.diverged_rgb[0]; rgb[1] = L.diverged_rgb[1]; rgb[2] = L.diverged_rgb[2];
    } else {
      double dir[3];
      metric_asymptotic_direction<K>(L.M, y, y + 4, dir);
      sky_sample(dir, L.show_stars != 0, rgb);
    }
    L.srgb[3 * ray + 0] = rgb[0];
    L.srgb[3 * ray + 1] = rgb[1];
    L.srgb[3 * ray + 2] = rgb[2];
    L.term[ray] = term;
    L.steps[ray] = steps;
    L.resid[ray] = resid;
  }
}

constexpr int TRACE_BLOCK = 128;
// Steps a lane takes between two refills of its warp: the ballots and the
// queue test are paid once per TRACE_INNER steps; a lane whose ray ends inside
// the group waits at most TRACE_INNER - 1 steps for the next ray.
constexpr int TRACE_INNER = 16;
enum : int { STEP_NONFINITE = 0, STEP_OK = 1, STEP_HORIZON = 2 };

// Up to TRACE_INNER steps of one ray (geodesic.rs:71-116): the step cap, the
// termination test before every step, the step, its NaN guard. n = steps the
// ray has taken so far; returns the new count. On termination sets t and
// taken (steps_taken of the reference: max_steps at the cap, the steps before
// a test that ends the ray or a non-finite step, one more after a horizon
// step). The counts inside the group are 32-bit; the ray's total is 64-bit.
template <class Stepper>
__device__ __forceinline__ int64_t group_steps(Stepper& st, const TraceLaunch& L, int64_t max_steps, int64_t n,
                                               int& t, int64_t& taken) {
  const int64_t left64 = max_steps - n;
  const int left = left64 < (int64_t)TRACE_INNER ? (int)left64 : TRACE_INNER;
  int done = 0, extra = 0;
  t = TERM_NONE;
#pragma unroll 1
  for (; done < left; ++done) {
    t = st.terminate(L);
    if (t != TERM_NONE) break;
    const int r = st.step(L);
    if (r != STEP_OK) {
      // NaN guard: Diverged with the pre-step state; horizon step: Captured
      // with one more step counted
      t = r == STEP_NONFINITE ? TERM_DIVERGED : TERM_CAPTURED;
      extra = r == STEP_NONFINITE ? 0 : 1;
      break;
    }
  }
  n += done;
  taken = n + extra;
  if (t == TERM_NONE) {
    if (done == TRACE_INNER) st.group_end(L);  // the ray survived a whole group of TRACE_INNER steps
    if (n >= max_steps) t = TERM_DIVERGED;     // loop exhausted: steps_taken = max_steps
  }
  return n;
}

// geodesic.rs:62-117 for every ray of the job, persistent over a work queue.
// Stepper owns the ray state: load(y0), to_double(y), terminate(L), step(L)
// returning STEP_OK (advanced), STEP_NONFINITE (state unchanged: Diverged) or
// STEP_HORIZON (state unchanged: Captured after this step).
template <class Stepper, int K, int SRC, int SINK>
__device__ __forceinline__ void trace_loop(const TraceLaunch& L) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  int64_t ray = -1;
  int64_t n = 0;
  Stepper st;
  bool queue_open = true;
  for (;;) {
    const unsigned need = __ballot_sync(FULL, ray < 0);
    if (need && queue_open) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(L.queue, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (base + __popc(need) >= (unsigned long long)L.n) queue_open = false;
      if (ray < 0) {
        const unsigned long long idx = base + __popc(need & lt_mask);
        if (idx < (unsigned long long)L.n) {
          ray = L.order ? (int64_t)L.order[idx] : (int64_t)idx;
          n = 0;
          if constexpr (SRC == SRC_STATE) {
            uint32_t w[16];
            load_words(L, ray, w);
            st.restore(L, w, 0);
          } else {
            double y0[8];
            load_ray<SRC>(L, ray, y0);
            st.load(L, y0);
            if constexpr (SRC == SRC_ARRAY) st.check_null(L, y0);  // camera and equatorial rays are null
          }
        }
      }
    }
    if (__ballot_sync(FULL, ray >= 0) == 0) break;
    if (ray >= 0) {
      int t = TERM_NONE;
      int64_t taken = 0;
      n = group_steps(st, L, L.max_steps, n, t, taken);
      if (t != TERM_NONE) {
        if constexpr (SINK == SINK_STATE) {
          uint32_t w[16];
          st.save(w);
          store_words(L, ray, w);
          L.term[ray] = t;
          L.steps[ray] = taken;
        } else {
          double y[8];
          st.to_double(y);
          store_ray<K, SINK>(L, ray, t, y, taken);
        }
        ray = -1;
      }
    }
  }
  st.finish(L);
}


// ---------------------------------------------------------------------------
// Several jobs in one persistent launch (e.g. renders of different metrics):
// one work queue over the concatenated rays, job j owning the global indices
// [start[j], start[j+1]). A lane that takes a ray finds its job by the offsets
// (a few compares: at most MULTI_MAX_JOBS jobs) and steps it with that job's
// metric, camera and outputs; the job table is in global memory (L1-resident).
// ---------------------------------------------------------------------------
// store_ray for a ray of metric kind `kind` (known at run time).
template <int SINK>
__device__ __forceinline__ void store_ray_any(const TraceLaunch& L, int kind, int64_t ray, int term,
                                              const double y[8], int64_t steps) {
  switch (kind) {
    case KIND_SCHWARZSCHILD: store_ray<KIND_SCHWARZSCHILD, SINK>(L, ray, term, y, steps); return;
    case KIND_ALCUBIERRE: store_ray<KIND_ALCUBIERRE, SINK>(L, ray, term, y, steps); return;
    case KIND_MORRIS_THORNE: store_ray<KIND_MORRIS_THORNE, SINK>(L, ray, term, y, steps); return;
    default: store_ray<KIND_MINKOWSKI, SINK>(L, ray, term, y, steps); return;
  }
}

// trace_loop over the rays of several jobs. Stepper additionally provides
// bind(L, src): take the constants and metric kind of job L for the next ray.
template <class Stepper, int SRC, int SINK>
__device__ __forceinline__ void trace_loop_multi(const TraceLaunch* __restrict__ jobs, const MultiDesc& D) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const unsigned long long total = (unsigned long long)D.start[D.njobs];
  int job = -1;
  int64_t ray = 0;
  int64_t n = 0;
  Stepper st;
  bool queue_open = true;
  for (;;) {
    const unsigned need = __ballot_sync(FULL, job < 0);
    if (need && queue_open) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(D.queue, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (base + __popc(need) >= total) queue_open = false;
      if (job < 0) {
        const unsigned long long idx = base + __popc(need & lt_mask);
        if (idx < total) {
          int j = 0;
          while (j + 1 < D.njobs && (int64_t)idx >= D.start[j + 1]) ++j;
          job = j;
          ray = (int64_t)idx - D.start[j];
          n = 0;
          const TraceLaunch& L = jobs[j];
          if constexpr (SRC == SRC_STATE) {
            uint32_t w[16];
            load_words(L, ray, w);
            st.bind(L, SRC_CAMERA);  // prepared camera rays
            st.restore(L, w, 0);
          } else {
            double y0[8];
            load_ray<SRC>(L, ray, y0);
            st.bind(L, SRC);
            st.load(L, y0);
            if constexpr (SRC == SRC_ARRAY) st.check_null(L, y0);
          }
        }
      }
    }
    if (__ballot_sync(FULL, job >= 0) == 0) break;
    if (job >= 0) {
      const TraceLaunch& L = jobs[job];
      int t = TERM_NONE;
      int64_t taken = 0;
      n = group_steps(st, L, L.max_steps, n, t, taken);
      if (t != TERM_NONE) {
        if constexpr (SINK == SINK_STATE) {
          uint32_t w[16];
          st.save(w);
          store_words(L, ray, w);
          L.term[ray] = t;
          L.steps[ray] = taken;
        } else {
          double y[8];
          st.to_double(y);
          store_ray_any<SINK>(L, L.M.kind, ray, t, y, taken);
        }
        job = -1;
      }
    }
  }
  st.finish(jobs[0]);
}

}  // namespace geon
