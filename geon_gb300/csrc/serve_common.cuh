// Device side of the serving engine (serve.cu): a work queue of ray jobs shared
// by many requests, and the persistent kernel loop that drains it.
//
// Each job holds a claim counter. Before every launch the host writes, per
// class (metric kind x precision), the claim order: the jobs that still have
// unclaimed rays, fewest first. A warp refills its idle lanes first from the
// class's resume pool (rays interrupted at the end of the previous launch),
// then from the jobs in that order, one atomic per warp per job. A launch runs
// a fixed number of warp iterations (one RK4 step each); rays still in flight
// then write their state to the other resume buffer and are picked up by the
// next launch, so ray state stays resident in HBM between launches and new
// requests join at every launch (continuous batching). All loops are bounded:
// the iteration budget, and the length of the claim order.
#pragma once
#include "trace_common.cuh"

namespace geon {

constexpr int SERVE_MAX_JOBS = 4096;              // job slots
constexpr unsigned SERVE_RING = SERVE_MAX_JOBS;   // claim-order entries per class
constexpr int SERVE_CLASSES = 8;        // 4 metric kinds x 2 precisions

struct ServeJob {
  TraceLaunch L;  // metric, source, sink and output pointers; L.n = rays
  int src, sink;
};

// Per-slot counters, kept in flat arrays so the host reads every job's
// progress with one small copy per launch.
struct ServeCounters {
  unsigned long long* next;   // next unclaimed ray (atomic)
  unsigned long long* done;   // rays finished (atomic)
  unsigned long long* steps;  // ray-steps integrated (atomic)
  const unsigned* cancel;     // non-zero: drop the job's rays (set by the host between launches)
};

struct ResumeEntry {
  int slot;
  int pad;
  long long ray;
  long long n;
  uint32_t w[16];
};

struct ServeClass {
  unsigned tail;                         // entries in the claim order (host, before each launch)
  unsigned head;                         // entries fully claimed (host sets 0; kernels, atomicMax)
  unsigned long long resume_count[2];    // entries in each resume buffer
  unsigned long long resume_claim;       // entries of the input buffer taken this launch
  unsigned long long resume_cap;         // capacity of each buffer
  unsigned long long resume_lost;        // entries that did not fit (must stay 0)
  ResumeEntry* resume[2];
  int* ring;
};

template <int K, int SRC>
__device__ __forceinline__ void serve_load(const TraceLaunch& L, int64_t ray, double y[8]) {
  load_ray<SRC>(L, ray, y);
}

template <class Stepper, int K>
__device__ __forceinline__ void serve_loop(const ServeJob* __restrict__ jobs, ServeCounters cnt, ServeClass* cl,
                                           const unsigned* epoch_ptr, int budget) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const unsigned epoch = *epoch_ptr;
  const int pin = (int)(epoch & 1u), pout = pin ^ 1;
  const unsigned long long in_count =
      cl->resume_count[pin] < cl->resume_cap ? cl->resume_count[pin] : cl->resume_cap;
  const ResumeEntry* in = cl->resume[pin];
  ResumeEntry* out = cl->resume[pout];
  const unsigned tail = cl->tail;
  int slot = -1;
  long long ray = 0, n = 0;
  Stepper st;
  bool resume_open = in_count > 0, jobs_open = true;
  for (int it = 0; it < budget; it += TRACE_INNER) {  // budget counts steps; TRACE_INNER per refill
    unsigned need = __ballot_sync(FULL, slot < 0);
    if (need && resume_open) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&cl->resume_claim, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (base + __popc(need) >= in_count) resume_open = false;
      if (slot < 0) {
        const unsigned long long idx = base + __popc(need & lt_mask);
        if (idx < in_count) {
          const ResumeEntry& e = in[idx];
          if (cnt.cancel[e.slot]) {
            atomicAdd(&cnt.done[e.slot], 1ull);
          } else {
            slot = e.slot;
            ray = e.ray;
            n = e.n;
            st.restore(jobs[slot].L, e.w, n);
            st.set_source(jobs[slot].src);
            st.resume_frame(jobs[slot].L, ray);
          }
        }
      }
      need = __ballot_sync(FULL, slot < 0);
    }
    // one read of the shared head per warp: every lane must walk the same
    // claim-order positions, since lane offsets are taken from the leader's claim
    unsigned pos = tail;
    if (jobs_open) {
      if (lane == 0) pos = atomicAdd(&cl->head, 0u);
      pos = __shfl_sync(FULL, pos, 0);
    }
    while (need && jobs_open) {
      if (pos >= tail) {
        jobs_open = false;
        break;
      }
      const int js = cl->ring[pos % SERVE_RING];
      if (cnt.cancel[js]) {  // cancelled job: nothing more to claim
        if (lane == 0) atomicMax(&cl->head, pos + 1);
        ++pos;
        continue;
      }
      const ServeJob& J = jobs[js];
      const int leader = __ffs(need) - 1;
      const unsigned c = __popc(need);
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(&cnt.next[js], (unsigned long long)c);
      base = __shfl_sync(FULL, base, leader);
      const unsigned long long total = (unsigned long long)J.L.n;
      if (base + c >= total) {  // this job has no unclaimed rays left after this claim
        if (lane == leader) atomicMax(&cl->head, pos + 1);
        ++pos;
      }
      if (base < total && slot < 0) {
        const unsigned long long idx = base + __popc(need & lt_mask);
        if (idx < total) {
          slot = js;
          ray = (long long)idx;
          n = 0;
          double y0[8];
          if (J.src == SRC_CAMERA) serve_load<K, SRC_CAMERA>(J.L, ray, y0);
          else if (J.src == SRC_EQUATORIAL) serve_load<K, SRC_EQUATORIAL>(J.L, ray, y0);
          else serve_load<K, SRC_ARRAY>(J.L, ray, y0);
          st.rebind(J.L);
          st.set_source(J.src);
          st.load(J.L, y0);
        }
      }
      need = __ballot_sync(FULL, slot < 0);
    }
    if (__ballot_sync(FULL, slot >= 0) == 0) break;
    if (slot >= 0) {
      const TraceLaunch& L = jobs[slot].L;
#pragma unroll 1
      for (int inner = 0; inner < TRACE_INNER; ++inner) {
        int t = TERM_NONE;
        long long taken = n;
        if (n >= L.max_steps) {
          t = TERM_DIVERGED;
          taken = L.max_steps;
        } else {
          t = st.terminate(L);
          if (t == TERM_NONE) {
            const int r = st.step(L);
            if (r == STEP_OK) {
              ++n;
            } else if (r == STEP_NONFINITE) {
              t = TERM_DIVERGED;
            } else {
              t = TERM_CAPTURED;
              taken = n + 1;
            }
          }
        }
        if (t != TERM_NONE) {
          double y[8];
          st.to_double(y);
          const int sink = jobs[slot].sink;
          if (sink == SINK_RENDER) store_ray<K, SINK_RENDER>(L, ray, t, y, taken);
          else if (sink == SINK_SHADOW) store_ray<K, SINK_SHADOW>(L, ray, t, y, taken);
          else store_ray<K, SINK_TRACE>(L, ray, t, y, taken);
          atomicAdd(&cnt.steps[slot], (unsigned long long)taken);
          __threadfence();
          atomicAdd(&cnt.done[slot], 1ull);
          slot = -1;
          break;
        }
      }
      if (slot >= 0) st.group_end(L);  // the ray survived a whole group of TRACE_INNER steps
    }
  }
  if (slot >= 0) {  // out of budget: park the ray for the next launch
    const unsigned long long idx = atomicAdd(&cl->resume_count[pout], 1ull);
    if (idx < cl->resume_cap) {
      ResumeEntry e;
      e.slot = slot;
      e.pad = 0;
      e.ray = ray;
      e.n = n;
      st.save(e.w);
      out[idx] = e;
    } else {
      atomicAdd(&cl->resume_lost, 1ull);
    }
  }
}

}  // namespace geon
