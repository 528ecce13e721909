// Serving engine: continuous batching of render, shadow-bisection and
// curvature requests on one GPU (the geon_server_* entry points).
//
// A server owns a device arena of `budget` bytes. A request is admitted when a
// job slot is free and its buffers fit in the arena; requests wait in arrival
// order, and a smaller one may pass a larger one that does not fit yet. Ray work
// (render samples, bisection rounds) goes to the device work queue of
// serve_common.cuh, one class per metric kind and precision. The serving thread
// runs launches ("epochs"): each is one CUDA graph - a prologue, one persistent
// kernel per class on parallel branches (each runs a bounded number of RK4
// steps), then a copy of every job's progress counters to pinned host memory.
// Between epochs the thread admits arrivals, publishes their rays, walks the
// finished bisection rounds (bin/validate_shadow.rs:70-77, a round's midpoints
// forming the tree of the next L halvings) and hands finished jobs to the
// completion thread, which runs the per-pixel reduction and copies results to
// the caller. Curvature requests run as grid kernels on their own stream.
// Latency = completion time - submission time on the host's steady clock.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "internal.h"
#include "serve_common.cuh"
#include "serve_host.h"

namespace geon {
cudaError_t launch_serve_fp64(int kind, const ServeJob* jobs, ServeCounters cnt, ServeClass* cl,
                              const unsigned* epoch, int budget, int blocks, cudaStream_t s);
cudaError_t launch_serve_mixed(int kind, const ServeJob* jobs, ServeCounters cnt, ServeClass* cl,
                               const unsigned* epoch, int budget, int blocks, cudaStream_t s);
int serve_fp64_blocks_per_sm(int kind);
int serve_mixed_blocks_per_sm(int kind);
cudaError_t launch_serve_prologue(ServeClass* cls, int nclasses, unsigned* epoch, cudaStream_t s);
}  // namespace geon

using namespace geon;
using namespace geon::serve_host;

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Carves consecutive 256-byte-aligned buffers out of a base pointer (or just
// sums their sizes when base is null).
struct Carve {
  char* base;
  size_t off = 0;
  explicit Carve(char* b) : base(b) {}
  template <class T>
  T* take(int64_t count) {
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += rup(sizeof(T) * (size_t)(count > 0 ? count : 1));
    return p;
  }
};

struct RenderBufs {
  float* srgb;
  int32_t* term;
  int64_t* steps;
  double* resid;
  float* rgb;
  int32_t* pcls;
  int64_t* pst;
  unsigned long long* stats;
  uint8_t* rgb8;
};
size_t render_bufs(char* base, int64_t nsamp, int64_t npix, RenderBufs* b) {
  Carve c(base);
  RenderBufs r;
  r.srgb = c.take<float>(3 * nsamp);
  r.term = c.take<int32_t>(nsamp);
  r.steps = c.take<int64_t>(nsamp);
  r.resid = c.take<double>(nsamp);
  r.rgb = c.take<float>(3 * npix);
  r.pcls = c.take<int32_t>(npix);
  r.pst = c.take<int64_t>(npix);
  r.stats = c.take<unsigned long long>(8);
  r.rgb8 = c.take<uint8_t>(3 * npix);
  if (b) *b = r;
  return c.off;
}

struct BisectBufs {
  double* alpha;
  int32_t* term;
  int64_t* steps;
};
size_t bisect_bufs(char* base, int levels, BisectBufs* b) {
  const int64_t per = ((int64_t)1 << levels) - 1;
  Carve c(base);
  BisectBufs r;
  r.alpha = c.take<double>(per);
  r.term = c.take<int32_t>(per);
  r.steps = c.take<int64_t>(per);
  if (b) *b = r;
  return c.off;
}

struct CurvBufs {
  double* einstein;
  double* nec;
  int* flags;
};
size_t curv_bufs(char* base, int64_t np, int64_t nk, bool einstein, CurvBufs* b) {
  Carve c(base);
  CurvBufs r;
  r.einstein = einstein ? c.take<double>(16 * np) : nullptr;
  r.nec = nk > 0 ? c.take<double>(nk * np) : nullptr;
  r.flags = c.take<int>(1);
  if (b) *b = r;
  return c.off;
}

// Tree depth per round: the largest L with 2^L - 1 <= rays_per_round (1..12).
int bisect_levels_of(const geon_job& j) {
  if (j.rays_per_round <= 0) return 5;
  int lv = 1;
  while (lv < 12 && (((int64_t)1 << (lv + 1)) - 1) <= j.rays_per_round) ++lv;
  return lv;
}

enum { ST_QUEUED = 0, ST_RUNNING = 1, ST_DONE = 2 };

struct HostJob {
  uint64_t id = 0;
  geon_job spec;
  int state = ST_QUEUED;
  int error = 0;
  bool tracing = false;       // rays published and not all finished
  int stop_req = 0;           // GEON_ERR_CANCELLED / GEON_ERR_TIMEOUT once asked to stop
  bool stop_flagged = false;  // device cancel flag written
  int64_t stop_epoch = 0;     // launches completed when the flag was written
  double t_submit = 0, t_done = 0, deadline = 0;
  size_t bytes = 0, off = 0;
  int slot = -1, cls = -1;
  geon_metric_t metric = nullptr;
  int64_t npix = 0, nsamp = 0, spa = 1, nrays = 0;
  double lo = 0, hi = 0;
  int remaining = 0, levels = 5;
  std::vector<double> alpha;
  int64_t path_steps = 0;
  double ray_steps = 0;
  cudaEvent_t ev = nullptr;  // curvature: grid kernel finished
};

int class_of(int kind, int precision) { return kind * 2 + (precision == GEON_MIXED ? 1 : 0); }

// Served mixed requests run the default mixed step whatever the process-wide
// options say: orbit-plane frame for camera rays, compensated null re-projection.
constexpr int SERVE_MIXED_FLAGS = MIXED_ORBIT | MIXED_NULLFIX;

}  // namespace

struct geon_server {
  int dev = 0;
  size_t budget = 0;
  char* d_arena = nullptr;
  Arena arena;
  ServeJob* d_jobs = nullptr;
  ServeClass* d_cls = nullptr;
  unsigned long long* d_counters = nullptr;  // next | done | steps, SERVE_MAX_JOBS each
  unsigned* d_cancel = nullptr;
  unsigned long long* h_counters = nullptr;  // pinned copy of next | done | steps
  int* h_flags = nullptr;                    // pinned, one per slot (curvature singular flag)
  ServeJob* h_jobs = nullptr;                // pinned staging of descriptors
  int* d_rings = nullptr;
  ResumeEntry* d_resume = nullptr;
  unsigned* d_epoch = nullptr;
  int* h_order = nullptr;                    // pinned claim order, SERVE_RING per class
  unsigned* h_tail_head = nullptr;           // pinned (tail, head = 0) per class
  unsigned* h_one = nullptr;                 // pinned constant 1
  int blocks[SERVE_CLASSES] = {};
  int iters[SERVE_CLASSES] = {};
  cudaStream_t s_main = nullptr, s_walk = nullptr, s_side = nullptr, s_done = nullptr;
  cudaStream_t s_cls[SERVE_CLASSES] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[SERVE_CLASSES] = {};
  cudaGraphExec_t graph = nullptr;
  std::vector<int> free_slots;
  std::deque<HostJob*> waiting;
  std::vector<HostJob*> active;
  std::deque<HostJob*> finishing;  // handed to the completion thread
  std::map<uint64_t, HostJob*> jobs;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_fin;
  std::thread th, th_fin;
  bool stop = false;
  uint64_t next_id = 1;
  int fatal = 0;
  std::vector<double> lat[3];
  int64_t submitted = 0, completed = 0, failed = 0;
  double ray_steps = 0, grid_points = 0, t_first = -1, t_last = 0;
  double ray_steps_unfinished = 0;  // steps of the finished rays of cancelled / timed-out requests
  int64_t epochs = 0;
  uint64_t gen = 0;  // bumped by every submission and completion
  bool in_launch = false;  // a serving launch is on the GPU (the graph may not change)
  std::condition_variable cv_idle;
};

namespace {

int build_graph(geon_server* S) {
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(S->s_main, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return GEON_ERR_CUDA;
  // the claim order the host wrote for this launch, and (tail, head = 0)
  cudaError_t e = cudaSuccess;
  for (int c = 0; c < SERVE_CLASSES && e == cudaSuccess; ++c) {
    e = cudaMemcpyAsync(S->d_rings + (size_t)c * SERVE_RING, S->h_order + (size_t)c * SERVE_RING,
                        sizeof(int) * SERVE_RING, cudaMemcpyHostToDevice, S->s_main);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&S->d_cls[c].tail, S->h_tail_head + 2 * c, 2 * sizeof(unsigned), cudaMemcpyHostToDevice,
                          S->s_main);
  }
  if (e == cudaSuccess) e = launch_serve_prologue(S->d_cls, SERVE_CLASSES, S->d_epoch, S->s_main);
  if (e == cudaSuccess) e = cudaEventRecord(S->ev_fork, S->s_main);
  ServeCounters cnt{S->d_counters, S->d_counters + SERVE_MAX_JOBS, S->d_counters + 2 * SERVE_MAX_JOBS,
                    S->d_cancel};
  for (int c = 0; c < SERVE_CLASSES && e == cudaSuccess; ++c) {
    e = cudaStreamWaitEvent(S->s_cls[c], S->ev_fork, 0);
    const int kind = c / 2;
    if (e == cudaSuccess) {
      e = (c & 1) ? launch_serve_mixed(kind, S->d_jobs, cnt, S->d_cls + c, S->d_epoch, S->iters[c], S->blocks[c],
                                       S->s_cls[c])
                  : launch_serve_fp64(kind, S->d_jobs, cnt, S->d_cls + c, S->d_epoch, S->iters[c], S->blocks[c],
                                      S->s_cls[c]);
    }
    if (e == cudaSuccess) e = cudaEventRecord(S->ev_join[c], S->s_cls[c]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(S->s_main, S->ev_join[c], 0);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(S->h_counters, S->d_counters, sizeof(unsigned long long) * 3 * SERVE_MAX_JOBS,
                        cudaMemcpyDeviceToHost, S->s_main);
  const cudaError_t e2 = cudaStreamEndCapture(S->s_main, &g);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return GEON_ERR_CUDA;
  }
  const cudaError_t e3 = cudaGraphInstantiate(&S->graph, g, 0);
  cudaGraphDestroy(g);
  return e3 == cudaSuccess ? GEON_OK : GEON_ERR_CUDA;
}

// Publish a ray job: descriptor, zeroed counters, cancel flag cleared. It
// enters the claim order at the next launch.
cudaError_t publish(geon_server* S, HostJob* J, const ServeJob& sj) {
  const int slot = J->slot;
  S->h_jobs[slot] = sj;
  S->h_jobs[slot].L.band = 0.0f;  // served mixed requests use the default mixed step
  S->h_jobs[slot].L.mixed_flags = SERVE_MIXED_FLAGS;
  cudaError_t e = cudaMemcpyAsync(S->d_jobs + slot, S->h_jobs + slot, sizeof sj, cudaMemcpyHostToDevice, S->s_main);
  for (int k = 0; k < 3 && e == cudaSuccess; ++k)
    e = cudaMemsetAsync(S->d_counters + (size_t)k * SERVE_MAX_JOBS + slot, 0, sizeof(unsigned long long), S->s_main);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->d_cancel + slot, 0, sizeof(unsigned), S->s_main);
  if (e == cudaSuccess) e = cudaStreamSynchronize(S->s_main);  // the descriptor staging is reused
  for (int k = 0; k < 3; ++k) S->h_counters[(size_t)k * SERVE_MAX_JOBS + slot] = 0;
  J->tracing = true;
  return e;
}

// The claim order of every class for the next launch: jobs with unclaimed
// rays, fewest unclaimed first (arrival order on ties), so a small request is
// not queued behind a large one; rays already in flight continue first.
void write_claim_order(geon_server* S) {
  std::vector<ClaimEntry> entries;
  for (const HostJob* J : S->active) {
    if (!J->tracing || J->stop_flagged) continue;
    const int64_t claimed = (int64_t)S->h_counters[J->slot];
    entries.push_back({J->cls, J->nrays - (claimed < J->nrays ? claimed : J->nrays), J->id, J->slot});
  }
  unsigned counts[SERVE_CLASSES];
  claim_order(entries, SERVE_CLASSES, SERVE_RING, S->h_order, counts);
  for (int c = 0; c < SERVE_CLASSES; ++c) {
    S->h_tail_head[2 * c] = counts[c];
    S->h_tail_head[2 * c + 1] = 0;
  }
}

cudaError_t bisect_publish_round(geon_server* S, HostJob* J) {
  const int L = J->remaining < J->levels ? J->remaining : J->levels;
  bisect_tree(J->lo, J->hi, L, J->alpha);
  J->nrays = (int64_t)J->alpha.size();
  BisectBufs b;
  bisect_bufs(S->d_arena + J->off, J->levels, &b);
  cudaError_t e = cudaMemcpyAsync(b.alpha, J->alpha.data(), sizeof(double) * J->nrays, cudaMemcpyHostToDevice,
                                  S->s_main);
  if (e != cudaSuccess) return e;
  ServeJob sj;
  std::memset(&sj, 0, sizeof sj);
  sj.L = trace_launch_defaults(J->metric, J->spec.step, J->spec.max_steps);
  sj.L.n = J->nrays;
  sj.L.alpha = b.alpha;
  sj.L.r_obs = J->spec.r_obs;
  sj.L.term = b.term;
  sj.L.steps = b.steps;
  sj.src = SRC_EQUATORIAL;
  sj.sink = SINK_SHADOW;
  return publish(S, J, sj);  // synchronises s_main, so the alpha copy's source may change after
}

// Start an admitted job. Returns an error status for the job, or GEON_OK.
int start_job(geon_server* S, HostJob* J) {
  const geon_job& q = J->spec;
  if (int rc = geon_metric_create(q.metric_kind, q.metric_params, q.nparams, &J->metric)) return rc;
  char* base = S->d_arena + J->off;
  if (q.type == GEON_JOB_CURVATURE) {
    GridDesc d;
    std::memcpy(d.lo, q.grid.lo, sizeof d.lo);
    std::memcpy(d.hi, q.grid.hi, sizeof d.hi);
    std::memcpy(d.n, q.grid.n, sizeof d.n);
    d.t = q.grid.t;
    const int64_t np = d.n[0] * d.n[1] * d.n[2];
    CurvBufs b;
    curv_bufs(base, np, q.nk, q.einstein != nullptr, &b);
    if (cudaMemsetAsync(b.flags, 0, sizeof(int), S->s_side) != cudaSuccess) return GEON_ERR_CUDA;
    note_launches(1);
    if (launch_curvature_grid(*metric_desc(J->metric), d, q.nk, q.seed, b.einstein, b.nec, nullptr, b.flags,
                              S->s_side) != cudaSuccess)
      return GEON_ERR_CUDA;
    if (cudaEventCreateWithFlags(&J->ev, cudaEventDisableTiming) != cudaSuccess) return GEON_ERR_CUDA;
    if (cudaEventRecord(J->ev, S->s_side) != cudaSuccess) return GEON_ERR_CUDA;
    return GEON_OK;
  }
  J->cls = class_of(q.metric_kind, q.precision);
  if (q.type == GEON_JOB_RENDER) {
    CameraDesc c;
    if (int rc = camera_desc_for(J->metric, &q.camera, J->spa, c, S->s_main)) return rc;
    RenderBufs b;
    render_bufs(base, J->nsamp, J->npix, &b);
    ServeJob sj;
    std::memset(&sj, 0, sizeof sj);
    sj.L = trace_launch_defaults(J->metric, q.render.step, q.render.max_steps);
    sj.L.cam = c;
    sj.L.n = J->nsamp;
    sj.L.srgb = b.srgb;
    sj.L.term = b.term;
    sj.L.steps = b.steps;
    sj.L.resid = b.resid;
    sj.L.show_stars = q.render.show_stars < 0 ? geon_get_show_stars() : (q.render.show_stars != 0);
    for (int k = 0; k < 3; ++k) {
      sj.L.captured_rgb[k] = q.render.captured_rgb[k];
      sj.L.diverged_rgb[k] = q.render.diverged_rgb[k];
    }
    sj.src = SRC_CAMERA;
    sj.sink = SINK_RENDER;
    J->nrays = J->nsamp;
    return publish(S, J, sj) == cudaSuccess ? GEON_OK : GEON_ERR_CUDA;
  }
  J->lo = q.lo;
  J->hi = q.hi;
  J->remaining = q.iters;
  if (J->remaining <= 0) return GEON_OK;  // nothing to trace: done at once
  return bisect_publish_round(S, J) == cudaSuccess ? GEON_OK : GEON_ERR_CUDA;
}

void release(geon_server* S, HostJob* J) {
  if (J->bytes && J->state != ST_QUEUED) S->arena.release(J->off, J->bytes);
  J->bytes = 0;
  if (J->slot >= 0) S->free_slots.push_back(J->slot);
  J->slot = -1;
  if (J->ev) {
    cudaEventDestroy(J->ev);
    J->ev = nullptr;
  }
  if (J->metric) {
    geon_metric_destroy(J->metric);
    J->metric = nullptr;
  }
}

// Record the end of a job (lock held).
void finish(geon_server* S, HostJob* J, int error) {
  release(S, J);
  J->t_done = now_s();
  J->error = error;
  J->state = ST_DONE;
  if (error) {
    ++S->failed;
    S->ray_steps_unfinished += J->ray_steps;
  } else {
    ++S->completed;
    S->lat[J->spec.type].push_back(1e3 * (J->t_done - J->t_submit));
    S->ray_steps += J->ray_steps;
    if (J->spec.type == GEON_JOB_CURVATURE)
      S->grid_points += (double)(J->spec.grid.n[0] * J->spec.grid.n[1] * J->spec.grid.n[2]);
  }
  S->t_last = J->t_done;
  ++S->gen;
  S->cv_done.notify_all();
}

void hand_off(geon_server* S, HostJob* J) {
  S->finishing.push_back(J);
  S->cv_fin.notify_all();
}

// A bisection round's rays all finished: walk its tree, then publish the next
// round or hand the job off (lock held).
int bisect_round_done(geon_server* S, HostJob* J) {
  BisectBufs b;
  bisect_bufs(S->d_arena + J->off, J->levels, &b);
  const int64_t per = J->nrays;
  int L = 0;
  while ((((int64_t)1 << (L + 1)) - 1) <= per) ++L;
  std::vector<int32_t> term(per);
  std::vector<int64_t> steps(per);
  cudaError_t e = cudaMemcpyAsync(term.data(), b.term, sizeof(int32_t) * per, cudaMemcpyDeviceToHost, S->s_walk);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(steps.data(), b.steps, sizeof(int64_t) * per, cudaMemcpyDeviceToHost, S->s_walk);
  if (e == cudaSuccess) e = cudaStreamSynchronize(S->s_walk);
  if (e != cudaSuccess) return GEON_ERR_CUDA;
  int64_t node = 1;
  for (int d = 0; d < L; ++d) {
    J->path_steps += steps[node - 1];
    if (term[node - 1] == TERM_CAPTURED) {
      J->lo = J->alpha[node - 1];
      node = 2 * node + 1;
    } else {
      J->hi = J->alpha[node - 1];
      node = 2 * node;
    }
  }
  J->remaining -= L;
  if (J->remaining > 0 && !J->stop_req) return bisect_publish_round(S, J) == cudaSuccess ? GEON_OK : GEON_ERR_CUDA;
  J->tracing = false;
  hand_off(S, J);
  return GEON_OK;
}

// A CUDA error ends the server: every job still queued or running fails.
void fail_all(geon_server* S, int code) {
  S->fatal = code;
  for (HostJob* J : S->active)
    if (J->state != ST_DONE) finish(S, J, code);
  S->active.clear();
  for (HostJob* J : S->waiting) finish(S, J, code);
  S->waiting.clear();
  S->finishing.clear();
  S->cv_fin.notify_all();
}

bool any_tracing(const geon_server* S) {
  for (const HostJob* J : S->active)
    if (J->tracing) return true;
  return false;
}

void server_loop(geon_server* S) {
  cudaSetDevice(S->dev);
  std::unique_lock<std::mutex> lk(S->mu);
  while (!S->stop && !S->fatal) {
    const double now = now_s();
    // 1. deadlines
    for (auto it = S->waiting.begin(); it != S->waiting.end();) {
      HostJob* J = *it;
      if (J->deadline > 0 && now > J->deadline) {
        it = S->waiting.erase(it);
        finish(S, J, GEON_ERR_TIMEOUT);
      } else {
        ++it;
      }
    }
    for (HostJob* J : S->active)
      if (J->deadline > 0 && now > J->deadline && !J->stop_req) J->stop_req = GEON_ERR_TIMEOUT;
    // 2. admission, in arrival order; a request that does not fit lets later ones pass
    for (auto it = S->waiting.begin(); it != S->waiting.end() && !S->fatal;) {
      HostJob* J = *it;
      size_t off = 0;
      if (S->free_slots.empty() || !S->arena.alloc(J->bytes, &off)) {
        ++it;
        continue;
      }
      J->off = off;
      J->slot = S->free_slots.back();
      S->free_slots.pop_back();
      J->state = ST_RUNNING;
      it = S->waiting.erase(it);
      const int rc = start_job(S, J);
      if (rc == GEON_ERR_CUDA) {
        finish(S, J, rc);
        fail_all(S, GEON_ERR_CUDA);
      } else if (rc) {
        finish(S, J, rc);
      } else {
        S->active.push_back(J);
        if (!J->tracing) hand_off(S, J);  // curvature, or a bisection with nothing to trace
      }
    }
    if (S->fatal) break;
    // 3. stop requests on tracing jobs: raise the device flag once
    for (HostJob* J : S->active) {
      if (J->stop_req && J->tracing && !J->stop_flagged) {
        if (cudaMemcpyAsync(S->d_cancel + J->slot, S->h_one, sizeof(unsigned), cudaMemcpyHostToDevice, S->s_main) !=
            cudaSuccess) {
          fail_all(S, GEON_ERR_CUDA);
          break;
        }
        J->stop_flagged = true;
        J->stop_epoch = S->epochs;
      }
    }
    if (S->fatal) break;
    if (!any_tracing(S)) {
      // sleep until a submission or a completion changes what can be admitted;
      // wake every millisecond while requests wait, for their deadlines
      const uint64_t g0 = S->gen;
      const auto pred = [S, g0] { return S->stop || S->fatal || S->gen != g0 || any_tracing(S); };
      if (S->waiting.empty()) S->cv_work.wait(lk, pred);
      else S->cv_work.wait_for(lk, std::chrono::milliseconds(1), pred);
      continue;
    }
    // 4. one serving launch: prologue, class kernels, counter copy-back
    write_claim_order(S);
    cudaGraphExec_t graph = S->graph;
    S->in_launch = true;
    lk.unlock();
    note_launches(1 + SERVE_CLASSES);
    cudaError_t e = cudaGraphLaunch(graph, S->s_main);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S->s_main);
    lk.lock();
    S->in_launch = false;
    S->cv_idle.notify_all();
    ++S->epochs;
    if (e != cudaSuccess) {
      fail_all(S, GEON_ERR_CUDA);
      break;
    }
    // 5. jobs whose rays are all finished (or that were stopped)
    for (size_t i = 0; i < S->active.size() && !S->fatal; ++i) {
      HostJob* J = S->active[i];
      if (!J->tracing) continue;
      if (J->stop_flagged) {
        if (S->epochs > J->stop_epoch) {  // a full launch since the flag: no lane holds the slot
          J->ray_steps += (double)S->h_counters[2 * SERVE_MAX_JOBS + J->slot];  // its finished rays
          J->tracing = false;
          hand_off(S, J);
        }
        continue;
      }
      const unsigned long long done = S->h_counters[SERVE_MAX_JOBS + J->slot];
      if ((int64_t)done < J->nrays) continue;
      J->ray_steps += (double)S->h_counters[2 * SERVE_MAX_JOBS + J->slot];
      if (J->spec.type == GEON_JOB_RENDER) {
        J->tracing = false;
        hand_off(S, J);
      } else if (bisect_round_done(S, J) != GEON_OK) {
        fail_all(S, GEON_ERR_CUDA);
      }
    }
  }
  S->cv_fin.notify_all();
  S->cv_done.notify_all();
}

// Completion thread: per-pixel reduction and copies to the caller's buffers,
// then the job's end is recorded and its memory returned to the arena.
void finish_loop(geon_server* S) {
  cudaSetDevice(S->dev);
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    S->cv_fin.wait(lk, [S] { return !S->finishing.empty() || S->stop || S->fatal; });
    if (S->finishing.empty()) {
      if (S->stop || S->fatal) break;
      continue;
    }
    HostJob* J = S->finishing.front();
    S->finishing.pop_front();
    if (J->state == ST_DONE) continue;
    int rc = J->stop_req;
    lk.unlock();
    const geon_job& q = J->spec;
    char* base = S->d_arena + J->off;
    cudaStream_t s = S->s_done;
    cudaError_t e = cudaSuccess;
    if (!rc && q.type == GEON_JOB_RENDER) {
      RenderBufs b;
      render_bufs(base, J->nsamp, J->npix, &b);
      e = cudaMemsetAsync(b.stats, 0, 8 * sizeof(unsigned long long), s);
      note_launches(1);
      if (e == cudaSuccess)
        e = launch_render_reduce(b.srgb, b.term, b.steps, b.resid, J->npix, J->spa, b.rgb, b.pcls, b.pst, b.stats, s,
                                 q.rgb8 ? b.rgb8 : nullptr);
      unsigned long long st[6] = {};
      if (e == cudaSuccess && q.rgb)
        e = cudaMemcpyAsync(q.rgb, b.rgb, sizeof(float) * 3 * J->npix, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess && q.rgb8)
        e = cudaMemcpyAsync(q.rgb8, b.rgb8, 3 * J->npix, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess && q.pixel_class)
        e = cudaMemcpyAsync(q.pixel_class, b.pcls, sizeof(int32_t) * J->npix, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess && q.pixel_steps)
        e = cudaMemcpyAsync(q.pixel_steps, b.pst, sizeof(int64_t) * J->npix, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(st, b.stats, sizeof st, cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e == cudaSuccess && q.render_stats) {
        q.render_stats->captured = (int64_t)st[0];
        q.render_stats->escaped = (int64_t)st[1];
        q.render_stats->diverged = (int64_t)st[2];
        std::memcpy(&q.render_stats->max_null_residual, &st[4], sizeof(double));
        q.render_stats->avg_steps = (double)(int64_t)st[3] / (double)J->npix;
        q.render_stats->total_steps = (int64_t)st[5];
      }
    } else if (!rc && q.type == GEON_JOB_BISECT) {
      *q.alpha_c = 0.5 * (J->lo + J->hi);
      if (q.lo_out) *q.lo_out = J->lo;
      if (q.hi_out) *q.hi_out = J->hi;
      if (q.steps_out) *q.steps_out = J->path_steps;
    } else if (q.type == GEON_JOB_CURVATURE) {
      e = cudaEventSynchronize(J->ev);  // also when stopped: the arena stays busy until the kernel ends
      const int64_t np = q.grid.n[0] * q.grid.n[1] * q.grid.n[2];
      CurvBufs b;
      curv_bufs(base, np, q.nk, q.einstein != nullptr, &b);
      if (!rc) {
        if (e == cudaSuccess && q.einstein)
          e = cudaMemcpyAsync(q.einstein, b.einstein, sizeof(double) * 16 * np, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && q.nk > 0)
          e = cudaMemcpyAsync(q.nec, b.nec, sizeof(double) * q.nk * np, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(S->h_flags + J->slot, b.flags, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e == cudaSuccess && (S->h_flags[J->slot] & 1)) rc = GEON_ERR_SINGULAR_METRIC;
        J->ray_steps = 0;
      }
    }
    if (e != cudaSuccess) rc = GEON_ERR_CUDA;
    lk.lock();
    if (J->state == ST_DONE) continue;  // the server failed meanwhile
    S->active.erase(std::remove(S->active.begin(), S->active.end(), J), S->active.end());
    finish(S, J, rc);
    if (rc == GEON_ERR_CUDA) fail_all(S, GEON_ERR_CUDA);
    S->cv_work.notify_all();  // arena space and a slot came free
  }
}

// Re-capture the launch graph with new per-class step budgets (lock held, no
// launch in flight).
int rebuild_graph(geon_server* S) {
  if (S->graph) cudaGraphExecDestroy(S->graph);
  S->graph = nullptr;
  return build_graph(S);
}

// Steps-per-launch candidates of the autotuner, per precision.
constexpr int TUNE_N = 5;
const int TUNE_STEPS[2][TUNE_N] = {{32, 64, 128, 256, 512}, {1024, 2048, 4096, 8192, 16384}};

double pct(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double k = p / 100.0 * (double)(v.size() - 1);
  const size_t i = (size_t)k;
  const double f = k - (double)i;
  return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

int validate(const geon_job* j) {
  if (j->type < GEON_JOB_RENDER || j->type > GEON_JOB_CURVATURE)
    return set_last_error(GEON_ERR_INVALID, "bad job type");
  if (j->metric_kind < GEON_MINKOWSKI || j->metric_kind > GEON_MORRIS_THORNE)
    return set_last_error(GEON_ERR_INVALID, "bad metric kind");
  if (j->nparams < 0 || j->nparams > 4) return set_last_error(GEON_ERR_INVALID, "bad metric parameter count");
  if (j->type != GEON_JOB_CURVATURE && j->precision != GEON_FP64 && j->precision != GEON_MIXED)
    return set_last_error(GEON_ERR_INVALID, "unknown precision");
  if (j->type == GEON_JOB_RENDER) {
    if (j->camera.width <= 0 || j->camera.height <= 0) return set_last_error(GEON_ERR_INVALID, "bad camera size");
    if (j->camera.forward_sign != 1 && j->camera.forward_sign != -1)
      return set_last_error(GEON_ERR_INVALID, "forward_sign must be +1 or -1");
    if (j->render.max_steps < 0) return set_last_error(GEON_ERR_INVALID, "max_steps < 0");
    if (!j->rgb && !j->rgb8) return set_last_error(GEON_ERR_INVALID, "null buffer");
  } else if (j->type == GEON_JOB_BISECT) {
    if (j->metric_kind != GEON_SCHWARZSCHILD)
      return set_last_error(GEON_ERR_INVALID, "shadow bisection needs a Schwarzschild metric");
    if (!j->alpha_c) return set_last_error(GEON_ERR_INVALID, "bad bisection arguments");
    if (j->max_steps < 0) return set_last_error(GEON_ERR_INVALID, "max_steps < 0");
  } else {
    if (j->grid.n[0] < 1 || j->grid.n[1] < 1 || j->grid.n[2] < 1) return set_last_error(GEON_ERR_INVALID, "bad grid");
    if (j->nk < 0 || (j->nk > 0 && !j->nec)) return set_last_error(GEON_ERR_INVALID, "nec output needed when nk > 0");
  }
  return GEON_OK;
}

}  // namespace

extern "C" {

int geon_server_create(size_t budget_bytes, geon_server_t* out) {
  if (!out || budget_bytes < 4096) return set_last_error(GEON_ERR_INVALID, "bad server budget");
  *out = nullptr;
  geon_server* S = new (std::nothrow) geon_server;
  if (!S) return set_last_error(GEON_ERR_OOM, "out of host memory");
  S->budget = budget_bytes;
  auto bad = [S](cudaError_t e, const char* what) {
    geon_server_destroy(S);
    return set_last_error(e == cudaErrorMemoryAllocation ? GEON_ERR_OOM : GEON_ERR_CUDA, what);
  };
  cudaError_t e = cudaGetDevice(&S->dev);
  if (e != cudaSuccess) return bad(e, "no CUDA device");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S->dev);
  if ((e = cudaMalloc(&S->d_arena, budget_bytes)) != cudaSuccess) return bad(e, "server arena");
  S->arena.init(budget_bytes);
  size_t resume_total = 0;
  unsigned long long caps[SERVE_CLASSES];
  for (int c = 0; c < SERVE_CLASSES; ++c) {
    const int kind = c / 2;
    const int per_sm = (c & 1) ? serve_mixed_blocks_per_sm(kind) : serve_fp64_blocks_per_sm(kind);
    S->blocks[c] = sms * per_sm;
    S->iters[c] = (c & 1) ? 4096 : 128;
    caps[c] = (unsigned long long)S->blocks[c] * TRACE_BLOCK;  // one parked ray per lane at most
    resume_total += 2 * caps[c];
  }
  if ((e = cudaMalloc(&S->d_jobs, sizeof(ServeJob) * SERVE_MAX_JOBS)) != cudaSuccess) return bad(e, "job table");
  if ((e = cudaMalloc(&S->d_cls, sizeof(ServeClass) * SERVE_CLASSES)) != cudaSuccess) return bad(e, "classes");
  if ((e = cudaMalloc(&S->d_counters, sizeof(unsigned long long) * 3 * SERVE_MAX_JOBS)) != cudaSuccess)
    return bad(e, "counters");
  if ((e = cudaMalloc(&S->d_cancel, sizeof(unsigned) * SERVE_MAX_JOBS)) != cudaSuccess) return bad(e, "flags");
  if ((e = cudaMallocHost(&S->h_counters, sizeof(unsigned long long) * 3 * SERVE_MAX_JOBS)) != cudaSuccess)
    return bad(e, "pinned counters");
  if ((e = cudaMallocHost(&S->h_flags, sizeof(int) * SERVE_MAX_JOBS)) != cudaSuccess) return bad(e, "pinned flags");
  if ((e = cudaMallocHost(&S->h_jobs, sizeof(ServeJob) * SERVE_MAX_JOBS)) != cudaSuccess)
    return bad(e, "pinned job table");
  if ((e = cudaMallocHost(&S->h_order, sizeof(int) * SERVE_RING * SERVE_CLASSES)) != cudaSuccess)
    return bad(e, "pinned claim order");
  if ((e = cudaMallocHost(&S->h_tail_head, sizeof(unsigned) * 2 * SERVE_CLASSES)) != cudaSuccess)
    return bad(e, "pinned claim order length");
  if ((e = cudaMallocHost(&S->h_one, sizeof(unsigned))) != cudaSuccess) return bad(e, "pinned flag");
  if ((e = cudaMalloc(&S->d_rings, sizeof(int) * SERVE_RING * SERVE_CLASSES)) != cudaSuccess) return bad(e, "rings");
  if ((e = cudaMalloc(&S->d_resume, sizeof(ResumeEntry) * resume_total)) != cudaSuccess)
    return bad(e, "resume pools");
  if ((e = cudaMalloc(&S->d_epoch, sizeof(unsigned))) != cudaSuccess) return bad(e, "epoch");
  *S->h_one = 1u;
  std::memset(S->h_order, 0, sizeof(int) * SERVE_RING * SERVE_CLASSES);
  std::memset(S->h_tail_head, 0, sizeof(unsigned) * 2 * SERVE_CLASSES);
  std::memset(S->h_counters, 0, sizeof(unsigned long long) * 3 * SERVE_MAX_JOBS);
  std::memset(S->h_flags, 0, sizeof(int) * SERVE_MAX_JOBS);
  cudaMemset(S->d_counters, 0, sizeof(unsigned long long) * 3 * SERVE_MAX_JOBS);
  cudaMemset(S->d_cancel, 0, sizeof(unsigned) * SERVE_MAX_JOBS);
  cudaMemset(S->d_epoch, 0, sizeof(unsigned));
  std::vector<ServeClass> hc(SERVE_CLASSES);
  std::memset(hc.data(), 0, sizeof(ServeClass) * SERVE_CLASSES);
  ResumeEntry* r = S->d_resume;
  for (int c = 0; c < SERVE_CLASSES; ++c) {
    hc[c].resume_cap = caps[c];
    hc[c].resume[0] = r;
    r += caps[c];
    hc[c].resume[1] = r;
    r += caps[c];
    hc[c].ring = S->d_rings + (size_t)c * SERVE_RING;
  }
  cudaMemcpy(S->d_cls, hc.data(), sizeof(ServeClass) * SERVE_CLASSES, cudaMemcpyHostToDevice);
  cudaStreamCreateWithFlags(&S->s_main, cudaStreamNonBlocking);
  cudaStreamCreateWithFlags(&S->s_walk, cudaStreamNonBlocking);
  // Curvature grid kernels run on s_side at the highest stream priority: the
  // persistent ray kernels hold every SM for one launch (a few ms), and when
  // they end the block scheduler takes the waiting curvature blocks first, so a
  // curvature request runs at nearly the full GPU's rate between two launches
  // instead of trickling into the slots the ray kernels leave.
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  cudaStreamCreateWithPriority(&S->s_side, cudaStreamNonBlocking, prio_greatest);
  cudaStreamCreateWithFlags(&S->s_done, cudaStreamNonBlocking);
  for (int c = 0; c < SERVE_CLASSES; ++c) {
    cudaStreamCreateWithFlags(&S->s_cls[c], cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&S->ev_join[c], cudaEventDisableTiming);
  }
  cudaEventCreateWithFlags(&S->ev_fork, cudaEventDisableTiming);
  for (int i = SERVE_MAX_JOBS - 1; i >= 0; --i) S->free_slots.push_back(i);
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return bad(e, "server set-up");
  if (build_graph(S) != GEON_OK) return bad(cudaGetLastError(), "capturing the serving launch graph");
  S->th = std::thread(server_loop, S);
  S->th_fin = std::thread(finish_loop, S);
  *out = S;
  return GEON_OK;
}

int geon_server_submit(geon_server_t S, const geon_job* job, uint64_t* id) {
  if (!S || !job) return set_last_error(GEON_ERR_INVALID, "null server or job");
  if (int rc = validate(job)) return rc;
  HostJob* J = new (std::nothrow) HostJob;
  if (!J) return set_last_error(GEON_ERR_OOM, "out of host memory");
  J->spec = *job;
  if (job->type == GEON_JOB_RENDER) {
    J->spa = job->render.samples_per_axis < 1 ? 1 : job->render.samples_per_axis;
    J->npix = job->camera.width * job->camera.height;
    J->nsamp = J->npix * J->spa * J->spa;
    J->bytes = render_bufs(nullptr, J->nsamp, J->npix, nullptr);
  } else if (job->type == GEON_JOB_BISECT) {
    J->levels = bisect_levels_of(*job);
    J->bytes = bisect_bufs(nullptr, J->levels, nullptr);
  } else {
    const int64_t np = job->grid.n[0] * job->grid.n[1] * job->grid.n[2];
    J->bytes = curv_bufs(nullptr, np, job->nk, job->einstein != nullptr, nullptr);
  }
  if (J->bytes > S->budget) {
    delete J;
    return set_last_error(GEON_ERR_ADMISSION, "request larger than the server's memory budget");
  }
  {
    std::lock_guard<std::mutex> g(S->mu);
    if (S->fatal || S->stop) {
      const int code = S->fatal ? S->fatal : GEON_ERR_CANCELLED;
      delete J;
      return set_last_error(code, "server is stopping");
    }
    J->id = S->next_id++;
    J->t_submit = now_s();
    if (job->deadline_s > 0) J->deadline = J->t_submit + job->deadline_s;
    if (S->t_first < 0) S->t_first = J->t_submit;
    S->jobs[J->id] = J;
    S->waiting.push_back(J);
    ++S->submitted;
    ++S->gen;
    if (id) *id = J->id;
  }
  S->cv_work.notify_all();
  return GEON_OK;
}

int geon_server_poll(geon_server_t S, uint64_t id) {
  if (!S) return set_last_error(GEON_ERR_INVALID, "null server");
  std::lock_guard<std::mutex> g(S->mu);
  auto it = S->jobs.find(id);
  if (it == S->jobs.end()) return set_last_error(GEON_ERR_NOT_FOUND, "unknown job id");
  const HostJob* J = it->second;
  if (J->state == ST_DONE && J->error) return J->error;
  return J->state;
}

int geon_server_wait(geon_server_t S, uint64_t id, double timeout_s) {
  if (!S) return set_last_error(GEON_ERR_INVALID, "null server");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->jobs.find(id);
  if (it == S->jobs.end()) return set_last_error(GEON_ERR_NOT_FOUND, "unknown job id");
  HostJob* J = it->second;
  const auto pred = [J] { return J->state == ST_DONE; };
  if (timeout_s < 0) {
    S->cv_done.wait(lk, pred);
  } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
    return set_last_error(GEON_ERR_TIMEOUT, "job not finished before the deadline");
  }
  return J->error;
}

int geon_server_wait_all(geon_server_t S, double timeout_s) {
  if (!S) return set_last_error(GEON_ERR_INVALID, "null server");
  std::unique_lock<std::mutex> lk(S->mu);
  const auto pred = [S] { return S->waiting.empty() && S->active.empty(); };
  if (timeout_s < 0) {
    S->cv_done.wait(lk, pred);
  } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
    return set_last_error(GEON_ERR_TIMEOUT, "jobs still running at the deadline");
  }
  return S->fatal;
}

int geon_server_cancel(geon_server_t S, uint64_t id) {
  if (!S) return set_last_error(GEON_ERR_INVALID, "null server");
  std::lock_guard<std::mutex> g(S->mu);
  auto it = S->jobs.find(id);
  if (it == S->jobs.end()) return set_last_error(GEON_ERR_NOT_FOUND, "unknown job id");
  HostJob* J = it->second;
  if (J->state == ST_QUEUED) {
    S->waiting.erase(std::remove(S->waiting.begin(), S->waiting.end(), J), S->waiting.end());
    finish(S, J, GEON_ERR_CANCELLED);
  } else if (J->state == ST_RUNNING && !J->stop_req) {
    J->stop_req = GEON_ERR_CANCELLED;
    S->cv_work.notify_all();
  }
  return GEON_OK;
}

int geon_server_set_steps_per_launch(geon_server_t S, int precision, int steps) {
  if (!S) return set_last_error(GEON_ERR_INVALID, "null server");
  if (precision != GEON_FP64 && precision != GEON_MIXED) return set_last_error(GEON_ERR_INVALID, "unknown precision");
  if (steps < 1 || steps > (1 << 24)) return set_last_error(GEON_ERR_INVALID, "steps per launch out of range");
  std::unique_lock<std::mutex> lk(S->mu);
  if (S->fatal) return set_last_error(S->fatal, "server stopped after a CUDA error");
  S->cv_idle.wait(lk, [S] { return !S->in_launch; });
  for (int c = 0; c < SERVE_CLASSES; ++c)
    if ((c & 1) == (precision == GEON_MIXED ? 1 : 0)) S->iters[c] = steps;
  if (rebuild_graph(S) != GEON_OK) {
    fail_all(S, GEON_ERR_CUDA);
    return set_last_error(GEON_ERR_CUDA, "re-capturing the serving launch graph");
  }
  return GEON_OK;
}

int geon_server_get_steps_per_launch(geon_server_t S, int precision) {
  if (!S || (precision != GEON_FP64 && precision != GEON_MIXED)) return GEON_ERR_INVALID;
  std::lock_guard<std::mutex> g(S->mu);
  return S->iters[precision == GEON_MIXED ? 1 : 0];
}

int geon_server_autotune(geon_server_t S, double* rates_out, int* best_out) {
  if (!S) return set_last_error(GEON_ERR_INVALID, "null server");
  double rates[2][TUNE_N] = {};
  int best[2] = {0, 0};
  for (int pi = 0; pi < 2; ++pi) {
    const int precision = pi == 0 ? GEON_FP64 : GEON_MIXED;
    // calibration: a Schwarzschild render at the reference CUDA program's settings
    // (r_obs 30, fov 60, h 0.05, cap 20000, escape 1000M), sized so every lane of
    // the class's grid is busy for several launches
    geon_job q;
    std::memset(&q, 0, sizeof q);
    q.type = GEON_JOB_RENDER;
    q.metric_kind = GEON_SCHWARZSCHILD;
    q.metric_params[0] = 1.0;
    q.metric_params[1] = 1.001;
    q.metric_params[2] = 1000.0;
    q.nparams = 3;
    q.precision = precision;
    q.camera.observer[1] = 30.0;
    q.camera.observer[2] = 1.5707963267948966;
    q.camera.fov_y_deg = 60.0;
    q.camera.width = pi == 0 ? 320 : 512;
    q.camera.height = pi == 0 ? 320 : 512;
    q.camera.forward_sign = 1;
    geon_render_config_default(&q.render);
    q.render.show_stars = 0;
    std::vector<float> rgb((size_t)q.camera.width * q.camera.height * 3);
    geon_render_stats st;
    q.rgb = rgb.data();
    q.render_stats = &st;
    double best_rate = 0.0;
    for (int k = 0; k < TUNE_N; ++k) {
      if (int rc = geon_server_set_steps_per_launch(S, precision, TUNE_STEPS[pi][k])) return rc;
      uint64_t id = 0;
      const double t0 = now_s();
      if (int rc = geon_server_submit(S, &q, &id)) return rc;
      if (int rc = geon_server_wait(S, id, -1.0)) return rc;
      const double dt = now_s() - t0;
      rates[pi][k] = dt > 0.0 ? (double)st.total_steps / dt : 0.0;
      if (rates[pi][k] > best_rate) best_rate = rates[pi][k];
    }
    // the fewest steps per launch (finest admission and completion granularity)
    // within 2 % of the best rate
    for (int k = 0; k < TUNE_N; ++k)
      if (rates[pi][k] >= 0.98 * best_rate) {
        best[pi] = TUNE_STEPS[pi][k];
        break;
      }
    if (int rc = geon_server_set_steps_per_launch(S, precision, best[pi])) return rc;
  }
  if (rates_out) std::memcpy(rates_out, rates, sizeof rates);
  if (best_out) {
    best_out[0] = best[0];
    best_out[1] = best[1];
  }
  return GEON_OK;
}

int geon_server_stats_get(geon_server_t S, geon_server_stats* out) {
  if (!S || !out) return set_last_error(GEON_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> g(S->mu);
  std::memset(out, 0, sizeof *out);
  std::vector<double> all;
  for (int t = 0; t < 3; ++t) {
    all.insert(all.end(), S->lat[t].begin(), S->lat[t].end());
    out->p50_ms_by_type[t] = pct(S->lat[t], 50);
    out->p99_ms_by_type[t] = pct(S->lat[t], 99);
    out->completed_by_type[t] = (int64_t)S->lat[t].size();
  }
  out->submitted = S->submitted;
  out->completed = S->completed;
  out->failed = S->failed;
  out->queued = (int64_t)S->waiting.size();
  out->running = (int64_t)S->active.size();
  out->p50_ms = pct(all, 50);
  out->p99_ms = pct(all, 99);
  double sum = 0;
  for (double x : all) sum += x;
  out->mean_ms = all.empty() ? 0.0 : sum / (double)all.size();
  out->ray_steps = S->ray_steps;
  out->ray_steps_unfinished = S->ray_steps_unfinished;
  out->grid_points = S->grid_points;
  out->wall_s = S->t_first < 0 ? 0.0 : (S->t_last - S->t_first);
  out->epochs = S->epochs;
  return GEON_OK;
}

int geon_server_destroy(geon_server_t S) {
  if (!S) return GEON_OK;
  if (S->th.joinable()) {
    std::unique_lock<std::mutex> lk(S->mu);
    for (HostJob* J : S->waiting) finish(S, J, GEON_ERR_CANCELLED);
    S->waiting.clear();
    for (HostJob* J : S->active)
      if (!J->stop_req) J->stop_req = GEON_ERR_CANCELLED;
    S->cv_work.notify_all();
    // jobs in flight stop within two launches; then both threads end
    S->cv_done.wait_for(lk, std::chrono::seconds(60), [S] { return S->active.empty() || S->fatal; });
    S->stop = true;
  }
  S->cv_work.notify_all();
  S->cv_fin.notify_all();
  if (S->th.joinable()) S->th.join();
  if (S->th_fin.joinable()) S->th_fin.join();
  if (S->s_main) cudaStreamSynchronize(S->s_main);
  if (S->s_side) cudaStreamSynchronize(S->s_side);
  if (S->s_done) cudaStreamSynchronize(S->s_done);
  for (auto& kv : S->jobs) {
    HostJob* J = kv.second;
    if (J->ev) cudaEventDestroy(J->ev);
    if (J->metric) geon_metric_destroy(J->metric);
    delete J;
  }
  if (S->graph) cudaGraphExecDestroy(S->graph);
  for (int c = 0; c < SERVE_CLASSES; ++c) {
    if (S->s_cls[c]) cudaStreamDestroy(S->s_cls[c]);
    if (S->ev_join[c]) cudaEventDestroy(S->ev_join[c]);
  }
  if (S->ev_fork) cudaEventDestroy(S->ev_fork);
  for (cudaStream_t s : {S->s_main, S->s_walk, S->s_side, S->s_done})
    if (s) cudaStreamDestroy(s);
  cudaFree(S->d_arena);
  cudaFree(S->d_jobs);
  cudaFree(S->d_cls);
  cudaFree(S->d_counters);
  cudaFree(S->d_cancel);
  for (void* p : {(void*)S->h_counters, (void*)S->h_flags, (void*)S->h_jobs, (void*)S->h_order,
                  (void*)S->h_tail_head, (void*)S->h_one})
    if (p) cudaFreeHost(p);
  cudaFree(S->d_rings);
  cudaFree(S->d_resume);
  cudaFree(S->d_epoch);
  delete S;
  return GEON_OK;
}

}  // extern "C"
