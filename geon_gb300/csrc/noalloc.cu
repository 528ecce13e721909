// Shadow bisection that allocates nothing: geon_shadow_bisect_dev_noalloc.
//
// geon_shadow_bisect_dev needs working memory of its own on the GPU: the
// brackets being narrowed, the tree of launch angles traced each round, their
// results and the ray queue. It takes that memory from the stream-ordered
// allocator on every call. Some callers cannot let a library allocate device
// memory while they run: a host that reserves the whole GPU up front and hands
// out memory only through its own pool, a real-time loop whose latency budget
// has no room for an allocator call, or a program that must never fail with
// "out of memory" halfway through a frame. For them this entry point keeps its
// working memory in one fixed array compiled into the library instead.
//
// The array (NOALLOC_SCRATCH_BYTES, 512 KiB) is a __device__ variable: once it
// is placed on a GPU it stays there until the process exits. It bounds the
// work: at most NOALLOC_MAX_BRACKETS (4096) brackets per call; larger requests
// are refused with GEON_ERR_INVALID. The speculative width of the bisection
// rounds is always the default one (geon_set_bisect_rays_per_round does not
// apply here): the array is sized for it.
//
// Host code cannot use the array's name as a device address (on the host it
// names a stand-in object), so every call, with the caller's device current,
// asks the runtime for the array's device address with cudaGetSymbolAddress,
// checks the result and hands that address to the kernels. The lookup is not
// cached: a cached address would go stale when the context it came from is
// destroyed (cudaDeviceReset) and another one takes its place. Under CUDA's
// lazy module loading the array is only placed on a device when this lookup
// first runs there, and the kernels' code when they first launch there, so the
// first call on a device is the one that takes device memory (the array's
// 512 KiB and the code): make it before the caller reserves the rest of the
// device's memory for its own pool, and before capturing any stream into a
// CUDA graph. Later calls find both loaded and take nothing.
//
// All calls share the one array and each leaves its contents behind; the entry
// point clears what must start at zero. Two calls whose work overlaps on the
// GPU (on different streams, or from different host threads) race on the array
// and corrupt each other's results: order them on one stream.
#include <cuda_runtime.h>

#include <cstring>

#include "internal.h"

namespace geon {

constexpr size_t NOALLOC_SCRATCH_BYTES = 512 * 1024;
constexpr size_t NOALLOC_MAX_BRACKETS = 4096;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

namespace {

// Device address of the scratch array in the current context (looked up on
// every call; the first lookup on a device loads the array there).
int noalloc_scratch(unsigned char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return set_last_error(GEON_ERR_CUDA, e != cudaSuccess ? cudaGetErrorString(e) : "null scratch address");
  *out = static_cast<unsigned char*>(p);
  return GEON_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace geon

using namespace geon;

extern "C" int geon_shadow_bisect_dev_noalloc(geon_metric_t m, double r_obs, const double* lo, const double* hi,
                                              size_t nb, int iters, double step, int64_t max_steps,
                                              int precision, double* alpha_c, double* lo_out,
                                              double* hi_out, int64_t* steps_out, void* stream) {
  const MetricDesc* d = metric_desc(m);
  if (!d) return set_last_error(GEON_ERR_INVALID, "null metric handle");
  if (d->kind != GEON_SCHWARZSCHILD) return set_last_error(GEON_ERR_INVALID, "shadow bisection needs a Schwarzschild metric");
  if (precision != GEON_FP64 && precision != GEON_MIXED && precision != GEON_ADAPTIVE &&
      precision != GEON_FP64_FAST)
    return set_last_error(GEON_ERR_INVALID, "unknown precision");
  if (nb == 0) return GEON_OK;
  if (nb > NOALLOC_MAX_BRACKETS)
    return set_last_error(GEON_ERR_INVALID,
                          "geon_shadow_bisect_dev_noalloc takes at most 4096 brackets per call (fixed 512 KiB scratch)");
  if (!lo || !hi || !alpha_c || iters < 0 || max_steps < 0)
    return set_last_error(GEON_ERR_INVALID, "bad bisection arguments");

  // Layout of the scratch: queue+flags | lo | hi | path steps | tree angles | tree terms | tree steps
  const int Lmax = bisect_levels_for(nb);
  const size_t cap = nb * (((size_t)1 << Lmax) - 1);
  const size_t off_work = 256;
  const size_t off_tree = align256(off_work + nb * (2 * sizeof(double) + sizeof(int64_t)));
  const size_t off_term = align256(off_tree + cap * sizeof(double));
  const size_t off_steps = align256(off_term + cap * sizeof(int32_t));
  const size_t total = off_steps + cap * sizeof(int64_t);
  if (total > NOALLOC_SCRATCH_BYTES)
    return set_last_error(GEON_ERR_INVALID, "bisection working set exceeds the fixed 512 KiB scratch");

  unsigned char* base = nullptr;
  if (int rc = noalloc_scratch(&base)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned long long* queue = reinterpret_cast<unsigned long long*>(base);
  double* wlo = reinterpret_cast<double*>(base + off_work);
  double* whi = wlo + nb;
  int64_t* wst = reinterpret_cast<int64_t*>(whi + nb);
  double* tree = reinterpret_cast<double*>(base + off_tree);
  int32_t* tterm = reinterpret_cast<int32_t*>(base + off_term);
  int64_t* tsteps = reinterpret_cast<int64_t*>(base + off_steps);

  cudaError_t e;
#define NOALLOC_CUDA(call)                                                            \
  do {                                                                                \
    e = (call);                                                                       \
    if (e != cudaSuccess) return set_last_error(GEON_ERR_CUDA, cudaGetErrorString(e)); \
  } while (0)
  NOALLOC_CUDA(cudaMemcpyAsync(wlo, lo, sizeof(double) * nb, cudaMemcpyDefault, s));
  NOALLOC_CUDA(cudaMemcpyAsync(whi, hi, sizeof(double) * nb, cudaMemcpyDefault, s));
  NOALLOC_CUDA(cudaMemsetAsync(wst, 0, sizeof(int64_t) * nb, s));
  int remaining = iters;
  while (remaining > 0) {
    const int L = remaining < Lmax ? remaining : Lmax;
    const int64_t per = ((int64_t)1 << L) - 1;
    NOALLOC_CUDA(launch_bisect_build((int64_t)nb, per, wlo, whi, tree, s));
    NOALLOC_CUDA(cudaMemsetAsync(queue, 0, 2 * sizeof(unsigned long long), s));  // queue and flags start at 0
    TraceLaunch T = trace_launch_defaults(m, step, max_steps);
    T.n = (int64_t)nb * per;
    T.alpha = tree;
    T.r_obs = r_obs;
    T.term = tterm;
    T.steps = tsteps;
    T.queue = queue;
    T.flags = reinterpret_cast<int*>(queue + 1);
    T.decide = 1;  // as geon_shadow_bisect_dev: only each ray's class matters
    NOALLOC_CUDA(launch_trace_any(T, precision, SRC_EQUATORIAL, SINK_SHADOW, s));
    NOALLOC_CUDA(launch_bisect_walk((int64_t)nb, per, L, tree, tterm, tsteps, wlo, whi, wst, s));
    note_launches(3);
    remaining -= L;
  }
  NOALLOC_CUDA(launch_bisect_finish((int64_t)nb, wlo, whi, alpha_c, s));
  note_launches(1);
  if (lo_out) NOALLOC_CUDA(cudaMemcpyAsync(lo_out, wlo, sizeof(double) * nb, cudaMemcpyDefault, s));
  if (hi_out) NOALLOC_CUDA(cudaMemcpyAsync(hi_out, whi, sizeof(double) * nb, cudaMemcpyDefault, s));
  if (steps_out) NOALLOC_CUDA(cudaMemcpyAsync(steps_out, wst, sizeof(int64_t) * nb, cudaMemcpyDefault, s));
#undef NOALLOC_CUDA
  return GEON_OK;
}
