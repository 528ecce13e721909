// FP64 parity path: the persistent ray-tracing kernel (loop in
// trace_common.cuh) with the reference's FP64 RK4 step, plus render reduction,
// point-wise functors, tetrad, camera/equatorial ray generation and sky kernels.
//
// Compiled with --fmad=false: every FP64 result must match the CPU oracle.
#include <cuda_runtime.h>

#include "internal.h"
#include "metric_fp64.cuh"
#include "serve_common.cuh"
#include "trace_common.cuh"

namespace geon {

// ---------------------------------------------------------------------------
// FP64 stepper: the reference's arithmetic, bit for bit.
// ---------------------------------------------------------------------------
template <int K>
struct Fp64Stepper {
  double y[8];
  bool singular = false;
  __device__ __forceinline__ void load(const TraceLaunch&, const double y0[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = y0[i];
  }
  __device__ __forceinline__ void to_double(double out[8]) const {
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = y[i];
  }
  __device__ __forceinline__ int terminate(const TraceLaunch& L) const { return metric_terminate<K>(L.M, y); }
  __device__ __forceinline__ int step(const TraceLaunch& L) {
    double yn[8];
    singular |= !rk4_step<K>(L.M, y, L.step, L.half_step, L.sixth, yn);
    bool finite = true;
#pragma unroll
    for (int i = 0; i < 8; ++i) finite &= isfinite(yn[i]);
    if (!finite) return STEP_NONFINITE;
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = yn[i];
    return STEP_OK;
  }
  __device__ __forceinline__ void group_end(const TraceLaunch&) {}
  __device__ __forceinline__ void check_null(const TraceLaunch&, const double*) {}
  __device__ __forceinline__ void finish(const TraceLaunch& L) {
    if (singular) atomicOr(L.flags, 1);
  }
  // Serving: a lane's ray state as 16 words, and its restoration.
  __device__ __forceinline__ void save(uint32_t w[16]) const {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(y[i]);
      w[2 * i] = (uint32_t)b;
      w[2 * i + 1] = (uint32_t)(b >> 32);
    }
  }
  __device__ __forceinline__ void restore(const TraceLaunch&, const uint32_t w[16], int64_t) {
#pragma unroll
    for (int i = 0; i < 8; ++i)
      y[i] = __longlong_as_double((long long)(((unsigned long long)w[2 * i + 1] << 32) | w[2 * i]));
  }
  __device__ __forceinline__ void rebind(const TraceLaunch&) {}
  __device__ __forceinline__ void set_source(int) {}
  __device__ __forceinline__ void resume_frame(const TraceLaunch&, int64_t) {}
};

// The FP64 stepper of a launch whose rays have different metric kinds (one
// persistent kernel over several renders): the kind is the lane's current
// ray's, and every call branches on it.
struct Fp64StepperAny {
  double y[8];
  int kind = KIND_MINKOWSKI;
  bool singular = false;
  __device__ __forceinline__ void bind(const TraceLaunch& L, int) { kind = L.M.kind; }
  __device__ __forceinline__ void load(const TraceLaunch&, const double y0[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = y0[i];
  }
  __device__ __forceinline__ void to_double(double out[8]) const {
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = y[i];
  }
  __device__ __forceinline__ int terminate(const TraceLaunch& L) const {
    switch (kind) {
      case KIND_SCHWARZSCHILD: return metric_terminate<KIND_SCHWARZSCHILD>(L.M, y);
      case KIND_ALCUBIERRE: return metric_terminate<KIND_ALCUBIERRE>(L.M, y);
      case KIND_MORRIS_THORNE: return metric_terminate<KIND_MORRIS_THORNE>(L.M, y);
      default: return metric_terminate<KIND_MINKOWSKI>(L.M, y);
    }
  }
  __device__ __forceinline__ int step(const TraceLaunch& L) {
    double yn[8];
    bool ok;
    switch (kind) {
      case KIND_SCHWARZSCHILD: ok = rk4_step<KIND_SCHWARZSCHILD>(L.M, y, L.step, L.half_step, L.sixth, yn); break;
      case KIND_ALCUBIERRE: ok = rk4_step<KIND_ALCUBIERRE>(L.M, y, L.step, L.half_step, L.sixth, yn); break;
      case KIND_MORRIS_THORNE: ok = rk4_step<KIND_MORRIS_THORNE>(L.M, y, L.step, L.half_step, L.sixth, yn); break;
      default: ok = rk4_step<KIND_MINKOWSKI>(L.M, y, L.step, L.half_step, L.sixth, yn); break;
    }
    singular |= !ok;
    bool finite = true;
#pragma unroll
    for (int i = 0; i < 8; ++i) finite &= isfinite(yn[i]);
    if (!finite) return STEP_NONFINITE;
#pragma unroll
    for (int i = 0; i < 8; ++i) y[i] = yn[i];
    return STEP_OK;
  }
  __device__ __forceinline__ void group_end(const TraceLaunch&) {}
  __device__ __forceinline__ void check_null(const TraceLaunch&, const double*) {}
  __device__ __forceinline__ void finish(const TraceLaunch& L) {
    if (singular) atomicOr(L.flags, 1);
  }
};

__global__ void __launch_bounds__(TRACE_BLOCK) trace_multi_fp64_kernel(const TraceLaunch* jobs, const MultiDesc D) {
  trace_loop_multi<Fp64StepperAny, SRC_CAMERA, SINK_RENDER>(jobs, D);
}

cudaError_t launch_trace_multi_fp64(const TraceLaunch* jobs, const MultiDesc& D, float reserve, cudaStream_t s) {
  static int sms = 0, per_sm = 0;
  if (sms == 0) {
    int dev = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, trace_multi_fp64_kernel, TRACE_BLOCK, 0);
    per_sm = occ < 1 ? 1 : occ;
  }
  const int64_t n = D.start[D.njobs];
  if (n <= 0) return cudaSuccess;
  const int64_t slots = persistent_slots(sms, per_sm, reserve);
  const int64_t need = (n + TRACE_BLOCK - 1) / TRACE_BLOCK;
  const int grid = (int)(need < slots ? need : slots);
  trace_multi_fp64_kernel<<<grid < 1 ? 1 : grid, TRACE_BLOCK, 0, s>>>(jobs, D);
  return cudaGetLastError();
}

template <int K, int SRC, int SINK>
__global__ void __launch_bounds__(TRACE_BLOCK) trace_fp64_kernel(const TraceLaunch L) {
  trace_loop<Fp64Stepper<K>, K, SRC, SINK>(L);
}

// Serving engine kernel for the FP64 classes (serve_common.cuh).
template <int K>
__global__ void __launch_bounds__(TRACE_BLOCK) serve_fp64_kernel(const ServeJob* jobs, ServeCounters cnt,
                                                                  ServeClass* cl, const unsigned* epoch, int budget) {
  serve_loop<Fp64Stepper<K>, K>(jobs, cnt, cl, epoch, budget);
}

template <int K>
static cudaError_t launch_serve_fp64_k(const ServeJob* jobs, ServeCounters cnt, ServeClass* cl, const unsigned* epoch,
                                       int budget, int blocks, cudaStream_t s) {
  serve_fp64_kernel<K><<<blocks, TRACE_BLOCK, 0, s>>>(jobs, cnt, cl, epoch, budget);
  return cudaGetLastError();
}

int serve_fp64_blocks_per_sm(int kind) {
  int occ = 0;
  switch (kind) {
    case KIND_MINKOWSKI: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_fp64_kernel<KIND_MINKOWSKI>, TRACE_BLOCK, 0); break;
    case KIND_SCHWARZSCHILD: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_fp64_kernel<KIND_SCHWARZSCHILD>, TRACE_BLOCK, 0); break;
    case KIND_ALCUBIERRE: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_fp64_kernel<KIND_ALCUBIERRE>, TRACE_BLOCK, 0); break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_fp64_kernel<KIND_MORRIS_THORNE>, TRACE_BLOCK, 0); break;
  }
  return occ < 1 ? 1 : occ;
}

cudaError_t launch_serve_fp64(int kind, const ServeJob* jobs, ServeCounters cnt, ServeClass* cl,
                              const unsigned* epoch, int budget, int blocks, cudaStream_t s) {
  switch (kind) {
    case KIND_MINKOWSKI: return launch_serve_fp64_k<KIND_MINKOWSKI>(jobs, cnt, cl, epoch, budget, blocks, s);
    case KIND_SCHWARZSCHILD: return launch_serve_fp64_k<KIND_SCHWARZSCHILD>(jobs, cnt, cl, epoch, budget, blocks, s);
    case KIND_ALCUBIERRE: return launch_serve_fp64_k<KIND_ALCUBIERRE>(jobs, cnt, cl, epoch, budget, blocks, s);
    case KIND_MORRIS_THORNE: return launch_serve_fp64_k<KIND_MORRIS_THORNE>(jobs, cnt, cl, epoch, budget, blocks, s);
  }
  return cudaErrorInvalidValue;
}

// Before each serving launch: advance the epoch, empty the output resume buffer
// of every class and reset the resume claim counters.
__global__ void serve_prologue_kernel(ServeClass* cls, int nclasses, unsigned* epoch) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const unsigned e = *epoch + 1u;
  const int pout = (int)(e & 1u) ^ 1;
  for (int c = 0; c < nclasses; ++c) {
    cls[c].resume_count[pout] = 0;
    cls[c].resume_claim = 0;
  }
  *epoch = e;
}

cudaError_t launch_serve_prologue(ServeClass* cls, int nclasses, unsigned* epoch, cudaStream_t s) {
  serve_prologue_kernel<<<1, 32, 0, s>>>(cls, nclasses, epoch);
  return cudaGetLastError();
}

template <int K, int SRC, int SINK>
static cudaError_t launch_kst(const TraceLaunch& L, cudaStream_t s) {
  static int sms = 0, per_sm = 0;
  if (sms == 0) {
    int dev = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, trace_fp64_kernel<K, SRC, SINK>, TRACE_BLOCK, 0);
    per_sm = occ < 1 ? 1 : occ;
  }
  // persistent grid: every resident slot, minus the blocks per SM the caller
  // keeps free for a concurrent job
  const int64_t slots = persistent_slots(sms, per_sm, L.reserve_per_sm);
  const int64_t need = (L.n + TRACE_BLOCK - 1) / TRACE_BLOCK;
  int grid = (int)(need < slots ? need : slots);
  if (grid < 1) grid = 1;
  trace_fp64_kernel<K, SRC, SINK><<<grid, TRACE_BLOCK, 0, s>>>(L);
  return cudaGetLastError();
}

template <int K>
static cudaError_t launch_k(const TraceLaunch& L, int src, int sink, cudaStream_t s) {
  if (src == SRC_ARRAY && sink == SINK_TRACE) return launch_kst<K, SRC_ARRAY, SINK_TRACE>(L, s);
  if (src == SRC_CAMERA && sink == SINK_RENDER) return launch_kst<K, SRC_CAMERA, SINK_RENDER>(L, s);
  if (src == SRC_CAMERA && sink == SINK_TRACE) return launch_kst<K, SRC_CAMERA, SINK_TRACE>(L, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_trace_fp64(const TraceLaunch& L, int src, int sink, cudaStream_t s) {
  if (L.n <= 0) return cudaSuccess;
  if (src == SRC_EQUATORIAL) {
    if (L.M.kind != KIND_SCHWARZSCHILD) return cudaErrorInvalidValue;
    if (sink == SINK_SHADOW) return launch_kst<KIND_SCHWARZSCHILD, SRC_EQUATORIAL, SINK_SHADOW>(L, s);
    if (sink == SINK_TRACE) return launch_kst<KIND_SCHWARZSCHILD, SRC_EQUATORIAL, SINK_TRACE>(L, s);
    return cudaErrorInvalidValue;
  }
  switch (L.M.kind) {
    case KIND_MINKOWSKI: return launch_k<KIND_MINKOWSKI>(L, src, sink, s);
    case KIND_SCHWARZSCHILD: return launch_k<KIND_SCHWARZSCHILD>(L, src, sink, s);
    case KIND_ALCUBIERRE: return launch_k<KIND_ALCUBIERRE>(L, src, sink, s);
    case KIND_MORRIS_THORNE: return launch_k<KIND_MORRIS_THORNE>(L, src, sink, s);
    case KIND_FIELD: return launch_k<KIND_FIELD>(L, src, sink, s);
  }
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// Per-pixel reduction of sub-samples (render.rs:77-136) and image statistics
// (render.rs:146-164). Sub-samples are summed in the reference's (sj, si) order.
// stats: [captured, escaped, diverged, sum of per-pixel step averages,
//         max residual bits, sum of all sample steps]
// ---------------------------------------------------------------------------
// write_png's tonemap (render.rs:174-178): clamp to [0, 1] (NaN passes
// through, as f32::clamp does), raise to the f32 power 1/2.2, scale by 255,
// round half away from zero and cast with saturation (NaN -> 0). The power is
// evaluated in FP64 and rounded once to f32; over every f32 in [0, 1] this
// gives the same byte as glibc's powf (checked exhaustively on the host).
__device__ __forceinline__ uint8_t tonemap_u8(float c) {
  float v = c;
  if (v < 0.0f) v = 0.0f;
  if (v > 1.0f) v = 1.0f;
  const float gamma_inv = 1.0f / 2.2f;
  const float p = __double2float_rn(pow((double)v, (double)gamma_inv));
  const float y = roundf(p * 255.0f);
  if (!(y > 0.0f)) return 0;
  if (y >= 255.0f) return 255;
  return (uint8_t)y;
}

__global__ void tonemap_kernel(const float* __restrict__ rgb, int64_t n, uint8_t* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = tonemap_u8(rgb[i]);
}

cudaError_t launch_tonemap(const float* rgb, int64_t n, uint8_t* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int block = 256;
  tonemap_kernel<<<(unsigned)((n + block - 1) / block), block, 0, s>>>(rgb, n, out);
  return cudaGetLastError();
}

__global__ void render_reduce_kernel(const float* __restrict__ srgb, const int32_t* __restrict__ term,
                                     const int64_t* __restrict__ steps, const double* __restrict__ resid,
                                     int64_t npix, int64_t spa, float* __restrict__ rgb,
                                     int32_t* __restrict__ pclass, int64_t* __restrict__ psteps,
                                     unsigned long long* __restrict__ stats, uint8_t* __restrict__ rgb8) {
  const int64_t pix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int c_cap = 0, c_esc = 0, c_div = 0;
  unsigned long long pst = 0, tot = 0, rbits = 0;
  if (pix < npix) {
    const int64_t spa2 = spa * spa;
    float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f;
    int64_t total = 0;
    double maxr = 0.0;
    unsigned nc = 0, ne = 0, nd = 0;
    for (int64_t q = 0; q < spa2; ++q) {
      const int64_t s = pix * spa2 + q;
      acc0 += srgb[3 * s];
      acc1 += srgb[3 * s + 1];
      acc2 += srgb[3 * s + 2];
      const int t = term[s];
      if (t == TERM_CAPTURED) ++nc;
      else if (t == TERM_DIVERGED) ++nd;
      else ++ne;
      total += steps[s];
      const double r = resid[s];
      if (isfinite(r) && r > maxr) maxr = r;
    }
    const float nf = (float)spa2;
    const float o0 = acc0 / nf, o1 = acc1 / nf, o2 = acc2 / nf;
    if (rgb) {
      rgb[3 * pix] = o0;
      rgb[3 * pix + 1] = o1;
      rgb[3 * pix + 2] = o2;
    }
    if (rgb8) {
      rgb8[3 * pix] = tonemap_u8(o0);
      rgb8[3 * pix + 1] = tonemap_u8(o1);
      rgb8[3 * pix + 2] = tonemap_u8(o2);
    }
    int cls;
    if (nd > 0 && nd >= nc && nd >= ne) cls = TERM_DIVERGED;
    else if (nc >= ne) cls = TERM_CAPTURED;
    else cls = TERM_ESCAPED;
    if (pclass) pclass[pix] = cls;
    const int64_t ps = total / spa2;
    if (psteps) psteps[pix] = ps;
    c_cap = cls == TERM_CAPTURED;
    c_esc = cls == TERM_ESCAPED;
    c_div = cls == TERM_DIVERGED;
    pst = (unsigned long long)ps;
    tot = (unsigned long long)total;
    rbits = (unsigned long long)__double_as_longlong(maxr);
  }
  // warp reduction, then one atomic per warp
  const unsigned FULL = 0xffffffffu;
  for (int o = 16; o > 0; o >>= 1) {
    c_cap += __shfl_down_sync(FULL, c_cap, o);
    c_esc += __shfl_down_sync(FULL, c_esc, o);
    c_div += __shfl_down_sync(FULL, c_div, o);
    pst += __shfl_down_sync(FULL, pst, o);
    tot += __shfl_down_sync(FULL, tot, o);
    const unsigned long long ob = __shfl_down_sync(FULL, rbits, o);
    rbits = ob > rbits ? ob : rbits;  // non-negative doubles order like their bits
  }
  if ((threadIdx.x & 31) == 0) {
    if (c_cap) atomicAdd(&stats[0], (unsigned long long)c_cap);
    if (c_esc) atomicAdd(&stats[1], (unsigned long long)c_esc);
    if (c_div) atomicAdd(&stats[2], (unsigned long long)c_div);
    if (pst) atomicAdd(&stats[3], pst);
    if (rbits) atomicMax(&stats[4], rbits);
    if (tot) atomicAdd(&stats[5], tot);
  }
}

cudaError_t launch_render_reduce(const float* srgb, const int32_t* term, const int64_t* steps,
                                 const double* resid, int64_t npix, int64_t spa, float* rgb,
                                 int32_t* pclass, int64_t* psteps, unsigned long long* stats,
                                 cudaStream_t s, uint8_t* rgb8) {
  if (npix <= 0) return cudaSuccess;
  const int block = 256;
  const int64_t grid = (npix + block - 1) / block;
  render_reduce_kernel<<<(unsigned)grid, block, 0, s>>>(srgb, term, steps, resid, npix, spa, rgb,
                                                        pclass, psteps, stats, rgb8);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Point-wise metric functors over n points (AoS in/out).
// ---------------------------------------------------------------------------
template <int K>
__global__ void pointwise_kernel(const MetricDesc M, int what, const double* __restrict__ in, int64_t n,
                                 double* __restrict__ out, int32_t* __restrict__ iout, int* flags) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (what == PW_ASYM) {
    const double* s = in + 8 * i;
    double x[4] = {s[0], s[1], s[2], s[3]}, p[4] = {s[4], s[5], s[6], s[7]}, d[3];
    metric_asymptotic_direction<K>(M, x, p, d);
    out[3 * i] = d[0]; out[3 * i + 1] = d[1]; out[3 * i + 2] = d[2];
    return;
  }
  const double x[4] = {in[4 * i], in[4 * i + 1], in[4 * i + 2], in[4 * i + 3]};
  if (what == PW_G) {
    double g[16];
    metric_g<K>(M, x, g);
    for (int q = 0; q < 16; ++q) out[16 * i + q] = g[q];
  } else if (what == PW_GINV) {
    double g[16];
    if (!metric_g_inv<K>(M, x, g)) atomicOr(flags, 1);
    for (int q = 0; q < 16; ++q) out[16 * i + q] = g[q];
  } else if (what == PW_DG) {
    double d[64];
    metric_dg<K>(M, x, d);
    for (int q = 0; q < 64; ++q) out[64 * i + q] = d[q];
  } else if (what == PW_CHRISTOFFEL) {
    double G[64];
    if (!metric_christoffel<K>(M, x, G)) atomicOr(flags, 1);
    for (int q = 0; q < 64; ++q) out[64 * i + q] = G[q];
  } else if (what == PW_TERMINATE) {
    iout[i] = metric_terminate<K>(M, x);
  }
}

cudaError_t launch_pointwise(const MetricDesc& M, int what, const double* in, int64_t n, double* out,
                             int32_t* iout, int* flags, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int block = 128;
  const unsigned grid = (unsigned)((n + block - 1) / block);
  switch (M.kind) {
    case KIND_MINKOWSKI: pointwise_kernel<KIND_MINKOWSKI><<<grid, block, 0, s>>>(M, what, in, n, out, iout, flags); break;
    case KIND_SCHWARZSCHILD: pointwise_kernel<KIND_SCHWARZSCHILD><<<grid, block, 0, s>>>(M, what, in, n, out, iout, flags); break;
    case KIND_ALCUBIERRE: pointwise_kernel<KIND_ALCUBIERRE><<<grid, block, 0, s>>>(M, what, in, n, out, iout, flags); break;
    case KIND_MORRIS_THORNE: pointwise_kernel<KIND_MORRIS_THORNE><<<grid, block, 0, s>>>(M, what, in, n, out, iout, flags); break;
    case KIND_FIELD: pointwise_kernel<KIND_FIELD><<<grid, block, 0, s>>>(M, what, in, n, out, iout, flags); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Camera tetrad by Gram-Schmidt against g (camera.rs:47-97), one thread.
// status: 0 ok, GEON_ERR_NOT_TIMELIKE, GEON_ERR_GRAM_SCHMIDT.
// ---------------------------------------------------------------------------
template <int K>
__global__ void tetrad_kernel(const MetricDesc M, const double* __restrict__ obs, double* __restrict__ out,
                              int* __restrict__ status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double x[4] = {obs[0], obs[1], obs[2], obs[3]};
  double g[16];
  metric_g<K>(M, x, g);
  double tet[4][4];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) tet[a][b] = 0.0;
  *status = 0;
  const double gtt = g[0];
  if (!(gtt < 0.0)) {
    *status = GEON_ERR_NOT_TIMELIKE;
    for (int q = 0; q < 16; ++q) out[q] = 0.0;
    return;
  }
  tet[0][0] = 1.0 / sqrt(-gtt);
  for (int i = 0; i < 3; ++i) {
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    v[i + 1] = 1.0;
    for (int k = 0; k <= i; ++k) {
      const double proj = dot4(g, tet[k], v);
      const double norm_k = dot4(g, tet[k], tet[k]);
      const double coeff = proj / norm_k;
      for (int mu = 0; mu < 4; ++mu) v[mu] -= coeff * tet[k][mu];
    }
    const double n2 = dot4(g, v, v);
    if (!(n2 > 0.0)) {
      *status = GEON_ERR_GRAM_SCHMIDT;
      break;
    }
    const double nn = sqrt(n2);
    for (int mu = 0; mu < 4; ++mu) tet[i + 1][mu] = v[mu] / nn;
  }
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) out[4 * a + b] = tet[a][b];
}

cudaError_t launch_tetrad(const MetricDesc& M, const double* obs, double* out16, int* status,
                          cudaStream_t s) {
  switch (M.kind) {
    case KIND_MINKOWSKI: tetrad_kernel<KIND_MINKOWSKI><<<1, 32, 0, s>>>(M, obs, out16, status); break;
    case KIND_SCHWARZSCHILD: tetrad_kernel<KIND_SCHWARZSCHILD><<<1, 32, 0, s>>>(M, obs, out16, status); break;
    case KIND_ALCUBIERRE: tetrad_kernel<KIND_ALCUBIERRE><<<1, 32, 0, s>>>(M, obs, out16, status); break;
    case KIND_MORRIS_THORNE: tetrad_kernel<KIND_MORRIS_THORNE><<<1, 32, 0, s>>>(M, obs, out16, status); break;
    case KIND_FIELD: tetrad_kernel<KIND_FIELD><<<1, 32, 0, s>>>(M, obs, out16, status); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Derived constants that need the deterministic tanh (alcubierre.rs:42).
__global__ void metric_init_kernel(MetricDesc* d) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (d->kind == KIND_ALCUBIERRE) d->alc_denom = 2.0 * dm::tanh_det(d->p[0] / d->p[1]);
}

cudaError_t launch_metric_init(MetricDesc* d_desc, cudaStream_t s) {
  metric_init_kernel<<<1, 32, 0, s>>>(d_desc);
  return cudaGetLastError();
}

__global__ void camera_rays_kernel(const CameraDesc c, double du, double dv, double* __restrict__ out) {
  const int64_t n = c.width * c.height;
  const int64_t pix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= n) return;
  // one sample per pixel at (du, dv): reuse camera_ray's arithmetic with spa = 1
  const int64_t j = pix / c.width, i = pix - j * c.width;
  const double u = (2.0 * ((double)i + du) / c.width_d - 1.0) * c.w_img;
  const double v = -(2.0 * ((double)j + dv) / c.height_d - 1.0) * c.h_img;
  const double fs = (double)c.forward_sign;
  const double dx = -fs;
  const double dy = -v;
  const double dz = c.forward_sign == 1 ? u : fs * u;
  const double norm = sqrt(dx * dx + dy * dy + dz * dz);
  const double n1 = dx / norm, n2 = dy / norm, n3 = dz / norm;
  double* y = out + 8 * pix;
  for (int mu = 0; mu < 4; ++mu) y[mu] = c.obs[mu];
  for (int mu = 0; mu < 4; ++mu)
    y[4 + mu] = c.tet[0][mu] + n1 * c.tet[1][mu] + n2 * c.tet[2][mu] + n3 * c.tet[3][mu];
}

cudaError_t launch_camera_rays(const CameraDesc& c, double du, double dv, double* out, cudaStream_t s) {
  const int64_t n = c.width * c.height;
  if (n <= 0) return cudaSuccess;
  camera_rays_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(c, du, dv, out);
  return cudaGetLastError();
}

__global__ void equatorial_rays_kernel(double m, double r_obs, const double* __restrict__ alpha, int64_t n,
                                       double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double y[8];
  equatorial_ray(m, r_obs, alpha[i], y);
  for (int q = 0; q < 8; ++q) out[8 * i + q] = y[q];
}

cudaError_t launch_equatorial_rays(double m, double r_obs, const double* alpha, int64_t n, double* out,
                                   cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  equatorial_rays_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(m, r_obs, alpha, n, out);
  return cudaGetLastError();
}

// Longest-first claim order of a shadow sweep (see internal.h). A ray's path
// length is set by its impact parameter b = r_obs sin(alpha) / sqrt(1 - 2M/r_obs)
// (bin/validate_shadow.rs:78-79): b > b_c = 3 sqrt(3) M escapes and runs to the
// escape radius, b near b_c orbits the photon sphere first, b < b_c falls in
// after a short path. Claiming the long ones first leaves short rays for the
// end of the sweep, when lanes run out of work. Only the order changes: each
// ray is integrated the same way wherever it runs.
__global__ void shadow_order_kernel(double m, double r_obs, const double* __restrict__ alpha, int64_t n,
                                    int32_t* __restrict__ order, unsigned long long* counters) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  bool is_long = false;
  if (valid) {
    const double b = r_obs * sin(alpha[i]) / sqrt(1.0 - 2.0 * m / r_obs);
    is_long = !(b < 0.998 * 5.196152422706632 * m);  // 3 sqrt(3) M; NaN angles go first
  }
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const unsigned want_long = __ballot_sync(FULL, valid && is_long);
  const unsigned want_short = __ballot_sync(FULL, valid && !is_long);
  unsigned long long bl = 0, bs = 0;
  if (lane == 0) {
    if (want_long) bl = atomicAdd(&counters[0], (unsigned long long)__popc(want_long));
    if (want_short) bs = atomicAdd(&counters[1], (unsigned long long)__popc(want_short));
  }
  bl = __shfl_sync(FULL, bl, 0);
  bs = __shfl_sync(FULL, bs, 0);
  if (!valid) return;
  if (is_long) order[bl + __popc(want_long & lt)] = (int32_t)i;
  else order[n - 1 - (int64_t)(bs + __popc(want_short & lt))] = (int32_t)i;
}

cudaError_t launch_shadow_order(double m, double r_obs, const double* alpha, int64_t n, int32_t* order,
                                unsigned long long* counters, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  shadow_order_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(m, r_obs, alpha, n, order, counters);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Device-side bisection rounds (bin/validate_shadow.rs:70-79, L levels per round)
// ---------------------------------------------------------------------------
// alpha[b*per + i-1] = midpoint of heap node i (1-based) of bracket b: the
// interval of node i follows from the bits of i below its leading one (1 =
// captured: lo = mid; 0 = escaped or diverged: hi = mid), with the same
// 0.5*(lo+hi) arithmetic as the sequential loop.
__global__ void bisect_build_kernel(int64_t nb, int64_t per, const double* __restrict__ lo,
                                    const double* __restrict__ hi, double* __restrict__ alpha) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nb * per) return;
  const int64_t b = t / per;
  const int64_t node = t - b * per + 1;
  double l = lo[b], h = hi[b];
  int depth = 63 - __clzll((long long)node);
  for (int d = depth - 1; d >= 0; --d) {
    const double mid = 0.5 * (l + h);
    if ((node >> d) & 1) l = mid;
    else h = mid;
  }
  alpha[t] = 0.5 * (l + h);
}

__global__ void bisect_walk_kernel(int64_t nb, int64_t per, int levels, const double* __restrict__ alpha,
                                   const int32_t* __restrict__ term, const int64_t* __restrict__ steps,
                                   double* __restrict__ lo, double* __restrict__ hi,
                                   int64_t* __restrict__ path_steps) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb) return;
  int64_t node = 1;
  double l = lo[b], h = hi[b];
  int64_t acc = path_steps ? path_steps[b] : 0;
  for (int d = 0; d < levels; ++d) {
    const int64_t q = b * per + node - 1;
    acc += steps[q];
    if (term[q] == TERM_CAPTURED) {
      l = alpha[q];
      node = 2 * node + 1;
    } else {
      h = alpha[q];
      node = 2 * node;
    }
  }
  lo[b] = l;
  hi[b] = h;
  if (path_steps) path_steps[b] = acc;
}

__global__ void bisect_finish_kernel(int64_t nb, const double* __restrict__ lo, const double* __restrict__ hi,
                                     double* __restrict__ alpha_c) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b < nb) alpha_c[b] = 0.5 * (lo[b] + hi[b]);
}

cudaError_t launch_bisect_build(int64_t nb, int64_t per, const double* lo, const double* hi, double* alpha,
                                cudaStream_t s) {
  const int64_t n = nb * per;
  bisect_build_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(nb, per, lo, hi, alpha);
  return cudaGetLastError();
}

cudaError_t launch_bisect_walk(int64_t nb, int64_t per, int levels, const double* alpha, const int32_t* term,
                               const int64_t* steps, double* lo, double* hi, int64_t* path_steps,
                               cudaStream_t s) {
  bisect_walk_kernel<<<(unsigned)((nb + 127) / 128), 128, 0, s>>>(nb, per, levels, alpha, term, steps, lo, hi,
                                                                  path_steps);
  return cudaGetLastError();
}

cudaError_t launch_bisect_finish(int64_t nb, const double* lo, const double* hi, double* alpha_c,
                                 cudaStream_t s) {
  bisect_finish_kernel<<<(unsigned)((nb + 127) / 128), 128, 0, s>>>(nb, lo, hi, alpha_c);
  return cudaGetLastError();
}

// FMA throughput probes for the roofline denominators (independent chains).
template <typename T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x * (T)1e-3, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

cudaError_t launch_fma_probe(int fp64, void* out, int blocks, int threads, int iters, cudaStream_t s) {
  if (fp64) fma_probe_kernel<double><<<blocks, threads, 0, s>>>((double*)out, iters, 0.999999, 1e-7);
  else fma_probe_kernel<float><<<blocks, threads, 0, s>>>((float*)out, iters, 0.999999f, 1e-7f);
  return cudaGetLastError();
}

__global__ void sky_kernel(const double* __restrict__ dir, int64_t n, int show, float* __restrict__ rgb) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d[3] = {dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]};
  float c[3];
  sky_sample(d, show != 0, c);
  rgb[3 * i] = c[0]; rgb[3 * i + 1] = c[1]; rgb[3 * i + 2] = c[2];
}

cudaError_t launch_sky(const double* dir, int64_t n, int show, float* rgb, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  sky_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(dir, n, show, rgb);
  return cudaGetLastError();
}

}  // namespace geon
