// FP64 curvature (curvature.rs:25-141): Riemann -> Ricci -> R -> Einstein ->
// T_mu_nu -> T(k, k), for batches of points.
//
// The reference differentiates the Christoffel symbols with a point-local
// central difference at x +- 1e-5 e_alpha (curvature.rs:25-46), so every point
// needs Gamma at 9 positions: x and its 8 stencil neighbours. A block handles
// PPB points; its threads first evaluate those 9*PPB Christoffel arrays in
// parallel into shared memory (the stencil "halo" lives there), then contract
// them. Riemann is formed once per point: the reference forms it twice inside
// einstein() (ricci and ricci_scalar each call riemann) and again for every k
// in nec_contraction(), but it is deterministic, so the bits are the same.
//
// Compiled with --fmad=false; results match the CPU oracle bit for bit.
#include <cuda_runtime.h>

#include <cstring>

#include "internal.h"
#include "metric_fp64.cuh"

namespace geon {

constexpr int CURV_PPB = 16;                 // points per block
constexpr int CURV_THREADS = CURV_PPB * 9;   // one thread per stencil position

// Point p of a grid job: index p = (iz * ny + iy) * nx + ix, coordinate
// x^i = lo_i + i_i * ((hi_i - lo_i) / (n_i - 1)) (endpoints included), x^0 = t.
__device__ __forceinline__ void grid_point(const GridDesc& G, int64_t p, double x[4]) {
  const int64_t ix = p % G.n[0];
  const int64_t iy = (p / G.n[0]) % G.n[1];
  const int64_t iz = p / (G.n[0] * G.n[1]);
  x[0] = G.t;
  x[1] = G.n[0] > 1 ? G.lo[0] + (double)ix * ((G.hi[0] - G.lo[0]) / (double)(G.n[0] - 1)) : G.lo[0];
  x[2] = G.n[1] > 1 ? G.lo[1] + (double)iy * ((G.hi[1] - G.lo[1]) / (double)(G.n[1] - 1)) : G.lo[1];
  x[3] = G.n[2] > 1 ? G.lo[2] + (double)iz * ((G.hi[2] - G.lo[2]) / (double)(G.n[2] - 1)) : G.lo[2];
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Null vector q of point p: k = e0 + n1 e1 + n2 e2 + n3 e3 in the point's static
// observer tetrad (Gram-Schmidt against g, as camera.rs:47-97 builds it), with
// n uniform on the unit sphere from the counter-based stream
// splitmix64(seed ^ (p * nk + q)): z = 2 u1 - 1, phi = 2 pi u2.
// Returns false where the point has no static observer (g_tt >= 0 or a failed
// Gram-Schmidt); k is then NaN.
__device__ __forceinline__ bool point_null_vector(const double g[16], uint64_t seed, int64_t p, int64_t nk,
                                                  int64_t q, double k[4]) {
  double tet[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) tet[a][b] = 0.0;
  bool ok = g[0] < 0.0;
  if (ok) {
    tet[0][0] = 1.0 / sqrt(-g[0]);
    for (int i = 0; i < 3 && ok; ++i) {
      double v[4] = {0.0, 0.0, 0.0, 0.0};
      v[i + 1] = 1.0;
      for (int kk = 0; kk <= i; ++kk) {
        const double coeff = dot4(g, tet[kk], v) / dot4(g, tet[kk], tet[kk]);
        for (int mu = 0; mu < 4; ++mu) v[mu] -= coeff * tet[kk][mu];
      }
      const double n2 = dot4(g, v, v);
      ok = n2 > 0.0;
      const double nn = sqrt(n2);
      for (int mu = 0; mu < 4; ++mu) tet[i + 1][mu] = v[mu] / nn;
    }
  }
  const uint64_t h = splitmix64(seed ^ (uint64_t)(p * nk + q));
  const uint64_t h2 = splitmix64(h);
  const double u1 = (double)(h >> 11) * 0x1p-53, u2 = (double)(h2 >> 11) * 0x1p-53;
  const double z = 2.0 * u1 - 1.0;
  const double rho = sqrt(fmax(0.0, 1.0 - z * z));
  double sp, cp;
  dm::sincos_det(6.283185307179586 * u2, &sp, &cp);
  const double n1 = rho * cp, n2v = rho * sp, n3 = z;
#pragma unroll
  for (int mu = 0; mu < 4; ++mu) k[mu] = tet[0][mu] + n1 * tet[1][mu] + n2v * tet[2][mu] + n3 * tet[3][mu];
  if (!ok) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    k[0] = k[1] = k[2] = k[3] = nan;
  }
  return ok;
}

// what: 0 riemann(256) 1 ricci(16) 2 ricci_scalar(1) 3 einstein(16) 4 stress_energy(16) 5 nec(nk)
//       6 grid job: einstein (out, 16 per point; may be null) and nec (out2, nk per point)
//         against generated null vectors (written to kout when not null)
template <int K, bool GRID>
__global__ void __launch_bounds__(CURV_THREADS)
curvature_kernel(const MetricDesc M, int what, const double* __restrict__ xs, int64_t n,
                 const double* __restrict__ ks, int64_t nk, int k_shared, double* __restrict__ out,
                 int* flags, const GridDesc grid, uint64_t seed, double* __restrict__ out2,
                 double* __restrict__ kout) {
  extern __shared__ double smem[];
  double* G = smem;                               // [PPB][9][64]
  double* RIC = smem + CURV_PPB * 9 * 64;         // [PPB][16]
  const int tid = threadIdx.x;
  const int64_t p0 = (int64_t)blockIdx.x * CURV_PPB;

  // 1. Christoffel symbols at the 9 stencil positions of each point.
  {
    const int p = tid / 9, o = tid - 9 * (tid / 9);
    const int64_t pt = p0 + p;
    if (pt < n) {
      double x[4];
      if (GRID) {
        grid_point(grid, pt, x);
      } else {
        x[0] = xs[4 * pt]; x[1] = xs[4 * pt + 1]; x[2] = xs[4 * pt + 2]; x[3] = xs[4 * pt + 3];
      }
      if (o > 0) {  // o = 1 + 2 alpha: x + h e_alpha; o = 2 + 2 alpha: x - h e_alpha
        const int alpha = (o - 1) >> 1;
        if (o & 1) x[alpha] += FD_H;
        else x[alpha] -= FD_H;
      }
      double g[64];
      if (!metric_christoffel<K>(M, x, g)) atomicOr(flags, 1);
      double* dst = G + (p * 9 + o) * 64;
#pragma unroll 8
      for (int q = 0; q < 64; ++q) dst[q] = g[q];
    }
  }
  __syncthreads();

  const double inv_2h = 1.0 / (2.0 * FD_H);
  // Riemann entry R^rho_{sigma mu nu} (curvature.rs:48-70) from the shared stencil.
  auto riem = [&](int p, int rho, int sigma, int mu, int nu) -> double {
    const double* g0 = G + (p * 9) * 64;
    const double* gpm = G + (p * 9 + 1 + 2 * mu) * 64;
    const double* gmm = G + (p * 9 + 2 + 2 * mu) * 64;
    const double* gpn = G + (p * 9 + 1 + 2 * nu) * 64;
    const double* gmn = G + (p * 9 + 2 + 2 * nu) * 64;
    const double term1 = (gpm[16 * rho + 4 * nu + sigma] - gmm[16 * rho + 4 * nu + sigma]) * inv_2h;
    const double term2 = (gpn[16 * rho + 4 * mu + sigma] - gmn[16 * rho + 4 * mu + sigma]) * inv_2h;
    double term3 = 0.0, term4 = 0.0;
#pragma unroll
    for (int lambda = 0; lambda < 4; ++lambda) {
      term3 += g0[16 * rho + 4 * mu + lambda] * g0[16 * lambda + 4 * nu + sigma];
      term4 += g0[16 * rho + 4 * nu + lambda] * g0[16 * lambda + 4 * mu + sigma];
    }
    return term1 - term2 + term3 - term4;
  };

  if (what == 0) {
    for (int e = tid; e < CURV_PPB * 256; e += CURV_THREADS) {
      const int p = e >> 8, q = e & 255;
      const int64_t pt = p0 + p;
      if (pt >= n) continue;
      out[256 * pt + q] = riem(p, q >> 6, (q >> 4) & 3, (q >> 2) & 3, q & 3);
    }
    return;
  }

  // 2. Ricci R_mu_nu = sum_alpha R^alpha_{mu alpha nu} (curvature.rs:72-85).
  for (int e = tid; e < CURV_PPB * 16; e += CURV_THREADS) {
    const int p = e >> 4, mu = (e >> 2) & 3, nu = e & 3;
    if (p0 + p >= n) continue;
    double s = 0.0;
#pragma unroll
    for (int alpha = 0; alpha < 4; ++alpha) s += riem(p, alpha, mu, alpha, nu);
    RIC[16 * p + 4 * mu + nu] = s;
  }
  __syncthreads();

  // 3. One thread per point: R, G, T, and the contractions.
  if (tid < CURV_PPB) {
    const int p = tid;
    const int64_t pt = p0 + p;
    if (pt >= n) return;
    const double* ric = RIC + 16 * p;
    if (what == 1) {
      for (int q = 0; q < 16; ++q) out[16 * pt + q] = ric[q];
      return;
    }
    double x[4];
    if (GRID) {
      grid_point(grid, pt, x);
    } else {
      x[0] = xs[4 * pt]; x[1] = xs[4 * pt + 1]; x[2] = xs[4 * pt + 2]; x[3] = xs[4 * pt + 3];
    }
    double gi[16];
    if (!metric_g_inv<K>(M, x, gi)) atomicOr(flags, 1);
    double rs = 0.0;  // curvature.rs:87-97
#pragma unroll
    for (int q = 0; q < 16; ++q) rs += gi[q] * ric[q];
    if (what == 2) {
      out[pt] = rs;
      return;
    }
    double g[16];
    metric_g<K>(M, x, g);
    double t[16], ein[16];
    const double factor = 1.0 / (8.0 * 3.141592653589793);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      ein[q] = ric[q] - 0.5 * g[q] * rs;            // curvature.rs:99-110
      t[q] = what == 3 ? ein[q] : ein[q] * factor;  // curvature.rs:112-122
    }
    if (what == 3 || what == 4) {
      for (int q = 0; q < 16; ++q) out[16 * pt + q] = t[q];
      return;
    }
    if (what == 6) {  // grid job: G_mu_nu, then T(k, k) for generated null vectors
      if (out)
        for (int q = 0; q < 16; ++q) out[16 * pt + q] = ein[q];
      for (int64_t c = 0; c < nk; ++c) {
        double k[4];
        point_null_vector(g, seed, pt, nk, c, k);
        if (kout)
          for (int mu = 0; mu < 4; ++mu) kout[4 * (pt * nk + c) + mu] = k[mu];
        double sacc = 0.0;  // nec_contraction (curvature.rs:127-136)
#pragma unroll
        for (int mu = 0; mu < 4; ++mu)
#pragma unroll
          for (int nu = 0; nu < 4; ++nu) sacc += t[4 * mu + nu] * k[mu] * k[nu];
        out2[pt * nk + c] = sacc;
      }
      return;
    }
    for (int64_t c = 0; c < nk; ++c) {  // curvature.rs:127-136
      const double* kp = k_shared ? ks + 4 * c : ks + 4 * (pt * nk + c);
      const double k[4] = {kp[0], kp[1], kp[2], kp[3]};
      double s = 0.0;
#pragma unroll
      for (int mu = 0; mu < 4; ++mu)
#pragma unroll
        for (int nu = 0; nu < 4; ++nu) s += t[4 * mu + nu] * k[mu] * k[nu];
      out[pt * nk + c] = s;
    }
  }
}

template <int K, bool GRID>
static cudaError_t launch_curv_k(const MetricDesc& M, int what, const double* x, int64_t n, const double* k,
                                 int64_t nk, int k_shared, double* out, int* flags, const GridDesc& grid,
                                 uint64_t seed, double* out2, double* kout, cudaStream_t s) {
  const size_t smem = (size_t)(CURV_PPB * 9 * 64 + CURV_PPB * 16) * sizeof(double);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(curvature_kernel<K, GRID>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr_set = true;
  }
  const int64_t blocks = (n + CURV_PPB - 1) / CURV_PPB;
  curvature_kernel<K, GRID><<<(unsigned)blocks, CURV_THREADS, smem, s>>>(M, what, x, n, k, nk, k_shared, out,
                                                                         flags, grid, seed, out2, kout);
  return cudaGetLastError();
}

template <bool GRID>
static cudaError_t launch_curv(const MetricDesc& M, int what, const double* x, int64_t n, const double* k,
                               int64_t nk, int k_shared, double* out, int* flags, const GridDesc& grid,
                               uint64_t seed, double* out2, double* kout, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  switch (M.kind) {
    case KIND_MINKOWSKI: return launch_curv_k<KIND_MINKOWSKI, GRID>(M, what, x, n, k, nk, k_shared, out, flags, grid, seed, out2, kout, s);
    case KIND_SCHWARZSCHILD: return launch_curv_k<KIND_SCHWARZSCHILD, GRID>(M, what, x, n, k, nk, k_shared, out, flags, grid, seed, out2, kout, s);
    case KIND_ALCUBIERRE: return launch_curv_k<KIND_ALCUBIERRE, GRID>(M, what, x, n, k, nk, k_shared, out, flags, grid, seed, out2, kout, s);
    case KIND_MORRIS_THORNE: return launch_curv_k<KIND_MORRIS_THORNE, GRID>(M, what, x, n, k, nk, k_shared, out, flags, grid, seed, out2, kout, s);
    case KIND_FIELD: return launch_curv_k<KIND_FIELD, GRID>(M, what, x, n, k, nk, k_shared, out, flags, grid, seed, out2, kout, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_curvature(const MetricDesc& M, int what, const double* x, int64_t n, const double* k,
                             int64_t nk, int k_shared, double* out, int* flags, cudaStream_t s) {
  GridDesc none;
  memset(&none, 0, sizeof none);
  return launch_curv<false>(M, what, x, n, k, nk, k_shared, out, flags, none, 0, nullptr, nullptr, s);
}

cudaError_t launch_curvature_grid(const MetricDesc& M, const GridDesc& grid, int64_t nk, uint64_t seed,
                                  double* einstein, double* nec, double* kout, int* flags, cudaStream_t s) {
  const int64_t n = grid.n[0] * grid.n[1] * grid.n[2];
  return launch_curv<true>(M, 6, nullptr, n, nullptr, nk, 0, einstein, flags, grid, seed, nec, kout, s);
}

}  // namespace geon
