// FP64 curvature (curvature.rs:25-141): Riemann -> Ricci -> R -> Einstein ->
// T_mu_nu -> T(k, k), for batches of points.
//
// The reference differentiates the Christoffel symbols with a point-local
// central difference at x +- 1e-5 e_alpha (curvature.rs:25-46), so every point
// needs Gamma at x and its 8 stencil neighbours. A block handles PPB points;
// its threads first evaluate those Christoffel arrays into shared memory (the
// stencil "halo" lives there), then contract them. Two facts cut the work
// without changing a bit:
//  - where g does not depend on x^alpha (every metric here ignores t; the
//    Schwarzschild and Morris-Thorne metrics also ignore phi), Gamma at
//    x +- h e_alpha is Gamma at x bit for bit, since no operation reads x^alpha.
//    Those stencil slots are not evaluated; the difference reads the centre
//    twice, (G - G) / 2h, as the reference's does.
//  - for the metrics with a generated sparse Christoffel (Alcubierre,
//    Morris-Thorne) the finite differences inside Gamma evaluate g at the
//    stencil point +- h e_beta. Those positions repeat between stencil points
//    (x + h e_1 + h e_2 serves both Gamma(x + h e_1) and Gamma(x + h e_2); the
//    coordinates are formed by the same additions), so g is evaluated once per
//    distinct position (31 instead of 63 for Alcubierre) and each Gamma is
//    formed from those values by the same generated expressions.
// Riemann is formed once per point: the reference forms it twice inside
// einstein() (ricci and ricci_scalar each call riemann) and again for every k
// in nec_contraction(), but it is deterministic, so the bits are the same.
//
// Compiled with --fmad=false; results match the CPU oracle bit for bit.
#include <cuda_runtime.h>

#include <cstring>

#include "internal.h"
#include "metric_fp64.cuh"

namespace geon {

constexpr int CURV_PPB = 16;       // points per block
constexpr int CURV_THREADS = 128;
static_assert(CURV_PPB <= 32 && CURV_THREADS >= 32 + CURV_PPB, "the tetrads run on the second warp");

// Axes g depends on (bit a for x^a).
template <int K>
constexpr int stencil_mask() {
  return K == KIND_MINKOWSKI ? 0 : (K == KIND_SCHWARZSCHILD || K == KIND_MORRIS_THORNE) ? 0x6 : 0xE;
}

__host__ __device__ constexpr int popcount4(int m) { return (m & 1) + ((m >> 1) & 1) + ((m >> 2) & 1) + ((m >> 3) & 1); }

// Stencil of one point for metric K. Slots: 0 the point, 1 + 2 i + m the point
// shifted by +h (m = 0) or -h (m = 1) along the i-th axis g depends on.
// Positions (metrics with values-based Gamma): 0 the point; 1 + 2 i + m one
// shift; 1 + 2 k + 4 i + 2 m + n two shifts along axis i, (x +- h) +- h;
// 1 + 6 k + 4 pair(i, j) + 2 m + n one shift along axis i and one along axis
// j > i.
template <int K>
struct Stencil {
  static constexpr int mask = stencil_mask<K>();
  static constexpr int k = popcount4(mask);
  static constexpr int slots = 1 + 2 * k;
  static constexpr int positions = 1 + 4 * k + 2 * k * k;

  __device__ static __forceinline__ int axis(int i) {  // i-th axis in the mask
    int seen = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a)
      if ((mask >> a) & 1) {
        if (seen == i) return a;
        ++seen;
      }
    return 0;
  }
  // Slot holding Gamma at x + h e_mu (minus = 0) or x - h e_mu (minus = 1).
  __device__ static __forceinline__ int slot_for(int mu, int minus) {
    if (!((mask >> mu) & 1)) return 0;
    return 1 + 2 * popcount4(mask & ((1 << mu) - 1)) + minus;
  }
  __device__ static __forceinline__ double shift(double v, int minus) { return minus ? v - FD_H : v + FD_H; }
  // Coordinates of slot s, formed as the reference forms its stencil points.
  __device__ static __forceinline__ void slot_point(const double x[4], int s, double xs[4]) {
    xs[0] = x[0]; xs[1] = x[1]; xs[2] = x[2]; xs[3] = x[3];
    if (s > 0) {
      const int a = axis((s - 1) >> 1);
      xs[a] = shift(x[a], (s - 1) & 1);
    }
  }
  __device__ static __forceinline__ int pair_index(int i, int j) { return i * (2 * k - i - 1) / 2 + (j - i - 1); }
  // Coordinates of position q: the stencil point, then the shift of the
  // finite difference inside Gamma (metric/mod.rs:25-43).
  __device__ static __forceinline__ void position(const double x[4], int q, double xq[4]) {
    xq[0] = x[0]; xq[1] = x[1]; xq[2] = x[2]; xq[3] = x[3];
    if (q == 0) return;
    q -= 1;
    if (q < 2 * k) {
      const int a = axis(q >> 1);
      xq[a] = shift(x[a], q & 1);
      return;
    }
    q -= 2 * k;
    if (q < 4 * k) {
      const int a = axis(q >> 2);
      xq[a] = shift(shift(x[a], (q >> 1) & 1), q & 1);
      return;
    }
    q -= 4 * k;
    const int pr = q >> 2;
    int i = 0, j = 1;
    for (int ii = 0; ii < k; ++ii)
      for (int jj = ii + 1; jj < k; ++jj)
        if (pair_index(ii, jj) == pr) { i = ii; j = jj; }
    const int a = axis(i), b = axis(j);
    xq[a] = shift(x[a], (q >> 1) & 1);
    xq[b] = shift(x[b], q & 1);
  }
  // Position of the finite-difference input `tag` of slot s; tag 0 is the
  // stencil point itself, tag 1 + 2 i + n its shift along the i-th axis.
  __device__ static __forceinline__ int input_position(int s, int tag) {
    if (s == 0) return tag;
    if (tag == 0) return s;
    const int i = (s - 1) >> 1, m = (s - 1) & 1;
    const int j = (tag - 1) >> 1, n = (tag - 1) & 1;
    if (i == j) return 1 + 2 * k + 4 * i + 2 * m + n;
    if (i < j) return 1 + 6 * k + 4 * pair_index(i, j) + 2 * m + n;
    return 1 + 6 * k + 4 * pair_index(j, i) + 2 * n + m;
  }
};

// Metric values at one position and Gamma from a slot's values: the metrics
// with a generated values-based Christoffel.
template <int K>
struct ValuesGamma {
  static constexpr int nv = 0;
};
template <>
struct ValuesGamma<KIND_ALCUBIERRE> {
  static constexpr int nv = ALCUBIERRE_VALUES;
  __device__ static __forceinline__ void eval(const MetricDesc& M, const double x[4], double* v) {
    alc_g00_g01(M, x, v, v + 1);
  }
  __device__ static __forceinline__ bool gamma(const double* gv, double* G) { return christoffel_alcubierre_from(gv, G); }
};
template <>
struct ValuesGamma<KIND_MORRIS_THORNE> {
  static constexpr int nv = MORRIS_THORNE_VALUES;
  __device__ static __forceinline__ void eval(const MetricDesc& M, const double x[4], double* v) {
    mt_g22_g33(M, x, v, v + 1);
  }
  __device__ static __forceinline__ bool gamma(const double* gv, double* G) {
    return christoffel_morris_thorne_from(gv, G);
  }
};

template <int K>
constexpr size_t curv_smem_doubles() {
  return (size_t)CURV_PPB * Stencil<K>::slots * 64 + (size_t)CURV_PPB * Stencil<K>::positions * ValuesGamma<K>::nv +
         (size_t)CURV_PPB * 16;
}

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

// Static observer tetrad of a point (Gram-Schmidt against g, as camera.rs:47-97
// builds it): rows e_0..e_3, tet[4 a + mu]. Returns false where the point has no
// static observer (g_tt >= 0 or a failed Gram-Schmidt step).
__device__ __forceinline__ bool point_tetrad(const double g[16], double tet[16]) {
#pragma unroll
  for (int q = 0; q < 16; ++q) tet[q] = 0.0;
  bool ok = g[0] < 0.0;
  if (ok) {
    tet[0] = 1.0 / sqrt(-g[0]);
    for (int i = 0; i < 3 && ok; ++i) {
      double v[4] = {0.0, 0.0, 0.0, 0.0};
      v[i + 1] = 1.0;
      for (int kk = 0; kk <= i; ++kk) {
        const double coeff = dot4(g, tet + 4 * kk, v) / dot4(g, tet + 4 * kk, tet + 4 * kk);
        for (int mu = 0; mu < 4; ++mu) v[mu] -= coeff * tet[4 * kk + mu];
      }
      const double n2 = dot4(g, v, v);
      ok = n2 > 0.0;
      const double nn = sqrt(n2);
      for (int mu = 0; mu < 4; ++mu) tet[4 * (i + 1) + mu] = v[mu] / nn;
    }
  }
  return ok;
}

// Null vector q of point p: k = e0 + n1 e1 + n2 e2 + n3 e3 in the point's static
// observer tetrad, with n uniform on the unit sphere from the counter-based
// stream splitmix64(seed ^ (p * nk + q)): z = 2 u1 - 1, phi = 2 pi u2. Where the
// point has no static observer (ok false) k is NaN. The tetrad does not depend
// on q, so a point's tetrad is built once and shared by its nk vectors.
__device__ __forceinline__ void point_null_vector(const double* tet, bool ok, uint64_t seed, int64_t p,
                                                  int64_t nk, int64_t q, double k[4]) {
  const uint64_t h = splitmix64(seed ^ (uint64_t)(p * nk + q));
  const uint64_t h2 = splitmix64(h);
  const double u1 = (double)(h >> 11) * 0x1p-53, u2 = (double)(h2 >> 11) * 0x1p-53;
  const double z = 2.0 * u1 - 1.0;
  const double rho = sqrt(fmax(0.0, 1.0 - z * z));
  double sp, cp;
  dm::sincos_det(6.283185307179586 * u2, &sp, &cp);
  const double n1 = rho * cp, n2v = rho * sp, n3 = z;
#pragma unroll
  for (int mu = 0; mu < 4; ++mu) k[mu] = tet[mu] + n1 * tet[4 + mu] + n2v * tet[8 + mu] + n3 * tet[12 + mu];
  if (!ok) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    k[0] = k[1] = k[2] = k[3] = nan;
  }
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
  using ST = Stencil<K>;
  using VG = ValuesGamma<K>;
  constexpr int NS = ST::slots, NP = ST::positions, NV = VG::nv;
  extern __shared__ double smem[];
  double* G = smem;                                     // [PPB][NS][64]
  double* PV = G + CURV_PPB * NS * 64;                  // [PPB][NP][NV]
  double* RIC = PV + CURV_PPB * NP * NV;                // [PPB][16]
  const int tid = threadIdx.x;
  const int64_t p0 = (int64_t)blockIdx.x * CURV_PPB;
  auto point = [&](int64_t pt, double x[4]) {
    if (GRID) {
      grid_point(grid, pt, x);
    } else {
      x[0] = xs[4 * pt]; x[1] = xs[4 * pt + 1]; x[2] = xs[4 * pt + 2]; x[3] = xs[4 * pt + 3];
    }
  };

  // 1. Christoffel symbols at the stencil slots of each point.
  if constexpr (NV > 0) {
    for (int e = tid; e < CURV_PPB * NP; e += CURV_THREADS) {
      const int p = e / NP, q = e - NP * (e / NP);
      if (p0 + p >= n) continue;
      double x[4], xq[4];
      point(p0 + p, x);
      ST::position(x, q, xq);
      VG::eval(M, xq, PV + (p * NP + q) * NV);
    }
    __syncthreads();
    for (int e = tid; e < CURV_PPB * NS; e += CURV_THREADS) {
      const int p = e / NS, sl = e - NS * (e / NS);
      if (p0 + p >= n) continue;
      double gv[NS * NV];
#pragma unroll
      for (int tag = 0; tag < NS; ++tag) {
        const double* v = PV + (p * NP + ST::input_position(sl, tag)) * NV;
#pragma unroll
        for (int c = 0; c < NV; ++c) gv[tag * NV + c] = v[c];
      }
      if (!VG::gamma(gv, G + (p * NS + sl) * 64)) atomicOr(flags, 1);
    }
  } else {
    for (int e = tid; e < CURV_PPB * NS; e += CURV_THREADS) {
      const int p = e / NS, sl = e - NS * (e / NS);
      if (p0 + p >= n) continue;
      double x[4], xsl[4];
      point(p0 + p, x);
      ST::slot_point(x, sl, xsl);
      if (!metric_christoffel<K>(M, xsl, G + (p * NS + sl) * 64)) atomicOr(flags, 1);
    }
  }
  __syncthreads();

  const double inv_2h = 1.0 / (2.0 * FD_H);
  // Riemann entry R^rho_{sigma mu nu} (curvature.rs:48-70) from the shared stencil.
  auto riem = [&](int p, int rho, int sigma, int mu, int nu) -> double {
    const double* g0 = G + (p * NS) * 64;
    const double* gpm = G + (p * NS + ST::slot_for(mu, 0)) * 64;
    const double* gmm = G + (p * NS + ST::slot_for(mu, 1)) * 64;
    const double* gpn = G + (p * NS + ST::slot_for(nu, 0)) * 64;
    const double* gmn = G + (p * NS + ST::slot_for(nu, 1)) * 64;
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

  // 3. One thread per point: R, G, T. Ricci, R, G and T end here.
  if (what <= 4) {
    if (tid >= CURV_PPB) return;
    const int p = tid;
    const int64_t pt = p0 + p;
    if (pt >= n) return;
    const double* ric = RIC + 16 * p;
    if (what == 1) {
      for (int q = 0; q < 16; ++q) out[16 * pt + q] = ric[q];
      return;
    }
    double x[4];
    point(pt, x);
    double g[16], gi[16];
    metric_g<K>(M, x, g);
    if (!metric_g_inv_given<K>(M, x, g, gi)) atomicOr(flags, 1);
    double rs = 0.0;  // curvature.rs:87-97
#pragma unroll
    for (int q = 0; q < 16; ++q) rs += gi[q] * ric[q];
    if (what == 2) {
      out[pt] = rs;
      return;
    }
    const double factor = 1.0 / (8.0 * 3.141592653589793);
    for (int q = 0; q < 16; ++q) {
      const double ein = ric[q] - 0.5 * g[q] * rs;             // curvature.rs:99-110
      out[16 * pt + q] = what == 3 ? ein : ein * factor;      // curvature.rs:112-122
    }
    return;
  }

  // what 5 and 6: T_mu_nu per point (written over the point's Ricci row), and
  // for the grid job the point's tetrad (over the first stencil slots: the
  // Christoffel arrays are no longer read).
  double* TT = RIC;
  double* TET = G;                                    // [PPB][16]
  int* TOK = (int*)(G + CURV_PPB * 16);               // [PPB]
  // The Einstein and stress-energy tensors on the first CURV_PPB threads and,
  // for the grid job, the tetrads on as many threads of the next warp (both
  // start from g of the point, evaluated on each side), so the block's serial
  // part is the longer of the two instead of their sum.
  if (tid < CURV_PPB && p0 + tid < n) {
    const int p = tid;
    const int64_t pt = p0 + p;
    double* ric = RIC + 16 * p;
    double x[4];
    point(pt, x);
    double g[16], gi[16];
    metric_g<K>(M, x, g);
    if (!metric_g_inv_given<K>(M, x, g, gi)) atomicOr(flags, 1);
    double rs = 0.0;  // curvature.rs:87-97
#pragma unroll
    for (int q = 0; q < 16; ++q) rs += gi[q] * ric[q];
    const double factor = 1.0 / (8.0 * 3.141592653589793);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const double ein = ric[q] - 0.5 * g[q] * rs;    // curvature.rs:99-110
      if (what == 6 && out) out[16 * pt + q] = ein;
      ric[q] = ein * factor;                           // curvature.rs:112-122
    }
  } else if (what == 6 && tid >= 32 && tid < 32 + CURV_PPB && p0 + (tid - 32) < n) {
    const int p = tid - 32;
    double x[4], g[16], tet[16];
    point(p0 + p, x);
    metric_g<K>(M, x, g);
    TOK[p] = point_tetrad(g, tet) ? 1 : 0;
#pragma unroll
    for (int q = 0; q < 16; ++q) TET[16 * p + q] = tet[q];
  }
  __syncthreads();

  // 4. T(k, k) (nec_contraction, curvature.rs:127-136), one (point, vector)
  // pair per thread.
  const int64_t pairs = (int64_t)CURV_PPB * nk;
  for (int64_t e = tid; e < pairs; e += CURV_THREADS) {
    const int p = (int)(e / nk);
    const int64_t c = e - (int64_t)p * nk;
    const int64_t pt = p0 + p;
    if (pt >= n) continue;
    const double* t = TT + 16 * p;
    double k[4];
    if (what == 6) {
      point_null_vector(TET + 16 * p, TOK[p] != 0, seed, pt, nk, c, k);
      if (kout)
        for (int mu = 0; mu < 4; ++mu) kout[4 * (pt * nk + c) + mu] = k[mu];
    } else {
      const double* kp = k_shared ? ks + 4 * c : ks + 4 * (pt * nk + c);
      k[0] = kp[0]; k[1] = kp[1]; k[2] = kp[2]; k[3] = kp[3];
    }
    double sacc = 0.0;
#pragma unroll
    for (int mu = 0; mu < 4; ++mu)
#pragma unroll
      for (int nu = 0; nu < 4; ++nu) sacc += t[4 * mu + nu] * k[mu] * k[nu];
    (what == 6 ? out2 : out)[pt * nk + c] = sacc;
  }
}

template <int K, bool GRID>
static cudaError_t launch_curv_k(const MetricDesc& M, int what, const double* x, int64_t n, const double* k,
                                 int64_t nk, int k_shared, double* out, int* flags, const GridDesc& grid,
                                 uint64_t seed, double* out2, double* kout, cudaStream_t s) {
  const size_t smem = curv_smem_doubles<K>() * sizeof(double);
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
