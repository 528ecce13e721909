// Procedural celestial sphere (sky.rs:16-120) on the device.
//
// The colour is piecewise constant in (theta, phi): a 6-sector palette times a
// 3-band and 24x12 checker modulation plus a hashed starfield on a 512x256 grid.
// acos/atan2 come from CUDA's libdevice; they can differ from glibc by an ulp,
// which changes a colour only when a direction lies within an ulp of a cell
// boundary. Integer hashing, floor, fmod and the f64->f32 casts are exact.
#pragma once
#include <stdint.h>

namespace geon {

constexpr double SKY_PHI_OFFSET = 0.37;
constexpr double SKY_THETA_OFFSET = 0.21;
constexpr double SKY_PI = 3.141592653589793;
constexpr double SKY_TAU = 6.283185307179586;

__device__ __forceinline__ uint64_t sky_hash1(uint64_t x) {  // sky.rs:26-34
  x *= 0x9E3779B97F4A7C15ull;
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  x ^= x >> 31;
  return x;
}

__device__ __forceinline__ uint64_t sky_hash2(int64_t a, int64_t b) {  // sky.rs:37-39
  return sky_hash1(((uint64_t)a * 73856093ull) ^ ((uint64_t)b * 19349663ull));
}

// Rust's saturating `f64 as i64` (NaN -> 0) for the finite, bounded values here.
__device__ __forceinline__ int64_t sky_to_i64(double v) {
  if (isnan(v)) return 0;
  if (v >= 9.2233720368547758e18) return INT64_MAX;
  if (v <= -9.2233720368547758e18) return INT64_MIN;
  return (int64_t)v;
}

__device__ __forceinline__ double sky_rem_euclid(double a, double b) {
  const double r = fmod(a, b);
  return r < 0.0 ? r + fabs(b) : r;
}

__device__ __forceinline__ int64_t sky_rem_euclid_i(int64_t a, int64_t b) {
  const int64_t r = a % b;
  return r < 0 ? r + (b < 0 ? -b : b) : r;
}

__device__ __forceinline__ double sky_clamp(double x, double lo, double hi) {
  if (x < lo) x = lo;
  if (x > hi) x = hi;
  return x;
}

__device__ __forceinline__ void sky_sample(const double dir[3], bool show_stars, float out[3]) {
  const double x = dir[0], y = dir[1], z = dir[2];
  const double r = fmax(sqrt(x * x + y * y + z * z), 1e-30);
  const double theta = acos(sky_clamp(z / r, -1.0, 1.0));
  const double phi = atan2(y, x);
  const double phi_shift = sky_rem_euclid(phi + SKY_PHI_OFFSET, SKY_TAU);
  const double theta_shift = sky_clamp(theta + SKY_THETA_OFFSET, 0.0, SKY_PI);
  // sectors (sky.rs:72-104)
  const int64_t phi_mod = sky_to_i64(floor(phi_shift / SKY_TAU * 6.0));
  const int64_t band = sky_to_i64(floor(theta_shift / SKY_PI * 3.0));
  const double pal[6][3] = {{0.15, 0.08, 0.20}, {0.08, 0.15, 0.22}, {0.20, 0.15, 0.08},
                            {0.10, 0.18, 0.10}, {0.22, 0.10, 0.10}, {0.10, 0.10, 0.22}};
  const int sector = (int)sky_rem_euclid_i(phi_mod, 6);
  const double band_mod = sky_rem_euclid_i(band, 2) == 0 ? 1.0 : 0.6;
  const int64_t ic = sky_to_i64(floor(phi_shift / SKY_TAU * 24.0));
  const int64_t jc = sky_to_i64(floor(theta_shift / SKY_PI * 12.0));
  const double check = sky_rem_euclid_i(ic + jc, 2) == 0 ? 1.0 : 0.55;
  float s0 = (float)(pal[sector][0] * band_mod * check);
  float s1 = (float)(pal[sector][1] * band_mod * check);
  float s2 = (float)(pal[sector][2] * band_mod * check);
  // stars (sky.rs:43-68)
  float t0 = 0.0f, t1 = 0.0f, t2 = 0.0f;
  if (show_stars) {
    const int64_t i = sky_to_i64(floor(phi_shift / SKY_TAU * 512.0));
    const int64_t j = sky_to_i64(floor(theta_shift / SKY_PI * 256.0));
    const uint64_t h = sky_hash2(i, j);
    const double prob = (double)(h & 0xFFFF) / 65535.0;
    if (prob < 0.004) {
      const double brightness = 0.4 + 0.6 * ((double)((h >> 16) & 0xFF) / 255.0);
      const double temp = (double)((h >> 24) & 0xFF) / 255.0;
      t0 = (float)(brightness * (1.0 - 0.3 * temp));
      t1 = (float)(brightness * (1.0 - 0.1 * fabs(temp - 0.5)));
      t2 = (float)(brightness * (0.7 + 0.3 * temp));
    }
  }
  out[0] = fminf(s0 + t0, 1.0f);
  out[1] = fminf(s1 + t1, 1.0f);
  out[2] = fminf(s2 + t2, 1.0f);
}

}  // namespace geon
