// Orbit-plane frame of a ray in a spherically symmetric metric (Schwarzschild,
// Morris-Thorne): the opt-in frame of the mixed-precision renders. Host and
// device code (the CPU tests compile it with g++).
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define GEON_HD __host__ __device__
#else
#define GEON_HD
#endif

namespace geon {

// The frame of a ray's orbit plane (spherically symmetric metrics). With the
// radial unit vector n = (sin th cos ph, sin th sin ph, cos th) and its rate
// w = p^th e_th + p^ph sin th e_ph, the ray moves in the plane of n and w; in
// the basis (e1 = n, e2 = w / |w|, e1 x e2) it starts at theta' = pi/2,
// phi' = 0 with p^theta' = 0 and p^phi' = |w|, while t, r and their momenta are
// unchanged. A radial ray (w = 0) takes e2 = e_th and p^phi' = 0.
GEON_HD inline void orbit_in(const double y[8], double yr[8], float e1[3], float e2[3]) {
  double st, ct, sp, cp;
  ::sincos(y[2], &st, &ct);
  ::sincos(y[3], &sp, &cp);
  const double n[3] = {st * cp, st * sp, ct};
  const double et[3] = {ct * cp, ct * sp, -st};
  const double ep[3] = {-sp, cp, 0.0};
  double w[3];
  for (int i = 0; i < 3; ++i) w[i] = y[6] * et[i] + y[7] * st * ep[i];
  const double wn = ::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  const bool turning = wn > 0.0 && wn < INFINITY;
  for (int i = 0; i < 3; ++i) {
    e1[i] = (float)n[i];
    e2[i] = (float)(turning ? w[i] / wn : et[i]);
  }
  yr[0] = y[0]; yr[1] = y[1]; yr[2] = 1.5707963267948966; yr[3] = 0.0;
  yr[4] = y[4]; yr[5] = y[5]; yr[6] = 0.0; yr[7] = turning ? wn : 0.0;
}

// Back from the orbit-plane frame: theta, phi from the final radial direction
// n = cos phi' e1 + sin phi' e2 (phi in (-pi, pi]: the orbit frame does not
// count turns), and p^theta, p^phi from its rate p^phi' (-sin phi' e1 + cos
// phi' e2).
GEON_HD inline void orbit_out(const double yr[8], const float e1[3], const float e2[3], double y[8]) {
  double sf, cf;
  ::sincos(yr[3], &sf, &cf);
  double n[3], w[3];
  for (int i = 0; i < 3; ++i) {
    n[i] = cf * (double)e1[i] + sf * (double)e2[i];
    w[i] = yr[7] * (cf * (double)e2[i] - sf * (double)e1[i]);
  }
  const double nn = ::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
  const double nz = ::fmin(1.0, ::fmax(-1.0, n[2] / nn));
  const double th = ::acos(nz), ph = ::atan2(n[1], n[0]);
  double st, ct, sp, cp;
  ::sincos(th, &st, &ct);
  ::sincos(ph, &sp, &cp);
  y[0] = yr[0]; y[1] = yr[1]; y[2] = th; y[3] = ph;
  y[4] = yr[4]; y[5] = yr[5];
  y[6] = w[0] * ct * cp + w[1] * ct * sp - w[2] * st;
  y[7] = (w[1] * cp - w[0] * sp) / st;
}

}  // namespace geon
