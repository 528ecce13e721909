// bin/energy_conditions.rs as one batched device job (geon_energy_conditions).
//
// The bin evaluates T(k, k), the Ricci scalar and T^mu_nu point by point in
// serial loops (energy_conditions.rs:37-156). Here every point of a metric's
// scans goes to the device in one batched launch of the curvature kernel
// (per-point null vectors where the bin uses them), and the host then forms
// the bin's minimum, its location and the negative-part integral in the bin's
// own loop order, so every number equals the one the point-wise calls give.
#include <cmath>
#include <vector>

#include "internal.h"

namespace {

struct Metric {
  geon_metric_t h = nullptr;
  int rc = GEON_OK;
  Metric(int kind, const double* p, int np) { rc = geon_metric_create(kind, p, np, &h); }
  ~Metric() {
    if (h) geon_metric_destroy(h);
  }
};

constexpr double HALF_PI = 1.5707963267948966;  // std::f64::consts::FRAC_PI_2

// The bin's x (or l) scan: -4.0 + 0.2 * n for n = 0..40 (energy_conditions.rs:86-87, 132-133).
double scan_coord(int n) { return -4.0 + 0.2 * (double)n; }

}  // namespace

extern "C" int geon_energy_conditions(double* out) {
  if (!out) return geon::set_last_error(GEON_ERR_INVALID, "null output");
  int w = 0;
  {  // Minkowski (:38-48): one point, k = (1, 1, 0, 0)
    Metric m(GEON_MINKOWSKI, nullptr, 0);
    if (m.rc) return m.rc;
    const double x[4] = {0.0, 1.0, 1.0, 1.0};
    const double k[4] = {1.0, 1.0, 0.0, 0.0};
    if (int rc = geon_nec_contraction(m.h, x, 1, k, 1, 1, out + w)) return rc;
    if (int rc = geon_ricci_scalar(m.h, x, 1, out + w + 1)) return rc;
    w += 2;
  }
  {  // Schwarzschild::new(1.0) (:50-67): r = 5, 10, 30 on the equator, k = (1/sqrt f, -sqrt f, 0, 0)
    const double p[1] = {1.0};
    Metric m(GEON_SCHWARZSCHILD, p, 1);
    if (m.rc) return m.rc;
    const double rs[3] = {5.0, 10.0, 30.0};
    double x[12], k[12], nec[3], ric[3];
    for (int i = 0; i < 3; ++i) {
      const double f = 1.0 - 2.0 / rs[i];
      const double xi[4] = {0.0, rs[i], HALF_PI, 0.0};
      const double ki[4] = {1.0 / std::sqrt(f), -std::sqrt(f), 0.0, 0.0};
      for (int c = 0; c < 4; ++c) {
        x[4 * i + c] = xi[c];
        k[4 * i + c] = ki[c];
      }
    }
    if (int rc = geon_nec_contraction(m.h, x, 3, k, 1, 0, nec)) return rc;
    if (int rc = geon_ricci_scalar(m.h, x, 3, ric)) return rc;
    for (int i = 0; i < 3; ++i) {
      out[w++] = nec[i];
      out[w++] = ric[i];
    }
  }
  {  // Alcubierre {R 2, thickness 0.5, v 2, x_s 0} (:69-121): the 41-point scan and the integral
    const double p[4] = {2.0, 0.5, 2.0, 0.0};
    Metric m(GEON_ALCUBIERRE, p, 4);
    if (m.rc) return m.rc;
    const double k[4] = {1.0, 1.0, 0.0, 0.0};
    std::vector<double> xs;
    for (int n = 0; n < 41; ++n) xs.push_back(scan_coord(n));
    const double dx = 0.05;
    int n_int = 0;
    for (double x_pos = -5.0; x_pos <= 5.0; x_pos += dx) {  // the bin's accumulated positions
      xs.push_back(x_pos);
      ++n_int;
    }
    std::vector<double> pts(4 * xs.size(), 0.0), nec(xs.size());
    for (size_t i = 0; i < xs.size(); ++i) pts[4 * i + 1] = xs[i];
    if (int rc = geon_nec_contraction(m.h, pts.data(), xs.size(), k, 1, 1, nec.data())) return rc;
    double min_val = INFINITY, min_x = 0.0;
    for (int n = 0; n < 41; ++n) {
      if (nec[n] < min_val) {
        min_val = nec[n];
        min_x = xs[n];
      }
      out[w++] = nec[n];
    }
    out[w++] = min_val;
    out[w++] = min_x;
    double integral = 0.0;
    for (int i = 0; i < n_int; ++i) {
      const double v = nec[41 + i];
      if (v < 0.0) integral += v * dx;
    }
    out[w++] = integral;
  }
  {  // Morris-Thorne {b0 1} (:123-156): the 41-point l scan and T^mu_nu at the throat
    const double p[1] = {1.0};
    Metric m(GEON_MORRIS_THORNE, p, 1);
    if (m.rc) return m.rc;
    const double k[4] = {1.0, 1.0, 0.0, 0.0};
    double pts[41 * 4], nec[41];
    for (int n = 0; n < 41; ++n) {
      pts[4 * n] = 0.0;
      pts[4 * n + 1] = scan_coord(n);
      pts[4 * n + 2] = HALF_PI;
      pts[4 * n + 3] = 0.0;
    }
    if (int rc = geon_nec_contraction(m.h, pts, 41, k, 1, 1, nec)) return rc;
    double min_val = INFINITY, min_l = 0.0;
    for (int n = 0; n < 41; ++n) {
      if (nec[n] < min_val) {
        min_val = nec[n];
        min_l = pts[4 * n + 1];
      }
      out[w++] = nec[n];
    }
    out[w++] = min_val;
    out[w++] = min_l;
    const double xt[4] = {0.0, 0.0, HALF_PI, 0.0};
    double t[16];
    if (int rc = geon_stress_energy(m.h, xt, 1, t)) return rc;
    for (int i = 0; i < 4; ++i) out[w++] = t[5 * i];
  }
  return GEON_OK;
}
