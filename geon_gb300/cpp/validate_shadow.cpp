// bin/validate_shadow.rs on the GPU through geon.hpp: the Schwarzschild shadow
// by bisection on the launch angle (same settings, same printed lines, exit 1
// on failure). The 60 halvings run as the library's speculative bisection,
// which replays the sequential loop (bin/validate_shadow.rs:70-77) bit for bit.
#include <cmath>
#include <cstdio>

#include "geon.hpp"
#include "rust_fmt.hpp"

using namespace rustfmt;

int main() {
  try {
    const geon::Metric metric = geon::Schwarzschild(1.0);
    const double mass = 1.0, r_obs = 20.0;
    const double b_analytic = std::sqrt(3.0) * 3.0;
    const double f = 1.0 - 2.0 * mass / r_obs;
    const double alpha_analytic = std::asin(b_analytic * std::sqrt(f) / r_obs);
    const double to_deg = 180.0 / 3.141592653589793;  // f64::to_degrees
    std::printf("== Schwarzschild shadow validation ==\n");
    std::printf("M = %s, r_obs = %s\n", display(mass).c_str(), display(r_obs).c_str());
    std::printf("analytic: b_c = 3√3 M = %s, α_c = %s rad = %s°\n", fixed(b_analytic, 6).c_str(),
                fixed(alpha_analytic, 6).c_str(), fixed(alpha_analytic * to_deg, 4).c_str());
    double lo = 0.0, hi = 1.5707963267948966 - 1e-3;
    auto captured = [&](double a) {
      return geon::trace(metric, geon::equatorial_ray(metric, r_obs, a), 0.01, 200000).termination ==
             geon::Termination::Captured;
    };
    if (!captured(lo)) {
      std::fprintf(stderr, "radial ray should be captured\n");
      return 101;
    }
    if (captured(hi)) {
      std::fprintf(stderr, "grazing ray should escape\n");
      return 101;
    }
    const double alpha_c = geon::shadow_bisect(metric, r_obs, lo, hi, 60);
    const double b_c = r_obs * std::sin(alpha_c) / std::sqrt(f);
    std::printf("measured: b_c = %s, α_c = %s rad = %s°\n", fixed(b_c, 6).c_str(), fixed(alpha_c, 6).c_str(),
                fixed(alpha_c * to_deg, 4).c_str());
    const double rel_err = std::fabs(b_c - b_analytic) / b_analytic;
    std::printf("relative error: %s\n", exp(rel_err, 4).c_str());
    if (rel_err < 0.01) {
      std::printf("PASS (< 1%% error)\n");
      return 0;
    }
    std::printf("FAIL — Phase 1 not validated. Integrator or metric is wrong.\n");
    return 1;
  } catch (const geon::Panic& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 101;
  }
}
