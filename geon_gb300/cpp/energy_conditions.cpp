// bin/energy_conditions.rs on the GPU: the bin's numbers from one batched
// device job (geon_energy_conditions) printed exactly as the bin prints them
// (print_row, energy_conditions.rs:26-34, and the println! lines of main).
#include <cmath>
#include <cstdio>
#include <string>

#include "geon.hpp"
#include "rust_fmt.hpp"

using namespace rustfmt;

static void header(const char* name) { std::printf("\n== %s ==\n", name); }

static void print_row(const std::string& label, double val, double threshold, const char* note) {
  const char* flag = val < -threshold ? "NEC VIOLATED" : (std::fabs(val) < threshold ? "≈ 0" : "NEC ok");
  std::printf("  %s  %s   [%s]  %s\n", pad_right(label, 28).c_str(), pad_left(exp(val, 4, true), 13).c_str(), flag,
              note);
}

int main() {
  double v[GEON_ENERGY_CONDITIONS_N];
  try {
    geon::check(geon_energy_conditions(v));
  } catch (const geon::Panic& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 101;
  }
  header("Minkowski (sanity, T = 0 expected)");
  print_row("T_μν k^μ k^ν", v[0], 1e-10, "should be 0");
  print_row("Ricci scalar", v[1], 1e-10, "should be 0");
  header("Schwarzschild (sanity, vacuum: T = 0, R = 0)");
  const int rs[3] = {5, 10, 30};
  for (int i = 0; i < 3; ++i) {
    char l[64];
    std::snprintf(l, sizeof l, "r = %4d  NEC contraction", rs[i]);
    print_row(l, v[2 + 2 * i], 1e-4, "vacuum → ~0");
    std::snprintf(l, sizeof l, "r = %4d  Ricci scalar", rs[i]);
    print_row(l, v[3 + 2 * i], 1e-4, "vacuum → ~0");
  }
  header("Alcubierre warp bubble (expecting NEC violation across bubble wall)");
  std::printf("  scanning along x at y=z=0:\n");
  for (int n = 0; n < 41; n += 4) {
    char l[64];
    std::snprintf(l, sizeof l, "x = %6.2f", -4.0 + 0.2 * n);
    print_row(l, v[8 + n], 1e-6, "");
  }
  std::printf("  minimum T_μν k^μ k^ν = %s at x = %s  (negative = exotic matter required)\n", exp(v[49], 4, true).c_str(),
              fixed(v[50], 2).c_str());
  std::printf("  ∫ T_kk dx (negative part only, axis only) ≈ %s  (rough exotic-mass proxy)\n",
              exp(v[51], 4, true).c_str());
  header("Morris–Thorne wormhole (expecting NEC violation near throat)");
  std::printf("  scanning along l (proper radial) at θ=π/2, φ=0:\n");
  for (int n = 0; n < 41; n += 4) {
    char l[64];
    std::snprintf(l, sizeof l, "l = %6.2f", -4.0 + 0.2 * n);
    print_row(l, v[52 + n], 1e-6, "");
  }
  std::printf("  minimum T_μν k^μ k^ν = %s at l = %s  (negative ⇒ exotic matter at throat)\n", exp(v[93], 4, true).c_str(),
              fixed(v[94], 2).c_str());
  std::printf("\n  T^μ_ν diagonal at throat (l=0):\n");
  for (int i = 0; i < 4; ++i) std::printf("    T[%d][%d] = %s\n", i, i, exp(v[95 + i], 4, true).c_str());
  return 0;
}
