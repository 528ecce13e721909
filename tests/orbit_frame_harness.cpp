// C entry points over geon_gb300/csrc/orbit_frame.cuh for the CPU tests
// (compiled by tests/test_orbit_frame.py into a temporary directory).
#include "orbit_frame.cuh"

extern "C" void orbit_in_n(const double* y, long n, double* yr, float* e1, float* e2) {
  for (long i = 0; i < n; ++i) geon::orbit_in(y + 8 * i, yr + 8 * i, e1 + 3 * i, e2 + 3 * i);
}
extern "C" void orbit_out_n(const double* yr, const float* e1, const float* e2, long n, double* y) {
  for (long i = 0; i < n; ++i) geon::orbit_out(yr + 8 * i, e1 + 3 * i, e2 + 3 * i, y + 8 * i);
}
