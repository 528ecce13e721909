// C entry points over geon_gb300/csrc/serve_host.h for the CPU tests
// (compiled by tests/test_serve_host.py into a temporary directory).
#include <cstdint>
#include <vector>

#include "serve_host.h"

using namespace geon::serve_host;

extern "C" {
void* arena_new(size_t n) {
  auto* a = new Arena();
  a->init(n);
  return a;
}
void arena_free(void* a) { delete static_cast<Arena*>(a); }
int arena_alloc(void* a, size_t n, size_t* off) { return static_cast<Arena*>(a)->alloc(n, off) ? 1 : 0; }
void arena_release(void* a, size_t off, size_t n) { static_cast<Arena*>(a)->release(off, n); }
size_t align_up(size_t n) { return rup(n); }

void tree(double lo, double hi, int levels, double* out) {
  std::vector<double> a;
  bisect_tree(lo, hi, levels, a);
  for (size_t i = 0; i < a.size(); ++i) out[i] = a[i];
}

void order(const int* cls, const int64_t* left, const uint64_t* id, const int* slot, int n, int nclasses,
           size_t stride, int* out, unsigned* counts) {
  std::vector<ClaimEntry> e;
  for (int i = 0; i < n; ++i) e.push_back({cls[i], left[i], id[i], slot[i]});
  claim_order(e, nclasses, stride, out, counts);
}
}
