// Host check of the fast division in exshalos_gb300/csrc/intdiv.cuh against the
// hardware division (run by tests/test_fixedpoint.py).
#include <cstdio>
#include <random>
#include <vector>
#include "intdiv.cuh"
int main() {
  using namespace exh;
  long bad = 0, n = 0;
  std::mt19937 g(11);
  std::vector<uint32_t> ds;
  for (uint32_t d = 1; d <= 5000; d++) ds.push_back(d);
  for (int e = 12; e < 32; e++) { ds.push_back(1u << e); ds.push_back((1u << e) - 1); ds.push_back((1u << e) + 1); }
  for (int t = 0; t < 2000; t++) ds.push_back(g() | 1u);
  ds.push_back(0xffffffffu);
  for (uint32_t d : ds) {
    const FastDiv f = make_fastdiv(d);
    for (int t = 0; t < 20000; t++) {
      uint32_t x = g();
      if (t < 64) x = 0xffffffffu - t;
      else if (t < 128) x = (uint32_t)(t - 64);
      else if (t < 256) x = (uint32_t)((uint64_t)d * (g() % ((uint64_t)0xffffffffu / d + 1)) - (t & 1));
      if (fd_div(x, f) != x / d) { if (bad < 5) printf("d %u x %u got %u want %u\n", d, x, fd_div(x, f), x / d); bad++; }
      n++;
    }
  }
  printf("checked %ld bad %ld\n", n, bad);
  return bad != 0;
}
