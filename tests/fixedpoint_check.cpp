// Host check of the fixed-point conversions in exshalos_gb300/csrc/fixedpoint.cuh
// against the FP64 expressions they restate (run by tests/test_fixedpoint.py).
#include <cfenv>
#include <cmath>
#include <cstdio>
#include <random>
#include "fixedpoint.cuh"
int main() {
  using namespace exh;
  long bad = 0, n = 0;
  for (uint32_t u = 0; u <= 0x3f800000u; u++) {
    float w; std::memcpy(&w, &u, 4);
    const uint64_t want = (uint64_t)std::nearbyint((double)w * 1099511627776.0);
    if (fp_quanta40(w) != want) { if (bad < 5) printf("quanta %08x %llu %llu\n", u, (unsigned long long)fp_quanta40(w), (unsigned long long)want); bad++; }
    n++;
  }
  std::mt19937_64 g(7);
  for (long t = 0; t < 20000000; t++) {
    uint64_t q = g();
    const int len = 1 + (int)(g() % 64);
    q = len == 64 ? q : (q & ((1ull << len) - 1ull));
    if (t % 4 == 1 && len > 30) q = (q >> 29 << 29) | (1ull << 28);       // exact ties below bit 29
    if (t % 4 == 2 && len > 12) q = (q >> 11 << 11) | (1ull << 10);       // ties at the 53-bit step
    const float want = (float)((double)q * 9.094947017729282379150390625e-13);
    const float got = fp_value40(q);
    if (std::memcmp(&want, &got, 4) != 0) { if (bad < 10) printf("value %llu %a %a\n", (unsigned long long)q, got, want); bad++; }
    n++;
  }
  printf("checked %ld bad %ld\n", n, bad);
  return bad != 0;
}
