// Host check of the FP32 restatements in exshalos_gb300/csrc/fp32sum.cuh
// against FP64 (run by tests/test_fixedpoint.py; compiled without FMA
// contraction so that every float operation rounds as on the device).
#include <cmath>
#include <cstdio>
#include <random>
#include "fp32sum.cuh"

int main() {
  using namespace exh;
  long bad = 0;
  // source_combine against (float)((double)diag - x^2 - y^2 - z^2): at most
  // one float ulp apart, and rarely (double-rounding boundaries)
  std::mt19937 g(3);
  std::normal_distribution<float> nd(0.f, 1.f);
  long n = 0, differ = 0;
  for (long t = 0; t < 20000000; t++) {
    float x = nd(g), y = nd(g), z = nd(g), a = nd(g), b = nd(g), c = nd(g);
    if (t % 3 == 0) { a = x; b = y; }                 // heavy cancellation
    if (t % 7 == 0) { x *= 1e-3f; a *= 1e3f; }       // terms of very different size
    const float diag = a * b + a * c + b * c;
    const float want = (float)((double)diag - (double)x * x - (double)y * y - (double)z * z);
    const float got = source_combine(diag, x, y, z);
    n++;
    if (got != want) {
      differ++;
      if (std::fabs((double)got - want) > std::fabs((double)std::nextafter(want, INFINITY) - want) * 1.0000001) {
        if (bad < 5) printf("source %a %a %a %a: %a vs %a\n", diag, x, y, z, got, want);
        bad++;
      }
    }
  }
  if (differ * 1e5 > n) { printf("source: %ld of %ld differ\n", differ, n); bad++; }
  // FSum against the exact sum (long double holds these sums exactly enough):
  // |value - exact| <= 2^-23 |exact| + 2^-44 sum |x|
  std::uniform_real_distribution<double> ud(-1.0, 1.0);
  std::uniform_int_distribution<int> ln(1, 96), ex(-20, 20);
  for (long t = 0; t < 2000000; t++) {
    const int len = ln(g);
    FSum s;
    long double exact = 0.0L, mag = 0.0L;
    for (int i = 0; i < len; i++) {
      const float v = (float)std::ldexp(ud(g), (t % 5 == 0) ? ex(g) : 0);
      s.add(v);
      exact += (long double)v;
      mag += std::fabs((long double)v);
    }
    const long double err = std::fabs((long double)s.value() - exact);
    if (err > std::ldexp((long double)std::fabs(exact), -23) + std::ldexp(mag, -44)) {
      if (bad < 10) printf("fsum len %d err %Lg exact %Lg\n", len, err, exact);
      bad++;
    }
  }
  printf("source cases %ld differ %ld; bad %ld\n", n, differ, bad);
  return bad != 0;
}
