// Host check of exshalos_gb300/csrc/taus_chunk.h (run by
// tests/test_fixedpoint.py; compiled without FMA contraction, as the
// reference's x86-64 GSL computes r2):
//  1. the acceptance test against r2 = x*x + y*y formed in double, on random
//     pairs and on pairs within a few units of 2^62 r2 = 2^62, where the
//     rounding of the double sum decides;
//  2. the chunked walk (counts per chunk, parity from the zeros before each
//     chunk, prefix sums, pairs per chunk) against the sequential polar
//     method (gsl_rng_uniform_pos skipping zeros, redraw while r2 > 1 or
//     r2 == 0) on streams with planted zeros, zero runs, near-circle pairs
//     and zeros at chunk boundaries.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>
#include "taus_chunk.h"

static bool direct_accept(unsigned v1, unsigned v2) {
  const double x = -1.0 + 2.0 * (v1 / 4294967296.0), y = -1.0 + 2.0 * (v2 / 4294967296.0);
  const double r2 = x * x + y * y;
  return !(r2 > 1.0 || r2 == 0.0);
}

static double direct_deviate(unsigned v1, unsigned v2) {
  const double x = -1.0 + 2.0 * (v1 / 4294967296.0), y = -1.0 + 2.0 * (v2 / 4294967296.0);
  const double r2 = x * x + y * y;
  return 1.0 * y * sqrt(-2.0 * log(r2) / r2);
}

// ln(c_i) and 1 / c_i of the table points c_i = 0.75 + (i + 1/2) / 256 as
// float pairs, as the library builds them
static void tables(float* lnc, float* invc) {
  for (int i = 0; i < 192; i++) {
    const double c = 0.75 + (i + 0.5) / 256.0;
    const double l = log(c), r = 1.0 / c;
    lnc[2 * i] = (float)l;
    lnc[2 * i + 1] = (float)(l - (double)lnc[2 * i]);
    invc[2 * i] = (float)r;
    invc[2 * i + 1] = (float)(r - (double)invc[2 * i]);
  }
}

// 3. the float-only deviate: whenever it decides, it is the float of the
// FP64 deviate; its double-float value is within 2^-42 of that deviate
static long check_f32_deviates(std::mt19937_64& g, long* undecided_out, double* worst_out) {
  float lnc[384], invc[384];
  tables(lnc, invc);
  long bad = 0, undecided = 0;
  double worst = 0.0;
  auto one = [&](unsigned v1, unsigned v2) {
    if (v1 == 0u || v2 == 0u || !direct_accept(v1, v2)) return;
    const double gd = direct_deviate(v1, v2);
    int und = 0;
    const float f = exh::polar_deviate_f32(v1, v2, lnc, invc, &und);
    const long long a = (long long)v1 - 2147483648LL, b = (long long)v2 - 2147483648LL;
    const unsigned long long S = (unsigned long long)(a * a) + (unsigned long long)(b * b);
    if (gd != 0.0 && S <= (1ull << 62) - (1ull << 50) && S >= (1ull << 20)) {      // where the double-float value is used
      const exh::DFloat df = exh::polar_deviate_df(v1, v2, lnc, invc);
      const double rel = std::fabs(((double)df.hi + (double)df.lo) - gd) / std::fabs(gd);
      if (rel > worst) worst = rel;
    }
    if (und) { undecided++; return; }
    if (f != (float)gd || std::signbit(f) != std::signbit((float)gd)) {
      if (bad < 5) printf("f32 deviate %08x %08x: %a vs %a\n", v1, v2, f, (float)gd);
      bad++;
    }
  };
  for (long t = 0; t < 12000000; t++) one((unsigned)g(), (unsigned)g());
  printf("random pairs: %ld of ~%ld deviates undecided\n", undecided, (long)(12000000 * 0.785));
  // r2 close to 1 (y small and x near +-1; the no-table path and its edge),
  // r2 tiny, y tiny
  for (long t = 0; t < 3000000; t++) {
    const unsigned r = (unsigned)g();
    const long long a = 2147483647LL - (long long)(g() % (1ull << (1 + t % 30)));
    const long long b = (long long)(g() % (1ull << (1 + (t / 7) % 31))) * (r & 1 ? 1 : -1);
    one((unsigned)((r & 2 ? a : -a) + 2147483648LL), (unsigned)(b + 2147483648LL));
    one((unsigned)((long long)(g() % 64) - 32 + 2147483648LL), (unsigned)((long long)(g() % 64) - 32 + 2147483648LL));
  }
  one(0xFFFFFFFFu, 0x80010000u);          // r2 rounds to 1: -0
  *undecided_out = undecided;
  *worst_out = worst;
  return bad;
}

int main() {
  long bad = 0;
  std::mt19937_64 g(11);
  // 1. acceptance
  long near = 0;
  for (long t = 0; t < 8000000; t++) {
    unsigned v1 = (unsigned)g(), v2 = (unsigned)g();
    if (t % 4 == 0) {                 // near the unit circle: a^2 + b^2 close to 2^62
      const double th = (g() >> 11) * (1.0 / 9007199254740992.0) * 1.5707963267948966;
      long long a = (long long)llround(2147483648.0 * cos(th)), b = (long long)llround(2147483648.0 * sin(th));
      a += (long long)(g() % 5) - 2;
      b += (long long)(g() % 5) - 2;
      if (a > 2147483647LL) a = 2147483647LL;
      if (b > 2147483647LL) b = 2147483647LL;
      v1 = (unsigned)(a + 2147483648LL);
      v2 = (unsigned)(b + 2147483648LL);
    }
    if (v1 == 0u || v2 == 0u) continue;
    const long long a = (long long)v1 - 2147483648LL, b = (long long)v2 - 2147483648LL;
    const unsigned long long s = (unsigned long long)(a * a) + (unsigned long long)(b * b);
    if (s + 4096ull >= (1ull << 62) && s <= (1ull << 62) + 4096ull) near++;
    if (exh::polar_accept(v1, v2) != direct_accept(v1, v2)) {
      if (bad < 5) printf("accept %08x %08x\n", v1, v2);
      bad++;
    }
    // r2 of the integer roundings against the double sum
    const double x = -1.0 + 2.0 * (v1 / 4294967296.0), y = -1.0 + 2.0 * (v2 / 4294967296.0);
    const double r2 = x * x + y * y;
    unsigned long long rb;
    __builtin_memcpy(&rb, &r2, 8);
    if (r2 != 0.0 && exh::r2_bits(v1, v2) != rb) {
      if (bad < 5) printf("r2 bits %08x %08x\n", v1, v2);
      bad++;
    }
  }
  // lattice pairs inside the band: a close to 2^31, b = the nearest integers to sqrt(2^62 - a^2)
  for (long long a = 2147483647LL; a > 2147483647LL - 200000; a--) {
    const long long b0 = (long long)sqrtl((long double)(1ull << 62) - (long double)(a * a));
    for (long long b = b0 - 2; b <= b0 + 2; b++) {
      if (b <= 0 || b > 2147483647LL) continue;
      const unsigned long long s = (unsigned long long)(a * a) + (unsigned long long)(b * b);
      if (s + 4096ull < (1ull << 62) || s > (1ull << 62) + 4096ull) continue;
      near++;
      for (int sg = 0; sg < 4; sg++) {
        const unsigned v1 = (unsigned)((sg & 1 ? -a : a) + 2147483648LL), v2 = (unsigned)((sg & 2 ? -b : b) + 2147483648LL);
        if (exh::polar_accept(v1, v2) != direct_accept(v1, v2) || exh::polar_accept(v2, v1) != direct_accept(v2, v1)) {
          if (bad < 5) printf("band %08x %08x\n", v1, v2);
          bad++;
        }
      }
    }
  }
  // the constructed case where the double sum rounds to 1 although 2^62 r2 = 2^62 + 1
  if (!exh::polar_accept(0xFFFFFFFFu, 0x80010000u) || !direct_accept(0xFFFFFFFFu, 0x80010000u)) bad++;
  printf("acceptance: %ld pairs in the rounding band\n", near);
  // 2. chunked walk against the sequential method
  auto logf64 = [](double r) { return log(r); };
  for (int trial = 0; trial < 40; trial++) {
    const int n = 2 * (1 + trial % 9);           // chunk sizes 2..18
    std::vector<unsigned> st(20000);
    for (auto& v : st) v = (unsigned)g();
    for (size_t i = 0; i < st.size(); i++) {
      const unsigned r = (unsigned)(g() % 1000);
      if (r < 20) st[i] = 0u;                    // isolated zeros
      else if (r < 23 && i + 3 < st.size()) st[i] = st[i + 1] = st[i + 2] = 0u;   // zero runs
      else if (r < 30 && i + 1 < st.size()) { st[i] = 0xFFFFFFFFu; st[i + 1] = 0x80010000u; }
    }
    for (size_t i = n; i < st.size(); i += 5 * n) st[i - 1] = 0u;   // zeros at chunk ends
    // sequential
    std::vector<double> want;
    {
      size_t p = 0;
      auto upos = [&](unsigned& v) {
        do { if (p >= st.size()) return false; v = st[p++]; } while (v == 0u);
        return true;
      };
      while (true) {
        unsigned v1, v2;
        bool ok = true;
        do {
          if (!upos(v1) || !upos(v2)) { ok = false; break; }
        } while (!direct_accept(v1, v2));
        if (!ok) break;
        want.push_back(direct_deviate(v1, v2));
      }
    }
    // chunked: only whole chunks whose lookahead stays inside the stream
    const int nch = (int)(st.size() / n) - 8;
    std::vector<unsigned> z(nch), a0(nch), a1(nch);
    for (int c = 0; c < nch; c++) {
      size_t p = (size_t)c * n;
      auto next = [&]() { return st[p++]; };
      exh::polar_chunk_count(next, n, &z[c], &a0[c], &a1[c]);
    }
    std::vector<double> got;
    unsigned zb = 0;
    for (int c = 0; c < nch; c++) {
      const unsigned par = zb & 1u;
      size_t p = (size_t)c * n;
      auto next = [&]() { return st[p++]; };
      size_t before = got.size();
      auto emit = [&](unsigned v1, unsigned v2) { got.push_back(exh::polar_deviate(v1, v2, logf64)); return true; };
      exh::polar_chunk_pairs(next, n, par, emit);
      if (got.size() - before != (par ? a1[c] : a0[c])) {
        if (bad < 5) printf("trial %d chunk %d: count %zu vs %u\n", trial, c, got.size() - before, par ? a1[c] : a0[c]);
        bad++;
      }
      zb += z[c];
    }
    for (size_t i = 0; i < got.size(); i++)
      if (i >= want.size() || got[i] != want[i]) {
        if (bad < 5) printf("trial %d deviate %zu: %a vs %a\n", trial, i, got[i], i < want.size() ? want[i] : 0.0);
        bad++;
        break;
      }
    if (got.size() + 64 < want.size() / 2) bad++;
  }
  long undecided = 0;
  double worst = 0.0;
  bad += check_f32_deviates(g, &undecided, &worst);
  printf("float deviates: %ld undecided, largest relative error of the double-float value %.3g\n", undecided,
         worst);
  // the decision margin is 2^-36: keep the observed error 8x inside it
  if (!(worst < std::ldexp(1.0, -39))) bad++;
  printf("bad %ld\n", bad);
  return bad != 0;
}
