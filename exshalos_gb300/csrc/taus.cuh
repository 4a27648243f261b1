// The reference's sequential random stream on the GPU: gsl_rng_taus (the
// combined Tausworthe generator of L'Ecuyer, Math. Comp. 65 (1996) 203-213,
// with the LCG(69069) seeding documented for GSL) advanced to any position by
// GF(2) jump matrices, and the natural cubic spline evaluated on the device
// with the operation order of the host set-up.  Used where the reference
// draws from one taus stream in a fixed order: the halo masses
// (find_halos.c:455-476) and the galaxy population (populate_halos.c:142-205,
// split_galaxies.c:34-72).
#pragma once
#include <cstring>

#include "exh_common.cuh"

namespace exh {

// jump matrices: for component c and power 2^e, 32 column words
struct TausJump {
  unsigned col[3][32][32];   // [component][bit e][column]
};

struct TausState {
  unsigned s[3];
};

__host__ __device__ __forceinline__ unsigned taus_step1(unsigned s, int c) {
  if (c == 0) return ((s & 0xFFFFFFFEu) << 12) ^ (((s << 13) ^ s) >> 19);
  if (c == 1) return ((s & 0xFFFFFFF8u) << 4) ^ (((s << 2) ^ s) >> 25);
  return ((s & 0xFFFFFFF0u) << 17) ^ (((s << 3) ^ s) >> 11);
}

inline void taus_seed_state(unsigned long seed, unsigned s0[3]) {
  // the seeding documented for gsl_rng_taus: LCG(69069) chain, minimum
  // values 2, 8, 16, six warm-up steps
  unsigned s = (unsigned)(seed & 0xFFFFFFFFul);
  if (s == 0) s = 1;
  unsigned s1 = 69069u * s;
  if (s1 < 2u) s1 += 2u;
  unsigned s2 = 69069u * s1;
  if (s2 < 8u) s2 += 8u;
  unsigned s3 = 69069u * s2;
  if (s3 < 16u) s3 += 16u;
  for (int w = 0; w < 6; w++) { s1 = taus_step1(s1, 0); s2 = taus_step1(s2, 1); s3 = taus_step1(s3, 2); }
  s0[0] = s1; s0[1] = s2; s0[2] = s3;
}

// one step of each component is linear over GF(2); column b of the step
// matrix is the image of bit b.  Squaring gives the 2^e-step matrices.
inline void taus_jump_tables(TausJump* J) {
  for (int c = 0; c < 3; c++) {
    unsigned cur[32];
    for (int b = 0; b < 32; b++) cur[b] = taus_step1(1u << b, c);     // one step
    for (int e = 0; e < 32; e++) {
      std::memcpy(J->col[c][e], cur, sizeof(cur));
      unsigned nx[32];
      for (int b = 0; b < 32; b++) {                                   // square
        unsigned v = cur[b], acc = 0;
        for (int q = 0; q < 32; q++)
          if ((v >> q) & 1u) acc ^= cur[q];
        nx[b] = acc;
      }
      std::memcpy(cur, nx, sizeof(nx));
    }
  }
}

// the jump matrices, built once per process (thread-safe local static)
inline const TausJump& taus_jump_host() {
  static const TausJump J = [] { TausJump t; taus_jump_tables(&t); return t; }();
  return J;
}

__device__ __forceinline__ unsigned gf2_apply(const unsigned* __restrict__ col, unsigned s) {
  unsigned acc = 0;
#pragma unroll 8
  for (int q = 0; q < 32; q++)
    if ((s >> q) & 1u) acc ^= col[q];
  return acc;
}

// state after n further steps (n < 2^32 per call)
__device__ __forceinline__ void taus_jump(const TausJump* __restrict__ J, unsigned s[3], unsigned long long n) {
  for (int e = 0; e < 32; e++)
    if ((n >> e) & 1ull)
      for (int c = 0; c < 3; c++) s[c] = gf2_apply(J->col[c][e], s[c]);
}

// one gsl_rng_get: advance, then the XOR of the three components
__device__ __forceinline__ unsigned taus_next(unsigned s[3]) {
  s[0] = ((s[0] & 0xFFFFFFFEu) << 12) ^ (((s[0] << 13) ^ s[0]) >> 19);
  s[1] = ((s[1] & 0xFFFFFFF8u) << 4) ^ (((s[1] << 2) ^ s[1]) >> 25);
  s[2] = ((s[2] & 0xFFFFFFF0u) << 17) ^ (((s[2] << 3) ^ s[2]) >> 11);
  return s[0] ^ s[1] ^ s[2];
}

// gsl_rng_uniform of the taus generator: get / 2^32
__device__ __forceinline__ double taus_u01(unsigned x) { return (double)x / 4294967296.0; }

struct DevSpline {
  const double* x;
  const double* y;
  const double* c;
  int n;
  // natural cubic spline, the same operations and order as the host set-up
  __device__ double eval(double q, int* bad) const {
    if (!(q >= x[0] && q <= x[n - 1])) { *bad = 1; return 0.0; }
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
      const int mid = (hi + lo) >> 1;
      if (x[mid] > q) hi = mid; else lo = mid;
    }
    const double xl = x[lo], dx = __dsub_rn(x[lo + 1], xl), dy = __dsub_rn(y[lo + 1], y[lo]);
    const double c0 = c[lo], c1 = c[lo + 1];
    const double bb = __dsub_rn(__ddiv_rn(dy, dx), __ddiv_rn(__dmul_rn(dx, __dadd_rn(c1, __dmul_rn(2.0, c0))), 3.0));
    const double dd = __ddiv_rn(__dsub_rn(c1, c0), __dmul_rn(3.0, dx));
    const double t = __dsub_rn(q, xl);
    return __dadd_rn(y[lo], __dmul_rn(t, __dadd_rn(bb, __dmul_rn(t, __dadd_rn(c0, __dmul_rn(t, dd))))));
  }
};

// The same spline with the per-interval coefficients bb, dd formed once on
// the host (Spline::eval's expressions, the same double operations), so an
// evaluation is the knot search and the Horner steps only
struct DevSplineCoef {
  const double* x;
  const double* y;
  const double* c;
  const double* bb;
  const double* dd;
  int n;
  __device__ double eval(double q, int* bad) const {
    if (!(q >= x[0] && q <= x[n - 1])) { *bad = 1; return 0.0; }
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
      const int mid = (hi + lo) >> 1;
      if (x[mid] > q) hi = mid; else lo = mid;
    }
    const double t = __dsub_rn(q, x[lo]);
    return __dadd_rn(y[lo], __dmul_rn(t, __dadd_rn(bb[lo], __dmul_rn(t, __dadd_rn(c[lo], __dmul_rn(t, dd[lo]))))));
  }
};

}  // namespace exh
