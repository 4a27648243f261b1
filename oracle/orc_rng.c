/* ORACLE — test infrastructure only (see orc.h).
 * Random streams used by the reference and by the GPU path. */
#include <math.h>
#include "orc.h"

/* Combined Tausworthe generator of L'Ecuyer, "Maximally equidistributed
 * combined Tausworthe generators", Math. Comp. 65 (1996) 203-213, three
 * components with (k,q,s) = (31,13,12), (29,2,4), (28,3,17).  The reference
 * allocates it as gsl_rng_taus (density_grid.c:90, find_halos.c:465). */
static inline uint32_t taus_component(uint32_t s, int q, int r, uint32_t mask, int sh) {
  return ((s & mask) << sh) ^ (((s << q) ^ s) >> r);
}

uint32_t orc_taus_get(orc_taus *t) {
  t->s1 = taus_component(t->s1, 13, 19, 0xFFFFFFFEu, 12);
  t->s2 = taus_component(t->s2, 2, 25, 0xFFFFFFF8u, 4);
  t->s3 = taus_component(t->s3, 3, 11, 0xFFFFFFF0u, 17);
  return t->s1 ^ t->s2 ^ t->s3;
}

/* Seeding as documented for gsl_rng_taus: each component comes from the
 * previous one through the LCG x -> 69069 x mod 2^32, is raised above its
 * minimum (2, 8, 16: the low bits a component discards), then six outputs
 * are discarded.  A zero seed is replaced by 1. */
void orc_taus_seed(orc_taus *t, unsigned long seed) {
  uint32_t s = (uint32_t)(seed & 0xFFFFFFFFul);
  if (s == 0) s = 1;
  t->s1 = 69069u * s;
  if (t->s1 < 2u) t->s1 += 2u;
  t->s2 = 69069u * t->s1;
  if (t->s2 < 8u) t->s2 += 8u;
  t->s3 = 69069u * t->s2;
  if (t->s3 < 16u) t->s3 += 16u;
  for (int i = 0; i < 6; i++) (void)orc_taus_get(t);
}

void orc_taus_state(const orc_taus *t, uint32_t out[3]) {
  out[0] = t->s1; out[1] = t->s2; out[2] = t->s3;
}

double orc_taus_uniform(orc_taus *t) { return orc_taus_get(t) / 4294967296.0; }

double orc_taus_uniform_pos(orc_taus *t) {
  double x;
  do { x = orc_taus_uniform(t); } while (x == 0.0);
  return x;
}

/* Marsaglia polar method (Knuth TAOCP vol. 2, Algorithm 3.4.1 P): a point in
 * the unit disc from two uniforms, then y * sqrt(-2 ln r2 / r2).  One normal
 * deviate per accepted pair, as gsl_ran_gaussian returns. */
double orc_gaussian(orc_taus *t, double sigma) {
  double x, y, r2;
  do {
    x = -1.0 + 2.0 * orc_taus_uniform_pos(t);
    y = -1.0 + 2.0 * orc_taus_uniform_pos(t);
    r2 = x * x + y * y;
  } while (r2 > 1.0 || r2 == 0.0);
  return sigma * y * sqrt(-2.0 * log(r2) / r2);
}

double orc_flat(orc_taus *t, double a, double b) {
  double u = orc_taus_uniform(t);
  return a * (1.0 - u) + b * u;
}

/* Philox4x32 with 10 rounds (Salmon, Moraes, Dror, Shaw, "Parallel random
 * numbers: as easy as 1, 2, 3", SC'11).  The GPU field synthesiser keys one
 * call per Fourier mode. */
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
