/* ORACLE — test infrastructure only (see orc.h).
 * Gaussian field synthesis, restating Compute_Den (density_grid.c:71-217). */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

#define ORC_F64 (sizeof(real) == 8)
#define PHILOX_KEY1 0x45584853u   /* second key word of the GPU field stream */

/* Which half-complex mode is a Hermitian copy of another (the four copy
 * rules of density_grid.c:109-150).  Returns 1 and the source index. */
static int hermitian_source(const orc_params *p, int i, int j, int k, size_t *src) {
  int n0 = p->nd[0], n1 = p->nd[1], n2 = p->nd[2], nz2 = p->nz2;
  if (!((k == 0 || k == n2 / 2) && (i > n0 / 2 || j > n1 / 2))) return 0;
  int si, sj;
  if (i > n0 / 2 && j > n1 / 2) { si = n0 - i; sj = n1 - j; }
  else if (i == 0 || i == n0 / 2) { si = i; sj = n1 - j; }
  else if (j == 0 || j == n1 / 2) { si = n0 - i; sj = j; }
  else if (i > n0 / 2 && j < n1 / 2) { si = n0 - i; sj = n1 - j; }
  else return 0;                     /* 0 < i < n0/2, j > n1/2: drawn */
  *src = ((size_t)si * n1 + sj) * nz2 + k;
  return 1;
}

static int self_conjugate(const orc_params *p, int i, int j, int k) {
  return (i == 0 || i == p->nd[0] / 2) && (j == 0 || j == p->nd[1] / 2) &&
         (k == 0 || k == p->nd[2] / 2);
}

int orc_field_modes(const orc_params *p, const float *K, const float *P, int Nk,
                    int stream, int fixed, float phase, float k_smooth, real *deltak) {
  int n0 = p->nd[0], n1 = p->nd[1], n2 = p->nd[2], nz2 = p->nz2;
  double *Kd = (double *)malloc(sizeof(double) * Nk), *Pd = (double *)malloc(sizeof(double) * Nk);
  for (int i = 0; i < Nk; i++) { Kd[i] = K[i]; Pd[i] = P[i]; }   /* Inter_Power :47-50 */
  orc_spline sp;
  int st = orc_spline_init(&sp, Kd, Pd, Nk);
  free(Kd); free(Pd);
  if (st) return 1;
  orc_taus rng;
  orc_taus_seed(&rng, (unsigned long)p->seed);
  const uint32_t key[2] = {(uint32_t)p->seed, PHILOX_KEY1};
  int err = 0;

  for (int i = 0; i < n0; i++) {
    for (int j = 0; j < n1; j++) {
      for (int k = 0; k < nz2; k++) {
        size_t ind = ((size_t)i * n1 + j) * nz2 + k, src;
        if (hermitian_source(p, i, j, k, &src)) {
          deltak[2 * ind] = deltak[2 * src];
          deltak[2 * ind + 1] = -deltak[2 * src + 1];
          continue;
        }
        int ii = i < n0 / 2 ? i : i - n0;
        int jj = j < n1 / 2 ? j : j - n1;
        int kk = k;
        if (k == n2 / 2) kk = -(n2 / 2);
        double re, im, A;
        if (!ORC_F64) {
          /* reference float arithmetic (density_grid.c:95-105,152-166) */
          float kx = ii * p->kl[0], ky = jj * p->kl[1], kz = k * p->kl[2];
          if (k == n2 / 2) kz = (float)(-n2 / 2.0 * p->kl[2]);
          float kmod = (float)sqrt(kx * kx + ky * ky + kz * kz);
          float Af = 0.0f;
          if (kmod <= k_smooth && kmod > 0.0f) {
            double v = orc_spline_eval(&sp, (double)kmod, &st);
            if (st) err = 2;
            Af = (float)sqrt(v / 2.0);
          }
          A = Af;
        } else {
          double kx = ii * p->kl_d[0], ky = jj * p->kl_d[1], kz = kk * p->kl_d[2];
          double kmod = sqrt(kx * kx + ky * ky + kz * kz);
          A = 0.0;
          if (kmod <= k_smooth && kmod > 0.0) {
            double v = orc_spline_eval(&sp, kmod, &st);
            if (st) err = 2;
            A = sqrt(v / 2.0);
          }
        }
        if (stream == 0) {
          /* reference stream, density_grid.c:169-186 */
          float Af = (float)A;
          if (self_conjugate(p, i, j, k)) {
            re = fixed ? (float)(sqrt(2.0) * Af) : (float)(sqrt(2.0) * Af * ((float)orc_gaussian(&rng, 1.0)));
            im = 0.0;
          } else if (fixed) {
            float theta = (float)orc_flat(&rng, 0.0, 2.0 * M_PI);
            re = (float)(Af * cos(theta));
            im = (float)(Af * sin(theta));
          } else {
            float g1 = (float)orc_gaussian(&rng, 1.0);
            float g2 = (float)orc_gaussian(&rng, 1.0);
            re = Af * g1;
            im = Af * g2;
          }
          if (ORC_F64) { /* keep the FP64 amplitude, reference draws */
            if (Af != 0.0f) { re = re / Af * A; im = im / Af * A; }
          }
        } else {
          /* Philox stream: one 4x32 block per independent mode, keyed by
           * (seed, half-complex index).  u1 in (0,1), u2, u3 in [0,1). */
          uint32_t ctr[4] = {(uint32_t)ind, (uint32_t)(ind >> 32), 0u, 0u}, o[4];
          orc_philox4x32(ctr, key, o);
          double u1 = ((double)(o[0] >> 8) + 0.5) * (1.0 / 16777216.0);
          double u2 = (double)(o[1] >> 8) * (1.0 / 16777216.0);
          double u3 = (double)(o[2] >> 8) * (1.0 / 16777216.0);
          double rad = sqrt(-2.0 * log(u1));
          double g1 = rad * cos(2.0 * M_PI * u2), g2 = rad * sin(2.0 * M_PI * u2);
          if (self_conjugate(p, i, j, k)) {
            re = fixed ? sqrt(2.0) * A : sqrt(2.0) * A * g1;
            im = 0.0;
          } else if (fixed) {
            re = A * cos(2.0 * M_PI * u3);
            im = A * sin(2.0 * M_PI * u3);
          } else {
            re = A * g1;
            im = A * g2;
          }
        }
        if (phase != 0.0f) {
          /* density_grid.c:189-192: the second line reads the rotated real part */
          real r0 = (real)(re * cos(phase) - im * sin(phase));
          real i0 = (real)(r0 * sin(phase) + im * cos(phase));
          re = r0; im = i0;
        }
        deltak[2 * ind] = (real)re;
        deltak[2 * ind + 1] = (real)im;
      }
    }
  }
  orc_spline_free(&sp);
  return err;
}

int orc_field_real(const orc_params *p, const real *deltak, real *delta) {
  if (orc_fft_c2r_3d(p->nd[0], p->nd[1], p->nd[2], deltak, delta)) return 1;
  real nx = ORC_F64 ? (real)p->Normx_d : (real)p->Normx;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)p->ng; i++) delta[i] = delta[i] * nx;
  return 0;
}

/* Smoothing ladder (FP64 oracle of the build-added stage; the window is
 * exshalos_h.c:35-40, the barrier find_halos.c:200-212): for i from n_radii-1
 * down to 0, delta_R = c2r(delta_k W(k R_i)) Normx, and each cell keeps the
 * first i with delta_R >= B_i; 255 = never. */
int orc_ladder(const orc_params *p, const real *deltak, int n_radii, const float *R, const float *B,
               unsigned char *cross) {
  int n0 = p->nd[0], n1 = p->nd[1], n2 = p->nd[2], nz2 = p->nz2;
  size_t nk = (size_t)n0 * n1 * nz2, ng = p->ng;
  real *tmp = (real *)malloc(sizeof(real) * 2 * nk), *dr = (real *)malloc(sizeof(real) * ng);
  if (!tmp || !dr) { free(tmp); free(dr); return 1; }
  memset(cross, 255, ng);
  for (int r = n_radii - 1; r >= 0; r--) {
    double Rr = R[r];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n0; i++) {
      double kx = ((2 * i < n0) ? i : i - n0) * p->kl_d[0];
      for (int j = 0; j < n1; j++) {
        double ky = ((2 * j < n1) ? j : j - n1) * p->kl_d[1];
        for (int k = 0; k < nz2; k++) {
          double kz = ((k == n2 / 2) ? -(n2 / 2) : k) * p->kl_d[2];
          double x = sqrt(kx * kx + ky * ky + kz * kz) * Rr;
          double w = x > 0.0 ? 3.0 * (sin(x) - x * cos(x)) / (x * x * x) : 1.0;
          size_t id = ((size_t)i * n1 + j) * nz2 + k;
          tmp[2 * id] = (real)(deltak[2 * id] * w);
          tmp[2 * id + 1] = (real)(deltak[2 * id + 1] * w);
        }
      }
    }
    orc_fft_c2r_3d(n0, n1, n2, tmp, dr);
    double nx = ORC_F64 ? p->Normx_d : (double)p->Normx;
    for (size_t c = 0; c < ng; c++)
      if (cross[c] == 255 && (double)dr[c] * nx >= (double)B[r]) cross[c] = (unsigned char)r;
  }
  free(tmp); free(dr);
  return 0;
}
