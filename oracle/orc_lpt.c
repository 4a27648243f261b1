/* ORACLE — test infrastructure only (see orc.h).
 * Lagrangian perturbation theory displacements, restating
 * src/exshalos/lpt.c:4-255.  Written over `real`: the float build keeps the
 * reference's float storage with double stencil arithmetic; the double
 * build is the FP64 oracle.
 * Divergence kept on purpose: the reference's y-stencils index the -1
 * neighbour with nd[0] instead of nd[1] (lpt.c:66,123,127,192); the two are
 * the same cell for ndx == ndy, the only case the tests use.  The correct
 * index is used here. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

#define ORC_F64 (sizeof(real) == 8)

static inline int cysum(int i, int j, int nd) {
  int r = i + j;
  if (r >= nd) r -= nd;
  if (r < 0) r += nd;
  return r;
}

/* sixth-order central difference numerator along one axis (lpt.c:64-68) */
static inline double fd6(const real *f, size_t stride_in, int stride_pts, const orc_params *p,
                         int axis, int i, int j, int k) {
  (void)stride_in; (void)stride_pts;
  int n0 = p->nd[0], n1 = p->nd[1], n2 = p->nd[2];
  int c[3] = {i, j, k}, n[3] = {n0, n1, n2};
  double w[6] = {1.0, -9.0, 45.0, -45.0, 9.0, -1.0};
  int off[6] = {3, 2, 1, -1, -2, -3};
  double acc = 0.0;
  for (int t = 0; t < 6; t++) {
    int cc[3] = {c[0], c[1], c[2]};
    cc[axis] = cysum(c[axis], off[t], n[axis]);
    size_t id = ((size_t)cc[0] * n1 + cc[1]) * (size_t)n2 + cc[2];
    acc = acc + w[t] * (double)f[id * stride_in + stride_pts];
  }
  return acc;
}

/* k-space Poisson kernel (lpt.c:12-44 and :141-173): value /= -k^2 */
static void poisson_k(const orc_params *p, real *fk, float k_smooth, int times_normk) {
  int n0 = p->nd[0], n1 = p->nd[1], n2 = p->nd[2], nz2 = p->nz2;
  real kl0 = ORC_F64 ? (real)p->kl_d[0] : p->kl[0];
  real kl1 = ORC_F64 ? (real)p->kl_d[1] : p->kl[1];
  real kl2 = ORC_F64 ? (real)p->kl_d[2] : p->kl[2];
  real nk = ORC_F64 ? (real)p->Normk_d : p->Normk;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n0; i++) {
    real kx = (2 * i < n0) ? i * kl0 : (i - n0) * kl0;
    for (int j = 0; j < n1; j++) {
      real ky = (2 * j < n1) ? j * kl1 : (j - n1) * kl1;
      for (int k = 0; k < nz2; k++) {
        real kz = k * kl2;
        if (k == n2 / 2) kz = (real)(-(real)n2 / 2.0 * kl2);
        real kmod = (real)sqrt(pow(kx, 2.0) + pow(ky, 2.0) + pow(kz, 2.0));
        size_t ind = ((size_t)i * n1 + j) * nz2 + k;
        if ((kx != 0.0 || ky != 0.0 || kz != 0.0) && (kmod <= k_smooth)) {
          real fact = (real)(-pow(kmod, 2.0));
          if (times_normk) {
            fk[2 * ind] = fk[2 * ind] / fact * nk;
            fk[2 * ind + 1] = fk[2 * ind + 1] / fact * nk;
          } else {
            fk[2 * ind] = fk[2 * ind] / fact;
            fk[2 * ind + 1] = fk[2 * ind + 1] / fact;
          }
        } else {
          fk[2 * ind] = 0; fk[2 * ind + 1] = 0;
        }
      }
    }
  }
}

int orc_lpt1(const orc_params *p, real *deltak, const int64_t *flag, size_t nh, float k_smooth,
             real *S, real *posh) {
  (void)nh;
  int n0 = p->nd[0], n1 = p->nd[1], n2 = p->nd[2];
  size_t ng = p->ng;
  poisson_k(p, deltak, k_smooth, 0);
  real *phi = (real *)malloc(sizeof(real) * ng);
  if (!phi) return 1;
  if (orc_fft_c2r_3d(n0, n1, n2, deltak, phi)) { free(phi); return 1; }
  double fac = ORC_F64 ? p->Normx_d / (60.0 * p->Lc_d) : 0.0;
  /* S for every cell (lpt.c:82-86), then the halo sums in row-major order */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n0; i++)
    for (int j = 0; j < n1; j++)
      for (int k = 0; k < n2; k++) {
        size_t ind = ((size_t)i * n1 + j) * n2 + k;
        for (int a = 0; a < 3; a++) {
          double v = fd6(phi, 1, 0, p, a, i, j, k);
          real s = ORC_F64 ? (real)(-v * fac) : (real)(-(v) * p->Normx / (60.0 * p->Lc));
          if (S) S[3 * ind + a] = s;
        }
      }
  if (posh && flag) {
    for (size_t ind = 0; ind < ng; ind++) {
      int64_t f = flag[ind];
      size_t t = (size_t)(f < 0 ? -f : f);
      if (t >= ng) continue;
      for (int a = 0; a < 3; a++) posh[3 * t + a] += S[3 * ind + a];
    }
  }
  free(phi);
  return 0;
}

int orc_lpt2(const orc_params *p, real *S, const int64_t *flag, size_t nh, float k_smooth,
             int add_to_S, real *posh) {
  (void)nh;
  int n0 = p->nd[0], n1 = p->nd[1], n2 = p->nd[2], nz2 = p->nz2;
  size_t ng = p->ng;
  real *phi = (real *)malloc(sizeof(real) * ng);
  real *phik = (real *)malloc(sizeof(real) * 2 * (size_t)n0 * n1 * nz2);
  if (!phi || !phik) { free(phi); free(phik); return 1; }
  double l60 = ORC_F64 ? 60.0 * p->Lc_d : 60.0 * p->Lc;
  /* second-order source, lpt.c:116-134 */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n0; i++)
    for (int j = 0; j < n1; j++)
      for (int k = 0; k < n2; k++) {
        size_t ind = ((size_t)i * n1 + j) * n2 + k;
        real pxx = (real)(fd6(S, 3, 0, p, 0, i, j, k) / l60);
        real pxy = (real)(fd6(S, 3, 0, p, 1, i, j, k) / l60);
        real pxz = (real)(fd6(S, 3, 0, p, 2, i, j, k) / l60);
        real pyy = (real)(fd6(S, 3, 1, p, 1, i, j, k) / l60);
        real pyz = (real)(fd6(S, 3, 1, p, 2, i, j, k) / l60);
        real pzz = (real)(fd6(S, 3, 2, p, 2, i, j, k) / l60);
        phi[ind] = (real)(pxx * pyy + pxx * pzz + pyy * pzz - pow(pxy, 2.0) - pow(pxz, 2.0) - pow(pyz, 2.0));
      }
  if (orc_fft_r2c_3d(n0, n1, n2, phi, phik)) { free(phi); free(phik); return 1; }
  poisson_k(p, phik, k_smooth, 1);
  if (orc_fft_c2r_3d(n0, n1, n2, phik, phi)) { free(phi); free(phik); return 1; }
  free(phik);
  double nxf = ORC_F64 ? p->Normx_d / (60.0 * p->Lc_d) : 0.0;
  double omz = ORC_F64 ? p->Omz_d : (double)p->Omz;
  double c2 = -3.0 / 7.0 * pow(omz, -1.0 / 143);
  real *S2 = (real *)malloc(sizeof(real) * 3 * ng);
  if (!S2) { free(phi); return 1; }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n0; i++)
    for (int j = 0; j < n1; j++)
      for (int k = 0; k < n2; k++) {
        size_t ind = ((size_t)i * n1 + j) * n2 + k;
        for (int a = 0; a < 3; a++) {
          double v = fd6(phi, 1, 0, p, a, i, j, k);
          real s = ORC_F64 ? (real)(v * nxf) : (real)(v * p->Normx / (60.0 * p->Lc));
          S2[3 * ind + a] = (real)(c2 * s);
        }
      }
  for (size_t ind = 0; ind < ng; ind++) {
    if (posh && flag) {
      int64_t f = flag[ind];
      size_t t = (size_t)(f < 0 ? -f : f);
      if (t < ng)
        for (int a = 0; a < 3; a++) posh[3 * t + a] += S2[3 * ind + a];
    }
    if (add_to_S)
      for (int a = 0; a < 3; a++) S[3 * ind + a] += S2[3 * ind + a];
  }
  free(S2); free(phi);
  return 0;
}

/* cysumf of exshalos_h.c:13-19 (one correction each way) */
static inline real cysumf(real x, real y, real L) {
  real r = x + y;
  if (r >= L) r -= L;
  if (r < 0) r += L;
  return r;
}

void orc_posh(const orc_params *p, size_t nh, const int *hx, const int *hcount, real *posh) {
  for (size_t i = 0; i < nh; i++)
    for (int j = 0; j < 3; j++) {
      real lc = ORC_F64 ? (real)p->Lc_d : p->Lc;
      real Lj = ORC_F64 ? (real)p->L_d[j] : p->L[j];
      real x = (real)(hx[3 * i + j] * lc + lc / 2.0);
      posh[3 * i + j] = cysumf(x, posh[3 * i + j] / hcount[i], Lj);
    }
}

void orc_pos(const orc_params *p, real *S) {
  real lc = ORC_F64 ? (real)p->Lc_d : p->Lc;
  for (int i = 0; i < p->nd[0]; i++)
    for (int j = 0; j < p->nd[1]; j++)
      for (int k = 0; k < p->nd[2]; k++) {
        size_t ind = ((size_t)i * p->nd[1] + j) * p->nd[2] + k;
        int c[3] = {i, j, k};
        for (int a = 0; a < 3; a++) {
          real La = ORC_F64 ? (real)p->L_d[a] : p->L[a];
          S[3 * ind + a] = cysumf((real)(c[a] * lc + lc / 2.0), S[3 * ind + a], La);
        }
      }
}
