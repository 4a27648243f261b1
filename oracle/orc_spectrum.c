/* ORACLE — test infrastructure only (see orc.h).
 * CIC density assignment and the shell-binned power spectrum, restating
 * src/spectrum/gridmodule.c:21-53,146-211, spectrum_h.c:4-167 and
 * powermodule.c:4-108 for one tracer type, l_max = 0, no interlacing. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

#define ORC_F64 (sizeof(real) == 8)

static inline int modi(int x, int y, int nd) {           /* spectrum_h.c:4-14 */
  int r = x + y;
  while (r >= nd) r -= nd;
  while (r < 0) r += nd;
  return r;
}
static inline real cysumf_w(real x, real y, real L) {    /* spectrum_h.c:17-27 */
  real r = x + y;
  while (r >= L) r -= L;
  while (r < 0.0) r += L;
  return r;
}

int orc_cic(const real *pos, size_t np, int nd, float L, real *grid) {
  size_t ng = (size_t)nd * nd * nd;
  memset(grid, 0, sizeof(real) * ng);
  real Ld = ORC_F64 ? (real)((double)L / nd) : (real)(L / nd);
  real Lr = (real)L;
  double M = 0.0;
  for (size_t p = 0; p < np; p++) {
    real x[3], dx[3], t[3];
    int xt[3], sg[3];
    for (int a = 0; a < 3; a++) {
      x[a] = cysumf_w(pos[3 * p + a], (real)0.0, Lr);
      xt[a] = (int)floor(x[a] / Ld);                       /* ind(), spectrum_h.c:73-80 */
      if (xt[a] == nd) xt[a] -= 1;
      dx[a] = (real)(x[a] / Ld - (xt[a] + 1.0 / 2.0));      /* gridmodule.c:30 */
      if (dx[a] >= 0.0) { sg[a] = 1; t[a] = (real)1.0 - dx[a]; }
      else { sg[a] = -1; dx[a] = -dx[a]; t[a] = (real)1.0 - dx[a]; }
    }
    int x1 = modi(xt[0], sg[0], nd), y1 = modi(xt[1], sg[1], nd), z1 = modi(xt[2], sg[2], nd);
    int x0 = xt[0], y0 = xt[1], z0 = xt[2];
#define G(a, b, c) grid[((size_t)(a) * nd + (b)) * nd + (c)]
    G(x0, y0, z0) += t[0] * t[1] * t[2];
    G(x1, y0, z0) += dx[0] * t[1] * t[2];
    G(x0, y1, z0) += t[0] * dx[1] * t[2];
    G(x0, y0, z1) += t[0] * t[1] * dx[2];
    G(x1, y1, z0) += dx[0] * dx[1] * t[2];
    G(x1, y0, z1) += dx[0] * t[1] * dx[2];
    G(x0, y1, z1) += t[0] * dx[1] * dx[2];
    G(x1, y1, z1) += dx[0] * dx[1] * dx[2];
#undef G
    M += 1.0;
  }
  double mean = M / (double)ng;                            /* gridmodule.c:206-211 */
  for (size_t i = 0; i < ng; i++) grid[i] = (real)(grid[i] / mean - 1.0);
  return 0;
}

static inline float sinc_f(float x) { return x != 0.0f ? (float)(sin(x) / x) : 1.0f; }
static inline double sinc_d(double x) { return x != 0.0 ? sin(x) / x : 1.0; }

int orc_power(const real *grid, int nd, float L, int window, int Nk, float kmin, float kmax,
              double *kmean, double *Pk, int64_t *count) {
  int nc = nd / 2 + 1;
  real *gk = (real *)malloc(sizeof(real) * 2 * (size_t)nd * nd * nc);
  if (!gk) return 1;
  if (orc_fft_r2c_3d(nd, nd, nd, grid, gk)) { free(gk); return 1; }
  float kn = (float)(2 * M_PI / L), Lb = L / nd;
  float Normk = (float)pow(L / (nd * nd), 3.0 / 2.0);       /* spectrum_h.c:90 */
  double kn_d = 2.0 * M_PI / (double)L, Lb_d = (double)L / nd;
  double Normk_d = pow((double)L / ((double)nd * nd), 1.5);
  float dk = (kmax - kmin) / Nk;                            /* powermodule.c:11 */
  for (int b = 0; b < Nk; b++) { kmean[b] = 0; Pk[b] = 0; count[b] = 0; }
  for (int i = 0; i < nd; i++) {
    float kx = (2 * i < nd) ? i * kn : (i - nd) * kn;
    for (int j = 0; j < nd; j++) {
      float ky = (2 * j < nd) ? j * kn : (j - nd) * kn;
      for (int k = 0; k < nc; k++) {
        float kz = (2 * k < nd) ? k * kn : (k - nd) * kn;
        /* mode-skip rule, powermodule.c:50-51 */
        if ((k == 0 || k == nd / 2) &&
            ((i > nd / 2 && j > nd / 2) || (i == 0 || i == nd / 2) || (j == 0 || j == nd / 2) ||
             (i > nd / 2 && j < nd / 2)))
          continue;
        float kmod = (float)sqrt(kx * kx + ky * ky + kz * kz);
        int b = (int)floor((kmod - kmin) / dk);             /* Indice, spectrum_h.c:39-48 */
        if (b < 0 || b >= Nk) continue;
        size_t id = ((size_t)i * nd + j) * nc + k;
        double pw;
        if (!ORC_F64) {
          float w = 1.0f;
          if (window == 1) w = sinc_f((float)(kx * Lb / 2.0)) * sinc_f((float)(ky * Lb / 2.0)) * sinc_f((float)(kz * Lb / 2.0));
          if (window == 2) w = (float)pow(sinc_f((float)(kx * Lb / 2.0)) * sinc_f((float)(ky * Lb / 2.0)) * sinc_f((float)(kz * Lb / 2.0)), 2.0);
          float re = (float)gk[2 * id] * Normk / w, im = (float)gk[2 * id + 1] * Normk / w;
          pw = (double)(re * re + im * im);
        } else {
          int ii = (2 * i < nd) ? i : i - nd, jj = (2 * j < nd) ? j : j - nd, kk = (2 * k < nd) ? k : k - nd;
          double qx = ii * kn_d, qy = jj * kn_d, qz = kk * kn_d, w = 1.0;
          if (window == 1) w = sinc_d(qx * Lb_d / 2) * sinc_d(qy * Lb_d / 2) * sinc_d(qz * Lb_d / 2);
          if (window == 2) { w = sinc_d(qx * Lb_d / 2) * sinc_d(qy * Lb_d / 2) * sinc_d(qz * Lb_d / 2); w = w * w; }
          double re = (double)gk[2 * id] * Normk_d / w, im = (double)gk[2 * id + 1] * Normk_d / w;
          pw = re * re + im * im;
        }
        Pk[b] += pw;
        kmean[b] += (double)kmod;
        count[b] += 1;
      }
    }
  }
  for (int b = 0; b < Nk; b++)
    if (count[b] > 0) { Pk[b] = Pk[b] / count[b]; kmean[b] = kmean[b] / count[b]; }
  free(gk);
  return 0;
}
