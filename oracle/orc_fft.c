/* ORACLE — test infrastructure only (see orc.h).
 * CPU FFT standing in for FFTW3 (fftwf_plan_dft_r2c_3d / _c2r_3d, used at
 * density_grid.c:208,225, lpt.c:50,112-113, spectrum_h.c:103-107).
 * Mixed-radix Stockham autosort (radices 4,2,3,5, generic odd prime) in the
 * build's precision with twiddles evaluated in double.  Conventions as
 * FFTW: forward sign -1, no normalisation, half-complex last axis. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "orc.h"

typedef struct { int n, nf, f[32]; real *tw; } plan1d;  /* tw: cos,sin of 2 pi k/n */

static int g_threads = 1;
void orc_set_threads(int n) {
  g_threads = n > 0 ? n : 1;
#ifdef _OPENMP
  omp_set_num_threads(g_threads);
#endif
}
int orc_get_threads(void) { return g_threads; }

static int plan_make(plan1d *p, int n) {
  p->n = n; p->nf = 0;
  int m = n;
  while (m % 4 == 0) { p->f[p->nf++] = 4; m /= 4; }
  while (m % 2 == 0) { p->f[p->nf++] = 2; m /= 2; }
  for (int q = 3; m > 1; q += 2)
    while (m % q == 0) { p->f[p->nf++] = q; m /= q; }
  p->tw = (real *)malloc(sizeof(real) * 2 * (size_t)n);
  if (!p->tw) return 1;
  for (int k = 0; k < n; k++) {
    double a = 2.0 * M_PI * (double)k / (double)n;
    p->tw[2 * k] = (real)cos(a);
    p->tw[2 * k + 1] = (real)sin(a);
  }
  return 0;
}
static void plan_free(plan1d *p) { free(p->tw); p->tw = NULL; }

/* one transform of length n: x -> x (uses scratch y of 2n reals) */
static void fft1d(const plan1d *p, real *x, real *y, int sign) {
  int n = p->n, Ns = 1;
  real *a = x, *b = y;
  real vr[64], vi[64], orr[64], oi[64];
  for (int s = 0; s < p->nf; s++) {
    int R = p->f[s], stride = n / R, step = n / (Ns * R);
    for (int j = 0; j < n / R; j++) {
      int k = j % Ns;
      for (int r = 0; r < R; r++) {
        real xr = a[2 * (j + r * stride)], xi = a[2 * (j + r * stride) + 1];
        int ti = (int)(((long)r * k * step) % n);
        real c = p->tw[2 * ti], sn = sign * p->tw[2 * ti + 1];
        vr[r] = xr * c - xi * sn;
        vi[r] = xr * sn + xi * c;
      }
      if (R == 2) {
        orr[0] = vr[0] + vr[1]; oi[0] = vi[0] + vi[1];
        orr[1] = vr[0] - vr[1]; oi[1] = vi[0] - vi[1];
      } else if (R == 4) {
        real t0r = vr[0] + vr[2], t0i = vi[0] + vi[2];
        real t1r = vr[0] - vr[2], t1i = vi[0] - vi[2];
        real t2r = vr[1] + vr[3], t2i = vi[1] + vi[3];
        real t3r = vr[1] - vr[3], t3i = vi[1] - vi[3];
        /* multiply t3 by sign*i */
        real ur = -sign * t3i, ui = sign * t3r;
        orr[0] = t0r + t2r; oi[0] = t0i + t2i;
        orr[2] = t0r - t2r; oi[2] = t0i - t2i;
        orr[1] = t1r + ur;  oi[1] = t1i + ui;
        orr[3] = t1r - ur;  oi[3] = t1i - ui;
      } else {
        for (int q = 0; q < R; q++) {
          double sr = 0, si = 0;
          for (int r = 0; r < R; r++) {
            int ti = (int)(((long)r * q % R) * (n / R));
            double c = p->tw[2 * ti], sn = sign * p->tw[2 * ti + 1];
            sr += vr[r] * c - vi[r] * sn;
            si += vr[r] * sn + vi[r] * c;
          }
          orr[q] = (real)sr; oi[q] = (real)si;
        }
      }
      int d = (j / Ns) * Ns * R + k;
      for (int r = 0; r < R; r++) { b[2 * (d + r * Ns)] = orr[r]; b[2 * (d + r * Ns) + 1] = oi[r]; }
    }
    Ns *= R;
    real *t = a; a = b; b = t;
  }
  if (a != x) memcpy(x, a, sizeof(real) * 2 * (size_t)n);
}

int orc_fft_c2c_1d(int n, real *data, int sign) {
  plan1d p;
  if (plan_make(&p, n)) return 1;
  real *y = (real *)malloc(sizeof(real) * 2 * (size_t)n);
  fft1d(&p, data, y, sign);
  free(y); plan_free(&p);
  return 0;
}

/* transform along axis y and x of a [nx][ny][nc] complex array */
static void fft_yx(int nx, int ny, int nc, real *a, int sign) {
  plan1d py, px;
  plan_make(&py, ny); plan_make(&px, nx);
#pragma omp parallel
  {
    int mx = nx > ny ? nx : ny;
    real *buf = (real *)malloc(sizeof(real) * 2 * (size_t)mx);
    real *scr = (real *)malloc(sizeof(real) * 2 * (size_t)mx);
#pragma omp for schedule(static)
    for (long t = 0; t < (long)nx * nc; t++) {
      int i = (int)(t / nc), k = (int)(t % nc);
      for (int j = 0; j < ny; j++) {
        size_t id = ((size_t)i * ny + j) * nc + k;
        buf[2 * j] = a[2 * id]; buf[2 * j + 1] = a[2 * id + 1];
      }
      fft1d(&py, buf, scr, sign);
      for (int j = 0; j < ny; j++) {
        size_t id = ((size_t)i * ny + j) * nc + k;
        a[2 * id] = buf[2 * j]; a[2 * id + 1] = buf[2 * j + 1];
      }
    }
#pragma omp for schedule(static)
    for (long t = 0; t < (long)ny * nc; t++) {
      int j = (int)(t / nc), k = (int)(t % nc);
      for (int i = 0; i < nx; i++) {
        size_t id = ((size_t)i * ny + j) * nc + k;
        buf[2 * i] = a[2 * id]; buf[2 * i + 1] = a[2 * id + 1];
      }
      fft1d(&px, buf, scr, sign);
      for (int i = 0; i < nx; i++) {
        size_t id = ((size_t)i * ny + j) * nc + k;
        a[2 * id] = buf[2 * i]; a[2 * id + 1] = buf[2 * i + 1];
      }
    }
    free(buf); free(scr);
  }
  plan_free(&py); plan_free(&px);
}

int orc_fft_r2c_3d(int nx, int ny, int nz, const real *in, real *out) {
  int nc = nz / 2 + 1;
  plan1d pz;
  if (plan_make(&pz, nz)) return 1;
#pragma omp parallel
  {
    real *buf = (real *)malloc(sizeof(real) * 2 * (size_t)nz);
    real *scr = (real *)malloc(sizeof(real) * 2 * (size_t)nz);
#pragma omp for schedule(static)
    for (long r = 0; r < (long)nx * ny; r++) {
      const real *row = in + (size_t)r * nz;
      for (int k = 0; k < nz; k++) { buf[2 * k] = row[k]; buf[2 * k + 1] = 0; }
      fft1d(&pz, buf, scr, -1);
      memcpy(out + (size_t)r * nc * 2, buf, sizeof(real) * 2 * (size_t)nc);
    }
    free(buf); free(scr);
  }
  plan_free(&pz);
  fft_yx(nx, ny, nc, out, -1);
  return 0;
}

/* c2r: the input is left unchanged (the reference's FFTW c2r may overwrite
 * its input; callers here never rely on it either way). */
int orc_fft_c2r_3d(int nx, int ny, int nz, const real *in, real *out) {
  int nc = nz / 2 + 1;
  size_t nk = (size_t)nx * ny * nc;
  real *tmp = (real *)malloc(sizeof(real) * 2 * nk);
  if (!tmp) return 1;
  memcpy(tmp, in, sizeof(real) * 2 * nk);
  fft_yx(nx, ny, nc, tmp, +1);
  plan1d pz;
  plan_make(&pz, nz);
#pragma omp parallel
  {
    real *buf = (real *)malloc(sizeof(real) * 2 * (size_t)nz);
    real *scr = (real *)malloc(sizeof(real) * 2 * (size_t)nz);
#pragma omp for schedule(static)
    for (long r = 0; r < (long)nx * ny; r++) {
      const real *h = tmp + (size_t)r * nc * 2;
      for (int k = 0; k < nc; k++) { buf[2 * k] = h[2 * k]; buf[2 * k + 1] = h[2 * k + 1]; }
      buf[1] = 0;                                  /* self-conjugate bins carry no */
      if (nz % 2 == 0) buf[2 * (nz / 2) + 1] = 0;  /* imaginary part in a c2r     */
      for (int k = nc; k < nz; k++) { buf[2 * k] = h[2 * (nz - k)]; buf[2 * k + 1] = -h[2 * (nz - k) + 1]; }
      fft1d(&pz, buf, scr, +1);
      real *o = out + (size_t)r * nz;
      for (int k = 0; k < nz; k++) o[k] = buf[2 * k];
    }
    free(buf); free(scr);
  }
  plan_free(&pz);
  free(tmp);
  return 0;
}
