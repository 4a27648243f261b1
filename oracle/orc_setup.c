/* ORACLE — test infrastructure only (see orc.h).
 * Box/cosmology parameters and the halo-finder tables, restated from
 * src/exshalos/exshalos_h.c and src/exshalos/find_halos.c with the
 * reference's float/double types kept expression by expression. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

#define ORC_M_MAX 1e+16     /* exshalos_h.h:47 */
#define ORC_LC_MAX 1.0e+2   /* exshalos_h.h:45 */

/* set_cosmology, exshalos_h.c:43-57 */
void orc_set_cosmology(orc_params *p, float Om0, float redshift, float dc) {
  p->Om0 = Om0;
  p->redshift = redshift;
  p->rhoc = 2.775e+11f;
  p->Hz = (float)(100.0 * sqrt(p->Om0 * pow(1.0 + p->redshift, 3.0) + (1.0 - p->Om0)));
  p->Omz = (float)(p->Om0 * pow(1.0 + p->redshift, 3.0) /
                   (p->Om0 * pow(1.0 + p->redshift, 3.0) + (1.0 - p->Om0)));
  p->rhomz = p->Om0 * p->rhoc;
  p->Dv = (float)((18 * M_PI * M_PI + 82.0 * (p->Omz - 1.0) - 39.0 * pow(p->Omz - 1.0, 2.0)) / p->Omz);
  if (dc <= 0.0f) p->dc = (float)(1.686 * pow(p->Omz, 0.0055));
  else p->dc = dc;
  double a3 = pow(1.0 + (double)redshift, 3.0);
  p->Hz_d = 100.0 * sqrt((double)Om0 * a3 + (1.0 - (double)Om0));
  p->Omz_d = (double)Om0 * a3 / ((double)Om0 * a3 + (1.0 - (double)Om0));
}

/* set_box, exshalos_h.c:69-106.  Only the "cell size given" branch is kept:
 * the reference tests the previous global's Lc there (exshalos_h.c:78); here
 * the argument itself is tested. Returns 1 for an unsupported Lc. */
int orc_set_box(orc_params *p, int ndx, int ndy, int ndz, float Lc) {
  p->nd[0] = ndx; p->nd[1] = ndy; p->nd[2] = ndz;
  p->ng = (size_t)ndx * (size_t)ndy * (size_t)ndz;
  p->nz2 = ndz / 2 + 1;
  if (!(Lc < ORC_LC_MAX) || !(Lc > 0.0f)) return 1;
  p->Lc = Lc;
  p->Mcell = (float)(p->rhomz * pow(Lc, 3.0));
  for (int i = 0; i < 3; i++) p->L[i] = p->Lc * p->nd[i];
  p->Mtot = p->rhomz * p->L[0] * p->L[1] * p->L[2];
  for (int i = 0; i < 3; i++) p->kl[i] = (float)(2.0 * M_PI / p->L[i]);
  p->Normx = (float)(1.0 / sqrt(p->L[0] * p->L[1] * p->L[2]));
  p->Normk = (float)(sqrt(p->L[0] * p->L[1] * p->L[2]) / (double)(p->nd[0] * p->nd[1] * p->nd[2]));
  p->Lc_d = (double)Lc;
  for (int i = 0; i < 3; i++) {
    p->L_d[i] = p->Lc_d * p->nd[i];
    p->kl_d[i] = 2.0 * M_PI / p->L_d[i];
  }
  p->Normx_d = 1.0 / sqrt(p->L_d[0] * p->L_d[1] * p->L_d[2]);
  p->Normk_d = sqrt(p->L_d[0] * p->L_d[1] * p->L_d[2]) / ((double)p->nd[0] * p->nd[1] * p->nd[2]);
  p->nmin = p->nd[0];
  if (p->nmin > p->nd[1]) p->nmin = p->nd[1];
  if (p->nmin > p->nd[2]) p->nmin = p->nd[2];
  return 0;
}

/* set_barrier, exshalos_h.c:60-66; DO_EB as decided at exshalos.c:737-740 */
void orc_set_barrier(orc_params *p, int Nmin, float a, float beta, float alpha, int seed) {
  p->Nmin = Nmin; p->a = a; p->beta = beta; p->alpha = alpha; p->seed = seed;
  p->DO_EB = (a == 1.0f && beta == 0.0f && alpha == 0.0f) ? 0 : 1;
}

int orc_ncells(const orc_params *p) { return (int)floor(ORC_M_MAX / p->Mcell); }

/* top-hat window, exshalos_h.c:35-40 (float result) */
static float W_f(float k, float R) {
  return (float)(3.0 / (pow(k * R, 2)) * (sin(k * R) / (k * R) - cos(k * R)));
}
static double W_d(double k, double R) {
  double x = k * R;
  return 3.0 / (x * x) * (sin(x) / x - cos(x));
}

/* calc_sigma, find_halos.c:4-13: float accumulator, double terms */
static float calc_sigma_f(const float *k, const float *P, int Nk, float R) {
  float resp = 0.0f;
  for (int i = 0; i < Nk - 1; i++)
    resp += (k[i + 1] - k[i]) / 2.0 *
            (P[i] * pow(k[i] * W_f(k[i], R), 2) + P[i + 1] * pow(k[i + 1] * W_f(k[i + 1], R), 2));
  return (float)(resp / (2.0 * M_PI * M_PI));
}
static double calc_sigma_d(const float *k, const float *P, int Nk, double R) {
  double resp = 0.0;
  for (int i = 0; i < Nk - 1; i++) {
    double k0 = k[i], k1 = k[i + 1];
    double w0 = k0 * W_d(k0, R), w1 = k1 * W_d(k1, R);
    resp += (k1 - k0) / 2.0 * ((double)P[i] * w0 * w0 + (double)P[i + 1] * w1 * w1);
  }
  return resp / (2.0 * M_PI * M_PI);
}

/* fh model 1 (Tinker, Delta=300), find_halos.c:47-69, float locals */
static float fh_f(float sigma) {
  float B = 0.466f, d = 2.06f, e = 0.99f, f = 0.48f, g = 1.310f;
  return (float)(B * (pow(sigma / e, -d) + pow(sigma, -f)) * exp(-g / (sigma * sigma)));
}
static double fh_d(double sigma) {
  double B = 0.466, d = 2.06, e = 0.99, f = 0.48, g = 1.310;
  return B * (pow(sigma / e, -d) + pow(sigma, -f)) * exp(-g / (sigma * sigma));
}

/* Compute_Sig (find_halos.c:16-44) and Compute_nh (find_halos.c:72-93) */
int orc_sigma_tables(const orc_params *p, const float *K, const float *P, int Nk,
                     int prec64, float *Sig_grid, double *M, double *Int) {
  int Nr = Nk, Ncells = orc_ncells(p);
  double *Sig = (double *)malloc(sizeof(double) * Nr);
  double *Rd = (double *)malloc(sizeof(double) * Nr);
  if (!Sig || !Rd) { free(Sig); free(Rd); return -1; }
  if (!prec64) {
    float Rmin = (float)pow(p->Mcell * 0.9 * 3.0 / (4.0 * M_PI * p->rhomz), 1.0 / 3.0);
    float Rmax = (float)pow(ORC_M_MAX * 3.0 / (4.0 * M_PI * p->rhomz), 1.0 / 3.0);
    for (int i = 0; i < Nr; i++) {
      float R = (float)pow(10, log10(Rmin) + i * (log10(Rmax) - log10(Rmin)) / (Nr - 1));
      Rd[i] = R;
      M[i] = (double)4.0 / 3.0 * M_PI * ((float)p->rhomz * pow(R, 3));
    }
    for (int i = 0; i < Nr; i++) Sig[i] = (double)sqrt(calc_sigma_f(K, P, Nk, (float)Rd[i]));
  } else {
    double Rmin = pow((double)p->Mcell * 0.9 * 3.0 / (4.0 * M_PI * (double)p->rhomz), 1.0 / 3.0);
    double Rmax = pow(ORC_M_MAX * 3.0 / (4.0 * M_PI * (double)p->rhomz), 1.0 / 3.0);
    for (int i = 0; i < Nr; i++) {
      Rd[i] = pow(10.0, log10(Rmin) + i * (log10(Rmax) - log10(Rmin)) / (Nr - 1));
      M[i] = 4.0 / 3.0 * M_PI * (double)p->rhomz * pow(Rd[i], 3);
    }
    for (int i = 0; i < Nr; i++) Sig[i] = sqrt(calc_sigma_d(K, P, Nk, Rd[i]));
  }
  orc_spline sp;
  if (orc_spline_init(&sp, M, Sig, Nr)) { free(Sig); free(Rd); return -1; }
  int st = 0;
  Sig_grid[0] = 1e+30f;
  for (int i = 1; i < Ncells; i++) {
    double v = orc_spline_eval(&sp, (double)i * p->Mcell, &st);
    Sig_grid[i] = (float)pow(v, 2.0);
  }
  orc_spline_free(&sp);
  /* cumulative mass-function integral */
  Int[0] = 0.0;
  for (int i = 1; i < Nr; i++) {
    if (!prec64) {
      float R1 = (float)Rd[i], R0 = (float)Rd[i - 1];
      Int[i] = Int[i - 1] - (double)(log(Sig[i]) - log(Sig[i - 1])) / 2.0 *
                                (fh_f((float)Sig[i]) / pow(R1, 3.0) + fh_f((float)Sig[i - 1]) / pow(R0, 3.0));
    } else {
      Int[i] = Int[i - 1] - (log(Sig[i]) - log(Sig[i - 1])) / 2.0 *
                                (fh_d(Sig[i]) / pow(Rd[i], 3.0) + fh_d(Sig[i - 1]) / pow(Rd[i - 1], 3.0));
    }
    if (Int[i] == Int[i - 1]) Int[i] = Int[i - 1] * 1.000001;
  }
  free(Sig); free(Rd);
  return st ? -1 : Ncells;
}

/* Barrier, find_halos.c:200-212 */
float orc_barrier(const orc_params *p, float S) {
  if (p->DO_EB == 0) return p->dc;
  return (float)(sqrt(p->a) * p->dc * (1.0 + p->beta * pow(S / (p->a * p->dc * p->dc), p->alpha)));
}

void orc_barrier_table(const orc_params *p, const float *Sig_grid, int Ncells, float *Btab) {
  for (int c = 0; c < Ncells; c++) Btab[c] = orc_barrier(p, Sig_grid[c]);
}

/* Compute_Spheres (find_halos.c:382-420): cumulative number of cells with
 * i^2+j^2+k^2 <= l over the non-empty shells l < lmax.  The reference scans a
 * cube per l; counting representations once over the full cube gives the same
 * numbers. */
int orc_cells_in_spheres(int lmax, int *out, int cap) {
  int t = (int)floor(sqrt((double)lmax)) + 1;
  long *hist = (long *)calloc((size_t)lmax, sizeof(long));
  if (!hist) return -1;
  for (int i = -t; i <= t; i++)
    for (int j = -t; j <= t; j++)
      for (int k = -t; k <= t; k++) {
        long d = (long)i * i + (long)j * j + (long)k * k;
        if (d < lmax) hist[d]++;
      }
  int m = 0;
  long cum = 0;
  for (int l = 0; l < lmax; l++) {
    if (hist[l] > 0) {
      cum += hist[l];
      if (m < cap) out[m] = (int)cum;
      m++;
    }
  }
  free(hist);
  return m;
}
