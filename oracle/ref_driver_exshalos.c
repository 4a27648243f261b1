/* REFERENCE BUILD — test infrastructure only.
 * Entry points into the reference's own exshalos core (src/exshalos/*.c,
 * compiled unmodified from the reference tree by oracle/ref_build.py against
 * the FFTW3/GSL stand-ins of oracle/ref_shim/), for tests/test_oracle_ref.py
 * to compare the oracle's restatement with.  Each sets the reference's
 * globals the way its Python binding does (src/exshalos/exshalos.c:735-744)
 * and calls the reference function named in its comment.
 * Status: 0 ok; 2 output capacity too small; 5 a spline evaluated outside
 * its knots (the reference's GSL would abort there). */
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "box.h"

extern long ref_gsl_domain_errors;

static void ref_setup(int nd, float Lc, float Om0, float z, float dc, int Nmin, float a, float beta, float alpha,
                      int seed, int out_den, int out_lpt, int do_2lpt, int nthreads) {
  const char do_eb = (a == 1.0f && beta == 0.0f && alpha == 0.0f) ? FALSE : TRUE;
  set_cosmology(Om0, z, dc);
  set_box(nd, nd, nd, Lc);
  set_barrier(Nmin, a, beta, alpha, seed);
  set_out((char)out_den, 1, (char)out_lpt, FALSE, (char)do_2lpt, do_eb, 0, FALSE, FALSE);
  omp_set_num_threads(nthreads > 0 ? nthreads : 1);
  ref_gsl_domain_errors = 0;
}

static int ref_copy_halos(size_t nh, const HALOS *halos, size_t cap, int *hx, int *hcount, float *Mh) {
  if (nh > cap) return 2;
  for (size_t i = 0; i < nh; i++) {
    for (int j = 0; j < 3; j++) hx[3 * i + j] = halos[i].x[j];
    hcount[i] = halos[i].count;
    Mh[i] = halos[i].Mh;
  }
  return 0;
}

/* Generate_Halos_Box_from_Pk (src/exshalos/box.c:4-68) with the density grid
 * and the flags kept; S (3 ng floats) receives the particle positions when
 * not NULL (OUT_LPT). */
int ref_halos_box_from_pk(const float *K, const float *P, int Nk, int nd, float Lc, float Om0, float z, float dc,
                          int Nmin, float a, float beta, float alpha, int seed, int fixed, float phase,
                          float k_smooth, int do_2lpt, int nthreads, float *delta, long *flag, float *S,
                          size_t cap, size_t *nh_out, int *hx, int *hcount, float *Mh, float *posh) {
  ref_setup(nd, Lc, Om0, z, dc, Nmin, a, beta, alpha, seed, TRUE, S != NULL, do_2lpt, nthreads);
  for (size_t i = 0; i < box.ng; i++) flag[i] = (long)box.ng;
  HALOS *halos = NULL;
  fft_real *ph = NULL, *vh = NULL;
  const size_t nh = Generate_Halos_Box_from_Pk((fft_real *)K, (fft_real *)P, Nk, 100000.0f, k_smooth, &halos, &ph,
                                               &vh, flag, delta, S, NULL, fixed, phase);
  int st = ref_gsl_domain_errors ? 5 : ref_copy_halos(nh, halos, cap, hx, hcount, Mh);
  if (!st) memcpy(posh, ph, sizeof(float) * 3 * nh);
  *nh_out = nh;
  free(ph);
  free(halos);
  return st;
}

/* Compute_Den (src/exshalos/density_grid.c:71-217): the field and its modes
 * (nd x nd x (nd/2 + 1) complex) as density_grid_compute sets them up
 * (src/exshalos/exshalos.c:71-73: a fixed cosmology, Nmin 1, no barrier). */
int ref_density_grid(const float *K, const float *P, int Nk, int nd, float Lc, int seed, int fixed, float phase,
                     float k_smooth, int nthreads, float *delta, float *deltak) {
  ref_setup(nd, Lc, 0.31f, 0.0f, 1.686f, 1, 1.0f, 0.0f, 0.0f, seed, TRUE, FALSE, FALSE, nthreads);
  Compute_Den((fft_real *)K, (fft_real *)P, Nk, 100000.0f, delta, (fft_complex *)deltak, fixed, phase, k_smooth);
  return ref_gsl_domain_errors ? 5 : 0;
}

/* Find_Halos (src/exshalos/find_halos.c:479-563) on a given grid */
int ref_find_halos(const float *delta, const float *K, const float *P, int Nk, int nd, float Lc, float Om0, float z,
                   float dc, int Nmin, float a, float beta, float alpha, int seed, int nthreads, long *flag,
                   size_t cap, size_t *nh_out, int *hx, int *hcount, float *Mh) {
  ref_setup(nd, Lc, Om0, z, dc, Nmin, a, beta, alpha, seed, FALSE, FALSE, FALSE, nthreads);
  for (size_t i = 0; i < box.ng; i++) flag[i] = (long)box.ng;
  HALOS *halos = NULL;
  const size_t nh = Find_Halos((fft_real *)delta, (fft_real *)K, (fft_real *)P, Nk, flag, &halos);
  const int st = ref_gsl_domain_errors ? 5 : ref_copy_halos(nh, halos, cap, hx, hcount, Mh);
  *nh_out = nh;
  free(halos);
  return st;
}

/* Compute_Sig (src/exshalos/find_halos.c:16-44) and the barrier
 * (:200-212) of every cell count: Sig_grid and Btab of Ncells floats */
int ref_sigma_barrier(const float *K, const float *P, int Nk, int nd, float Lc, float Om0, float z, float dc,
                      float a, float beta, float alpha, int Ncells, float *Sig_grid, float *Btab) {
  ref_setup(nd, Lc, Om0, z, dc, 1, a, beta, alpha, 1, FALSE, FALSE, FALSE, 1);
  fft_real *R = (fft_real *)malloc(sizeof(fft_real) * Nk);
  double *M = (double *)malloc(sizeof(double) * Nk), *Sig = (double *)malloc(sizeof(double) * Nk);
  Compute_Sig(Nk, R, M, Sig, Sig_grid, (fft_real *)K, (fft_real *)P, Nk);
  for (int i = 0; i < Ncells; i++) Btab[i] = Barrier(Sig_grid[i]);
  free(R); free(M); free(Sig);
  return ref_gsl_domain_errors ? 5 : 0;
}

/* Compute_1LPT / Compute_2LPT / Compute_Posh / Compute_Pos
 * (src/exshalos/lpt.c:4-255) on given modes and a given labelling: posh
 * (3 nh floats) the halo positions, S (3 ng floats) the particle positions */
int ref_lpt(const float *deltak_in, int nd, float Lc, float Om0, float z, int do_2lpt, float k_smooth, int nthreads,
            const long *flag_in, size_t nh, const int *hx, const int *hcount, float *posh, float *S) {
  ref_setup(nd, Lc, Om0, z, -1.0f, 1, 1.0f, 0.0f, 0.0f, 1, FALSE, TRUE, do_2lpt, nthreads);
  const size_t nk = (size_t)box.nd[0] * box.nd[1] * box.nz2;
  fft_complex *dk = (fft_complex *)malloc(sizeof(fft_complex) * nk);
  memcpy(dk, deltak_in, sizeof(fft_complex) * nk);
  long *flag = (long *)malloc(sizeof(long) * box.ng);
  memcpy(flag, flag_in, sizeof(long) * box.ng);
  HALOS *halos = (HALOS *)calloc(nh ? nh : 1, sizeof(HALOS));
  for (size_t i = 0; i < nh; i++) {
    for (int j = 0; j < 3; j++) halos[i].x[j] = hx[3 * i + j];
    halos[i].count = hcount[i];
  }
  memset(posh, 0, sizeof(float) * 3 * nh);
  Compute_1LPT(dk, posh, NULL, S, NULL, flag, k_smooth);
  if (do_2lpt) Compute_2LPT(posh, NULL, S, NULL, flag, k_smooth);
  Compute_Posh(halos, posh, NULL, nh);
  Compute_Pos(S);
  free(dk); free(flag); free(halos);
  return 0;
}
