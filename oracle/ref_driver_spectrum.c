/* REFERENCE BUILD — test infrastructure only.
 * Entry points into the reference's own spectrum core (src/spectrum/*.c,
 * compiled unmodified by oracle/ref_build.py against the stand-ins of
 * oracle/ref_shim/), for tests/test_oracle_ref.py. */
#include <omp.h>
#include <stdlib.h>

#include "gridmodule.h"
#include "powermodule.h"

/* Tracer_Grid (src/spectrum/gridmodule.c:146-211) of np unit-mass tracers
 * with the CIC window, one type, no interlacing or redshift-space shift, on
 * one thread (the reference's threaded scatter races, gridmodule.c:173-204);
 * grid must hold nd^3 zeros */
void ref_cic(const float *pos, size_t np, int nd, float L, float *grid) {
  omp_set_num_threads(1);
  Tracer_Grid(grid, nd, L, -1, (fft_real *)pos, NULL, np, NULL, NULL, 1, 2, 4.0f, 5.0f, FALSE, 0.31f, 0.0f, 1);
}

/* Power_Spectrum (src/spectrum/powermodule.c:4-108) of one grid, l_max = 0,
 * as power_compute sets it up (src/spectrum/spectrum.c:111-197); the long
 * double bin sums come back rounded to double */
void ref_power(const float *grid, int nd, float L, int window, int Nk, float k_min, float k_max, int nthreads,
               double *Kmean, double *P, long *count) {
  omp_set_num_threads(nthreads > 0 ? nthreads : 1);
  long double *Pk = (long double *)calloc((size_t)Nk, sizeof(long double));
  long double *Km = (long double *)calloc((size_t)Nk, sizeof(long double));
  for (int i = 0; i < Nk; i++) count[i] = 0;
  Power_Spectrum((fft_real *)grid, nd, L, 1, window, 4.0f, FALSE, Nk, k_min, k_max, Km, Pk, count, 0, -1);
  for (int i = 0; i < Nk; i++) {
    Kmean[i] = (double)Km[i];
    P[i] = (double)Pk[i];
  }
  free(Pk); free(Km);
}
