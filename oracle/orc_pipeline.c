/* ORACLE — test infrastructure only (see orc.h).
 * Generate_Halos_Box_from_Pk (src/exshalos/box.c:4-68) driven from the
 * stage restatements in this directory. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "orc.h"

#define ORC_F64 (sizeof(real) == 8)

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

void orc_free(void *ptr) { free(ptr); }

void orc_result_free(orc_result *r) {
  free(r->Mh); free(r->posh); free(r->hx); free(r->hcount);
  free(r->delta); free(r->flag); free(r->S);
  memset(r, 0, sizeof(*r));
}

int orc_halos_box_from_pk(const float *K, const float *P, int Nk, int nd, float Lc, float Om0,
                          float z, float dc, int Nmin, float a, float beta, float alpha, int seed,
                          int stream, int fixed, float phase, float k_smooth, int do_2lpt,
                          int prec64, int keep_S, orc_result *res) {
  memset(res, 0, sizeof(*res));
  orc_params p;
  memset(&p, 0, sizeof(p));
  orc_set_cosmology(&p, Om0, z, dc);
  if (orc_set_box(&p, nd, nd, nd, Lc)) return 1;
  orc_set_barrier(&p, Nmin, a, beta, alpha, seed);
  size_t ng = p.ng, nk = (size_t)nd * nd * p.nz2;

  double t0 = now_s();
  real *deltak = (real *)malloc(sizeof(real) * 2 * nk);
  real *delta = (real *)malloc(sizeof(real) * ng);
  if (!deltak || !delta) { free(deltak); free(delta); return 2; }
  /* box.c:18 passes k_smooth = 1e5 to the field */
  if (orc_field_modes(&p, K, P, Nk, stream, fixed, phase, 100000.0f, deltak)) { free(deltak); free(delta); return 3; }
  orc_field_real(&p, deltak, delta);
  res->delta = (float *)malloc(sizeof(float) * ng);
  for (size_t i = 0; i < ng; i++) res->delta[i] = (float)delta[i];
  free(delta);
  double t1 = now_s();

  int Ncells = orc_ncells(&p);
  float *Sig = (float *)malloc(sizeof(float) * Ncells), *Btab = (float *)malloc(sizeof(float) * Ncells);
  double *M = (double *)malloc(sizeof(double) * Nk), *Int = (double *)malloc(sizeof(double) * Nk);
  if (orc_sigma_tables(&p, K, P, Nk, prec64, Sig, M, Int) < 0) { free(deltak); return 4; }
  orc_barrier_table(&p, Sig, Ncells, Btab);
  size_t np = orc_count_peaks(&p, res->delta);
  res->flag = (int64_t *)malloc(sizeof(int64_t) * ng);
  res->hx = (int *)malloc(sizeof(int) * 3 * (np ? np : 1));
  res->hcount = (int *)malloc(sizeof(int) * (np ? np : 1));
  res->Mh = (float *)malloc(sizeof(float) * (np ? np : 1));
  size_t nh = orc_find_halos(&p, res->delta, Btab, Ncells, M, Int, Nk, res->flag, res->hx,
                             res->hcount, res->Mh, np, &res->np);
  free(Sig); free(Btab); free(M); free(Int);
  /* 5: a halo mass outside the mass-function splines (where the reference's
   * gsl_spline_eval aborts, find_halos.c:472-474); 7: growth failed */
  if (nh == (size_t)-2 || nh == (size_t)-1) {
    free(deltak);
    orc_result_free(res);
    return nh == (size_t)-2 ? 5 : 7;
  }
  res->nh = nh;
  double t2 = now_s();

  res->posh = (real *)calloc(3 * (nh ? nh : 1), sizeof(real));
  real *S = (real *)malloc(sizeof(real) * 3 * ng);
  orc_lpt1(&p, deltak, res->flag, nh, k_smooth, S, res->posh);
  free(deltak);
  if (do_2lpt) orc_lpt2(&p, S, res->flag, nh, k_smooth, keep_S, res->posh);
  orc_posh(&p, nh, res->hx, res->hcount, res->posh);
  if (keep_S) { orc_pos(&p, S); res->S = S; }
  else free(S);
  double t3 = now_s();
  res->t_field = t1 - t0; res->t_halos = t2 - t1; res->t_lpt = t3 - t2;
  return 0;
}
