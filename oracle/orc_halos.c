/* ORACLE — test infrastructure only (see orc.h).
 * Halo finder restated from src/exshalos/find_halos.c in the reference's
 * types: float densities and barriers, double running means. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

static inline int cysum(int i, int j, int nd) {        /* exshalos_h.c:21-32 */
  int r = i + j;
  if (r >= nd) r -= nd;
  if (r < 0) r += nd;
  return r;
}

static inline int is_peak(const orc_params *p, const float *d, int i, int j, int k, float den) {
  int n0 = p->nd[0], n1 = p->nd[1], n2 = p->nd[2];
#define IDX(a, b, c) (((size_t)(a) * n1 + (b)) * (size_t)n2 + (size_t)(c))
  return den > d[IDX(cysum(i, 1, n0), j, k)] && den > d[IDX(cysum(i, -1, n0), j, k)] &&
         den > d[IDX(i, cysum(j, 1, n1), k)] && den > d[IDX(i, cysum(j, -1, n1), k)] &&
         den > d[IDX(i, j, cysum(k, 1, n2))] && den > d[IDX(i, j, cysum(k, -1, n2))];
#undef IDX
}

/* Count_Peaks, find_halos.c:108-126 */
size_t orc_count_peaks(const orc_params *p, const float *delta) {
  size_t np = 0;
  for (int i = 0; i < p->nd[0]; i++)
    for (int j = 0; j < p->nd[1]; j++)
      for (int k = 0; k < p->nd[2]; k++) {
        size_t ind = ((size_t)i * p->nd[1] + j) * p->nd[2] + k;
        if (is_peak(p, delta, i, j, k, delta[ind])) np++;
      }
  return np;
}

/* Find_Peaks, find_halos.c:129-156 (row-major order) */
size_t orc_find_peaks(const orc_params *p, const float *delta, orc_peak *pk) {
  size_t c = 0;
  for (int i = 0; i < p->nd[0]; i++)
    for (int j = 0; j < p->nd[1]; j++)
      for (int k = 0; k < p->nd[2]; k++) {
        size_t ind = ((size_t)i * p->nd[1] + j) * p->nd[2] + k;
        float den = delta[ind];
        if (is_peak(p, delta, i, j, k, den)) {
          pk[c].x[0] = i; pk[c].x[1] = j; pk[c].x[2] = k; pk[c].den = den;
          c++;
        }
      }
  return c;
}

static inline void swap_pk(orc_peak *a, orc_peak *b) { orc_peak t = *a; *a = *b; *b = t; }

/* partition_peaks / quickSort_peaks, find_halos.c:175-197: Lomuto scheme,
 * last element as pivot, "<=" to the left.  The recursion on the larger side
 * is turned into a loop; the order of the partitions is unchanged. */
void orc_quicksort_peaks(orc_peak *a, long long low, long long high) {
  while (low < high) {
    float pivot = a[high].den;
    long long i = low - 1;
    for (long long j = low; j < high; j++)
      if (a[j].den <= pivot) { i++; swap_pk(&a[i], &a[j]); }
    swap_pk(&a[i + 1], &a[high]);
    long long pi = i + 1;
    if (pi - low < high - pi) { orc_quicksort_peaks(a, low, pi - 1); low = pi + 1; }
    else { orc_quicksort_peaks(a, pi + 1, high); high = pi - 1; }
  }
}

/* dist2(i,j,k) == g over the cube of half-width t, in the reference's loop
 * order i, j, k ascending (find_halos.c:295-306). */

/* Grow_Halos, find_halos.c:215-379 (box output, no profiles). */
size_t orc_grow_halos(const orc_params *p, size_t np, const orc_peak *pk,
                      const float *delta, const float *Btab, int Ncells,
                      int64_t *flag, int *hx, int *hcount) {
  const int n0 = p->nd[0], n1 = p->nd[1], n2 = p->nd[2];
  const int64_t ng = (int64_t)p->ng;
  const float Bmin = Btab[Ncells - 1];
  const int tcap = p->nmin / 2;
  /* a growth past every shell inside the capped cube would never stop in
   * the reference; it is reported as a range error here */
  const int gmax = 3 * tcap * tcap + 1;
  size_t nh = 0;
  if (np < 2) return 0;   /* the reference loop needs l > 0 (find_halos.c:226) */
#define CELL(x0, y0, z0, a, b, c) \
  (((size_t)cysum(x0, a, n0) * n1 + (size_t)cysum(y0, b, n1)) * (size_t)n2 + (size_t)cysum(z0, c, n2))
  for (size_t l = np - 1; l > 0; l--) {
    const int x0 = pk[l].x[0], y0 = pk[l].x[1], z0 = pk[l].x[2];
    if (pk[l].den < Bmin) break;
    if (flag[((size_t)x0 * n1 + y0) * (size_t)n2 + z0] != ng) continue;
    double den = (double)pk[l].den, den_tmp = (double)pk[l].den;
    int count = 0, count_tmp = 1, grows_tmp = 0, grows = 0, tmp;
    while (den_tmp >= Bmin) {
      if (count < count_tmp) grows = grows_tmp;
      grows_tmp++;
      if (grows_tmp > gmax) return (size_t)-1;
      den = den_tmp;
      count = count_tmp;
      den_tmp = den * (double)count;
      tmp = (int)floor(sqrt((double)grows_tmp));
      if (tmp > tcap) tmp = tcap;
      for (int i = -tmp; i <= tmp; i++)
        for (int j = -tmp; j <= tmp; j++)
          for (int k = -tmp; k <= tmp; k++)
            if (i * i + j * j + k * k == grows_tmp) {
              size_t ind = CELL(x0, y0, z0, i, j, k);
              if (flag[ind] != ng) den_tmp += (double)-p->Mtot;
              else den_tmp += (double)delta[ind];
              count_tmp++;
            }
      den_tmp = den_tmp / (double)count_tmp;
    }
    while (count > 0 && (count >= Ncells || den < Btab[count])) {
      if (count >= Ncells) return (size_t)-1;    /* Sig_Grid[count] past its end */
      den_tmp = den;
      count_tmp = count;
      den = den * (double)count;
      tmp = (int)floor(sqrt((double)grows));
      if (tmp > tcap) tmp = tcap;
      for (int i = -tmp; i <= tmp; i++)
        for (int j = -tmp; j <= tmp; j++)
          for (int k = -tmp; k <= tmp; k++)
            if (i * i + j * j + k * k == grows) {
              den -= (double)delta[CELL(x0, y0, z0, i, j, k)];
              count--;
            }
      if (count > 0) den = den / (double)count;
      if (count < count_tmp) grows_tmp = grows;
      grows--;
    }
    if (count == 0) continue;
    tmp = (int)floor(sqrt((double)grows_tmp));
    for (int i = -tmp; i <= tmp; i++)
      for (int j = -tmp; j <= tmp; j++)
        for (int k = -tmp; k <= tmp; k++)
          if (i * i + j * j + k * k < grows_tmp) flag[CELL(x0, y0, z0, i, j, k)] = (int64_t)nh;
    flag[((size_t)x0 * n1 + y0) * (size_t)n2 + z0] = -(int64_t)nh;
    if (count >= p->Nmin) {
      hcount[nh] = count;
      hx[3 * nh] = x0; hx[3 * nh + 1] = y0; hx[3 * nh + 2] = z0;
      nh++;
    } else {
      for (int i = -tmp; i <= tmp; i++)
        for (int j = -tmp; j <= tmp; j++)
          for (int k = -tmp; k <= tmp; k++)
            if (i * i + j * j + k * k < grows_tmp) flag[CELL(x0, y0, z0, i, j, k)] = ng + 1;
    }
  }
#undef CELL
  return nh;
}

/* Compute_Mass, find_halos.c:455-476, with Next_Count (:442-452) */
int orc_compute_mass(const orc_params *p, size_t nh, const int *hcount, const int *spheres,
                     int nspheres, int Ncells, const double *M, const double *Int, int Nr,
                     float *Mh) {
  orc_spline sI, sInv;
  if (orc_spline_init(&sI, M, Int, Nr)) return 1;
  if (orc_spline_init(&sInv, Int, M, Nr)) { orc_spline_free(&sI); return 1; }
  orc_taus rng;
  orc_taus_seed(&rng, (unsigned long)p->seed);
  int err = 0, st = 0;
  int lim = Ncells < nspheres ? Ncells : nspheres;
  for (size_t i = 0; i < nh; i++) {
    int c = -1;
    for (int q = 0; q < lim; q++)
      if (spheres[q] == hcount[i]) { c = q + 1; break; }
    if (c < 0 || c >= nspheres) { err = 2; Mh[i] = NAN; continue; }
    float m0 = hcount[i] * p->Mcell, m1 = spheres[c] * p->Mcell;
    double i0 = orc_spline_eval(&sI, (double)m0, &st);
    double i1 = orc_spline_eval(&sI, (double)m1, &st);
    double i0b = orc_spline_eval(&sI, (double)m0, &st);
    float den_tmp = (float)(i0 + (i1 - i0b) * orc_taus_uniform(&rng));
    Mh[i] = (float)orc_spline_eval(&sInv, (double)den_tmp, &st);
    if (st) err = 3;
  }
  orc_spline_free(&sI); orc_spline_free(&sInv);
  return err;
}

/* Find_Halos, find_halos.c:479-563, from prepared tables */
size_t orc_find_halos(const orc_params *p, const float *delta, const float *Btab, int Ncells,
                      const double *M, const double *Int, int Nr, int64_t *flag, int *hx,
                      int *hcount, float *Mh, size_t cap, size_t *np_out) {
  size_t np = orc_count_peaks(p, delta);
  orc_peak *pk = (orc_peak *)malloc(sizeof(orc_peak) * (np ? np : 1));
  if (!pk) return (size_t)-1;
  orc_find_peaks(p, delta, pk);
  if (np > 0) orc_quicksort_peaks(pk, 0, (long long)np - 1);
  if (np_out) *np_out = np;
  for (size_t i = 0; i < p->ng; i++) flag[i] = (int64_t)p->ng;
  int *hx_l = hx, *hc_l = hcount;
  int own = 0;
  if (cap < np) {
    hx_l = (int *)malloc(sizeof(int) * 3 * (np ? np : 1));
    hc_l = (int *)malloc(sizeof(int) * (np ? np : 1));
    own = 1;
  }
  size_t nh = orc_grow_halos(p, np, pk, delta, Btab, Ncells, flag, hx_l, hc_l);
  free(pk);
  if (nh != (size_t)-1) {
    if (own) {
      if (nh > cap) nh = (size_t)-1;
      else { memcpy(hx, hx_l, sizeof(int) * 3 * nh); memcpy(hcount, hc_l, sizeof(int) * nh); }
    }
  }
  if (own) { free(hx_l); free(hc_l); }
  if (nh == (size_t)-1) return nh;
  static int spheres[8400];
  static int nsph = 0;
  if (!nsph) nsph = orc_cells_in_spheres(10000, spheres, 8400);
  if (orc_compute_mass(p, nh, hcount, spheres, nsph, Ncells, M, Int, Nr, Mh)) return (size_t)-2;
  return nh;
}
