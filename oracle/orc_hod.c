/* ORACLE — test infrastructure only (see orc.h).
 * Galaxy population of a halo catalogue and its colour split, restated from
 * src/hod/populate_halos.c (Ncentral_tot :4-6, Nsatellite_tot :9-18, f_c
 * :21-27, Profile :30-36, Interpolate_r_Eps :56-104, Generate_r :107-117,
 * Populate_total :120-217), src/hod/hod.c:31-160 (populate_halos) and
 * src/hod/split_galaxies.c (Occ_cen :4-17, Occ_sat :20-33, Galaxy_Types
 * :37-72).  `real` is the reference's fft_real: float in liborc_f32.
 *
 * One taus stream, seeded with `seed`, is consumed in halo order exactly as
 * the reference does: one uniform for the central, the Poisson draw of the
 * satellite number, then three uniforms (phi, theta, eps) per satellite.
 * The Poisson draw is Knuth's multiplicative method (TAOCP vol. 2, 3.4.1),
 * which is what gsl_ran_poisson does for means up to 10 (k + 1 uniforms for
 * a result k); for larger means GSL reduces through gamma and binomial
 * variates, which are not restated: here the multiplicative method goes on,
 * in pieces of mean <= 500.  The satellite radius is the r(Eps) spline value
 * itself, not multiplied by the virial radius, and the concentration-bin
 * index is the reference's floor((log c - log cmin) / (log cmax - log cmin))
 * (0, or 1 for the most concentrated halo): both as populate_halos.c:171-193
 * computes them. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

#define HOD_R_MIN 1.0e-3   /* hod_h.h:29-35 */
#define HOD_R_MAX 10.0
#define HOD_NRS 500
#define HOD_NCS 100
#define HOD_NEPS 1000
#define HOD_TOL 0.001
#define HOD_NEWTON_CAP 100000

typedef struct {
  real logMmin, siglogM, logM0, logM1, alpha, sigma, redshift, Mstar;
} hod_par;

static real ncentral_tot(const hod_par *h, real M) {            /* :4-6 */
  return 0.5 * (1.0 + erf((log10(M) - h->logMmin) / h->siglogM));
}

static real nsatellite_tot(const hod_par *h, real M) {          /* :9-18 */
  real resp;
  if (M >= pow(10.0, h->logM0))
    resp = pow((M - pow(10.0, h->logM0)) / pow(10.0, h->logM1), h->alpha) * ncentral_tot(h, M);
  else
    resp = 0.0;
  return resp;
}

static real f_c(const hod_par *h, real Mv) {                   /* :21-27 */
  return 9.0 / (1.0 + h->redshift) * pow(Mv / h->Mstar, -0.13);
}

static real profile(const hod_par *h, real x, real c) {        /* :30-36 */
  return 1.0 / (c * x * pow(1.0 + c * x, 2.0)) / (1.0 + pow(x, 2.0 / h->sigma));
}

/* Interpolate_r_Eps (:56-104): r(Eps) splines for NCs concentration bins.
 * Returns 0, or 1 when a spline leaves its domain or Newton never settles. */
static int interpolate_r_eps(const hod_par *h, real cmin, real cmax, orc_spline *spline_r) {
  double x[HOD_NRS], Int[HOD_NRS], Eps[HOD_NEPS], r[HOD_NEPS];
  for (int i = 0; i < HOD_NRS; i++)
    x[i] = pow(10.0, log10(HOD_R_MIN) + (log10(HOD_R_MAX) - log10(HOD_R_MIN)) * i / (HOD_NRS - 1));
  for (int i = 0; i < HOD_NEPS; i++) Eps[i] = ((double)i) / (HOD_NEPS - 1);
  for (int i = 0; i < HOD_NCS; i++) {
    const real c = pow(10.0, log10(cmin) + (log10(cmax) - log10(cmin)) * i / (HOD_NCS - 1));
    Int[0] = 0.0;
    for (int j = 1; j < HOD_NRS; j++)
      Int[j] = Int[j - 1] + (profile(h, x[j], c) * x[j] * x[j] + profile(h, x[j - 1], c) * x[j - 1] * x[j - 1]) *
                                (x[j] - x[j - 1]) / 2.0;
    orc_spline sI;
    if (orc_spline_init(&sI, x, Int, HOD_NRS)) return 1;
    int bad = 0;
    const real A = orc_spline_eval(&sI, HOD_R_MAX, &bad);
    r[0] = HOD_R_MIN;
    for (int j = 1; j < HOD_NEPS - 1 && !bad; j++) {
      if (j > 1) r[j] = r[j - 1];
      else r[j] = HOD_R_MIN + Eps[j];
      real rtmp = r[j] + 1.0;
      int it = 0;
      while (fabs(r[j] - rtmp) > HOD_TOL) {
        if (++it > HOD_NEWTON_CAP) { bad = 1; break; }
        rtmp = r[j];
        r[j] = r[j] - (orc_spline_eval(&sI, r[j], &bad) / A - Eps[j]) / (profile(h, r[j], c) * r[j] * r[j] / A);
        if (r[j] >= HOD_R_MAX || r[j] <= HOD_R_MIN) r[j] = Eps[j];
      }
    }
    r[HOD_NEPS - 1] = HOD_R_MAX;
    orc_spline_free(&sI);
    if (bad || orc_spline_init(&spline_r[i], Eps, r, HOD_NEPS)) {
      for (int q = 0; q < i; q++) orc_spline_free(&spline_r[q]);
      return 1;
    }
  }
  return 0;
}

/* gsl_ran_poisson's multiplicative branch (Knuth); pieces of mean <= 500
 * beyond it.  *used = uniforms consumed. */
static unsigned poisson(orc_taus *t, double mu, long long *used) {
  unsigned total = 0;
  double rem = mu;
  long long n = 0;
  for (;;) {
    const double m = rem > 500.0 ? 500.0 : rem;
    const double emu = exp(-m);
    double prod = 1.0;
    unsigned k = 0;
    do {
      prod *= orc_taus_uniform(t);
      n++;
      k++;
    } while (prod > emu);
    total += k - 1;
    rem -= m;
    if (!(rem > 0.0)) break;
  }
  *used = n;
  return total;
}

static real cysumf(real x, real y, real L) {                    /* hod_h.c:4-13 */
  real resp = x + y;
  if (resp >= L) resp -= L;
  if (resp < 0) resp += L;
  return resp;
}

/* Populate_total (:120-217) after populate_halos' set-up (hod.c:64-95).
 * Ch_in may be NULL (concentrations from f_c).  Outputs up to cap galaxies;
 * returns the number of galaxies, -1 when cap is exceeded, -2 on a table
 * error.  nsat_out[nh] (optional) receives each halo's satellite count and
 * ncen_out[nh] (optional) its central flag. */
long long orc_populate_halos(const real *posh, const real *velh, const real *Mh, const real *Ch_in, long long nh,
                             real Lc, real redshift, int ndx, int ndy, int ndz, real logMmin, real siglogM,
                             real logM0, real logM1, real alpha, real sigma, int seed, int out_vel,
                             long long cap, real *posg, real *velg, int64_t *gal_type, int *nsat_out,
                             int *ncen_out) {
  if (nh <= 0) return 0;
  hod_par h = {logMmin, siglogM, logM0, logM1, alpha, sigma, redshift, (real)4.638211e+12};
  const real L[3] = {Lc * ndx, Lc * ndy, Lc * ndz};            /* hod_h.c:62-66 */
  real *Ch = (real *)malloc(sizeof(real) * nh);
  for (long long i = 0; i < nh; i++) Ch[i] = Ch_in ? Ch_in[i] : f_c(&h, Mh[i]);
  real cmin = Ch[0], cmax = Ch[0];
  for (long long i = 1; i < nh; i++) {
    if (Ch[i] < cmin) cmin = Ch[i];
    if (Ch[i] > cmax) cmax = Ch[i];
  }
  orc_spline spline_r[HOD_NCS];
  if (interpolate_r_eps(&h, cmin, cmax, spline_r)) { free(Ch); return -2; }
  orc_taus t;
  orc_taus_seed(&t, (unsigned long)seed);
  long long count = 0;
  int bad = 0;
  for (long long i = 0; i < nh && count >= 0; i++) {
    const int Ncen = ncentral_tot(&h, Mh[i]) >= orc_taus_uniform(&t) ? 1 : 0;
    long long used;
    const int Nsat = (int)poisson(&t, (double)nsatellite_tot(&h, Mh[i]), &used);
    if (nsat_out) nsat_out[i] = Nsat;
    if (ncen_out) ncen_out[i] = Ncen;
    if (Ncen + Nsat == 0) continue;
    if (count + Ncen + Nsat > cap) { count = -1; break; }
    if (Ncen == 1) {
      for (int d = 0; d < 3; d++) {
        posg[3 * count + d] = posh[3 * i + d];
        if (out_vel) velg[3 * count + d] = velh[3 * i + d];
      }
      gal_type[count] = -(int64_t)i;
      count++;
    }
    if (Nsat == 0) continue;
    size_t ind_h;
    real w1, w2, Rv;
    if (cmax == cmin) {          /* the reference divides 0 by 0 here */
      ind_h = 0;
      w1 = 0.0;
      w2 = 1.0;
    } else {
      ind_h = (size_t)floor((log10(Ch[i]) - log10(cmin)) / (log10(cmax) - log10(cmin)));
      if (ind_h == HOD_NCS) ind_h = ind_h - 1;
      w1 = Ch[i] - pow(10.0, log10(cmin) + (log10(cmax) - log10(cmin)) * ind_h / (HOD_NCS - 1));
      w2 = pow(10.0, log10(cmin) + (log10(cmax) - log10(cmin)) * (ind_h + 1) / (HOD_NCS - 1)) - Ch[i];
      Rv = w1 + w2;
      w1 = w1 / Rv;
      w2 = w2 / Rv;
    }
    for (int j = 0; j < Nsat; j++) {
      const real phi = 2.0 * M_PI * orc_taus_uniform(&t);
      const real theta = M_PI * orc_taus_uniform(&t);
      const double eps = (real)orc_taus_uniform(&t);
      const real r1 = orc_spline_eval(&spline_r[ind_h], eps, &bad);
      const real r2 = orc_spline_eval(&spline_r[ind_h + 1], eps, &bad);
      const real r = r1 * w1 + r2 * w2;
      posg[3 * count] = cysumf(posh[3 * i], r * sin(theta) * cos(phi), L[0]);
      posg[3 * count + 1] = cysumf(posh[3 * i + 1], r * sin(theta) * sin(phi), L[1]);
      posg[3 * count + 2] = cysumf(posh[3 * i + 2], r * cos(theta), L[2]);
      if (out_vel)
        for (int d = 0; d < 3; d++) velg[3 * count + d] = velh[3 * i + d];
      gal_type[count] = (int64_t)i;
      count++;
    }
  }
  for (int i = 0; i < HOD_NCS; i++) orc_spline_free(&spline_r[i]);
  free(Ch);
  return bad ? -2 : count;
}

/* Occ_cen / Occ_sat (split_galaxies.c:4-33) */
static real occ(const real *params, int order, real log10Mh) {
  real resp = 0.0;
  for (int i = 0; i < order; i++) resp += params[i] * pow(log10Mh, i);
  if (resp < 0.0) resp = 0.0;
  if (resp > 1.0) resp = 1.0;
  return resp;
}

/* Galaxy_Types (split_galaxies.c:37-72) with its own taus stream (hod.c:
 * 192-197).  params_cen[(ntypes-1) * order_cen], params_sat likewise.
 * Returns 0, or 1 when a flag names a halo outside [0, nh). */
int orc_split_galaxies(long long ng, const real *Mh, long long nh, const int64_t *flag, const real *params_cen,
                       const real *params_sat, int ntypes, int order_cen, int order_sat, int seed, int *type) {
  orc_taus t;
  orc_taus_seed(&t, (unsigned long)seed);
  for (long long i = 0; i < ng; i++) {
    const real rnd = (real)orc_taus_uniform(&t);
    real Occ = 0.0;
    const long long hh = flag[i] > 0 ? flag[i] : -flag[i];
    if (hh >= nh) return 1;
    int j;
    if (flag[i] > 0) {
      for (j = 0; j < ntypes - 1; j++) {
        Occ += occ(params_sat + (size_t)j * order_sat, order_sat, log10(Mh[hh]));
        if (rnd <= Occ) { type[i] = j + 1; break; }
      }
      if (rnd > Occ) type[i] = ntypes;
    } else {
      for (j = 0; j < ntypes - 1; j++) {
        Occ += occ(params_cen + (size_t)j * order_cen, order_cen, log10(Mh[hh]));
        if (rnd <= Occ) { type[i] = -(j + 1); break; }
      }
      if (rnd > Occ) type[i] = -ntypes;
    }
  }
  return 0;
}
