/* REFERENCE BUILD — test infrastructure only.
 * Implementations of the FFTW3 and GSL stand-ins in oracle/ref_shim/ over the
 * oracle's restatements (oracle/orc_fft.c compiled in float, orc_rng.c,
 * orc_spline.c).  Linked only into oracle/_ref/, the reference's own C
 * compiled where it lies by oracle/ref_build.py; with identical library
 * arithmetic on both sides, the reference's loops and the oracle's
 * restatement of them can be compared bit for bit. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"
#include "gsl/gsl_randist.h"
#include "gsl/gsl_rng.h"
#include "gsl/gsl_sf.h"
#include "gsl/gsl_spline.h"
#include "orc.h"

/* ---------------------------------------------------------------- FFTW3 */
enum { REF_R2C = 1, REF_C2R = 2, REF_DFT1 = 3 };

struct ref_fft_plan {
  int kind, n0, n1, n2, sign;
  void *in, *out;
};

static struct ref_fft_plan *new_plan(int kind, int n0, int n1, int n2, int sign, void *in, void *out) {
  struct ref_fft_plan *p = (struct ref_fft_plan *)calloc(1, sizeof(*p));
  p->kind = kind; p->n0 = n0; p->n1 = n1; p->n2 = n2; p->sign = sign; p->in = in; p->out = out;
  return p;
}

fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float *in, fftwf_complex *out, unsigned flags) {
  (void)flags;
  return new_plan(REF_R2C, n0, n1, n2, -1, in, out);
}

fftwf_plan fftwf_plan_dft_c2r_3d(int n0, int n1, int n2, fftwf_complex *in, float *out, unsigned flags) {
  (void)flags;
  return new_plan(REF_C2R, n0, n1, n2, +1, in, out);
}

void fftwf_execute(const fftwf_plan p) {
  if (p->kind == REF_R2C) orc_fft_r2c_3d(p->n0, p->n1, p->n2, (const float *)p->in, (float *)p->out);
  else if (p->kind == REF_C2R) orc_fft_c2r_3d(p->n0, p->n1, p->n2, (const float *)p->in, (float *)p->out);
}

void fftwf_destroy_plan(fftwf_plan p) { free(p); }
void *fftwf_malloc(size_t n) { return malloc(n); }
/* the reference also passes plans here (src/spectrum/spectrum_h.c:162,165):
 * both come from malloc/calloc */
void fftwf_free(void *p) { free(p); }
int fftwf_init_threads(void) { return 1; }
void fftwf_plan_with_nthreads(int n) { (void)n; }
void fftwf_cleanup_threads(void) {}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
  (void)flags;
  return new_plan(REF_DFT1, n, 0, 0, sign, in, out);
}

/* FFTLog's transforms (cold: only for R_max < 1e5): the plain O(n^2) DFT,
 * out[k] = sum_j in[j] exp(sign 2 pi i j k / n), in place allowed */
void fftw_execute(const fftw_plan p) {
  const int n = p->n0;
  const double *in = (const double *)p->in;
  double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  for (int k = 0; k < n; k++) {
    double re = 0.0, im = 0.0;
    for (int j = 0; j < n; j++) {
      const double a = p->sign * 2.0 * M_PI * (double)(((long long)j * k) % n) / n;
      re += in[2 * j] * cos(a) - in[2 * j + 1] * sin(a);
      im += in[2 * j] * sin(a) + in[2 * j + 1] * cos(a);
    }
    tmp[2 * k] = re;
    tmp[2 * k + 1] = im;
  }
  memcpy(p->out, tmp, sizeof(double) * 2 * (size_t)n);
  free(tmp);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

/* ----------------------------------------------------------------- GSL */
struct ref_gsl_rng { orc_taus t; };
static const gsl_rng_type ref_taus_type = {"taus"};
const gsl_rng_type *gsl_rng_taus = &ref_taus_type;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) {
  (void)T;
  gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
  orc_taus_seed(&r->t, 0);                  /* GSL seeds a new generator with its default seed, 0 */
  return r;
}
void gsl_rng_set(const gsl_rng *r, unsigned long seed) { orc_taus_seed(&((gsl_rng *)r)->t, seed); }
void gsl_rng_free(gsl_rng *r) { free(r); }
unsigned long gsl_rng_get(const gsl_rng *r) { return orc_taus_get(&((gsl_rng *)r)->t); }
double gsl_rng_uniform(const gsl_rng *r) { return orc_taus_uniform(&((gsl_rng *)r)->t); }
double gsl_rng_uniform_pos(const gsl_rng *r) { return orc_taus_uniform_pos(&((gsl_rng *)r)->t); }
double gsl_ran_gaussian(const gsl_rng *r, double sigma) { return orc_gaussian(&((gsl_rng *)r)->t, sigma); }
double gsl_ran_flat(const gsl_rng *r, double a, double b) { return orc_flat(&((gsl_rng *)r)->t, a, b); }

static const gsl_interp_type ref_cspline_type = {"cspline"};
const gsl_interp_type *gsl_interp_cspline = &ref_cspline_type;
struct ref_gsl_interp_accel { int unused; };
struct ref_gsl_spline { orc_spline s; size_t n; int ready; };

/* spline evaluations outside the knots since the last reset (GSL would
 * abort the program there) */
long ref_gsl_domain_errors = 0;

gsl_interp_accel *gsl_interp_accel_alloc(void) { return (gsl_interp_accel *)calloc(1, sizeof(gsl_interp_accel)); }
void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }

gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t size) {
  (void)T;
  gsl_spline *s = (gsl_spline *)calloc(1, sizeof(gsl_spline));
  s->n = size;
  return s;
}

int gsl_spline_init(gsl_spline *spline, const double xa[], const double ya[], size_t size) {
  if (spline->ready) orc_spline_free(&spline->s);
  spline->ready = orc_spline_init(&spline->s, xa, ya, (int)size) == 0;
  return spline->ready ? 0 : 1;
}

double gsl_spline_eval(const gsl_spline *spline, double x, gsl_interp_accel *a) {
  (void)a;
  int st = 0;
  const double v = orc_spline_eval(&spline->s, x, &st);
  if (st) {
    ref_gsl_domain_errors++;
    return NAN;
  }
  return v;
}

void gsl_spline_free(gsl_spline *spline) {
  if (spline && spline->ready) orc_spline_free(&spline->s);
  free(spline);
}

double gsl_sf_legendre_Pl(const int l, const double x) {
  if (l == 0) return 1.0;
  double p0 = 1.0, p1 = x;
  for (int k = 2; k <= l; k++) {
    const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = p2;
  }
  return p1;
}
