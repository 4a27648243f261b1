/* ORACLE — test infrastructure only (see orc.h).
 * Natural cubic spline, the interpolant the reference builds with
 * gsl_interp_cspline at density_grid.c:79-82, find_halos.c:33-41 and
 * find_halos.c:88-89.  S_i(x) = y_i + b_i dx + c_i dx^2 + d_i dx^3 with
 * c_0 = c_{n-1} = 0; the interior c solve the tridiagonal system
 *   h_{i-1} c_{i-1} + 2 (h_{i-1} + h_i) c_i + h_i c_{i+1}
 *       = 3 ((y_{i+1} - y_i)/h_i - (y_i - y_{i-1})/h_{i-1})
 * (forward elimination / back substitution).  b and d follow from c at
 * evaluation time. */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"

int orc_spline_init(orc_spline *s, const double *x, const double *y, int n) {
  memset(s, 0, sizeof(*s));
  if (n < 3) return 1;
  for (int i = 0; i + 1 < n; i++)
    if (!(x[i + 1] > x[i])) return 2;          /* GSL rejects non-increasing x */
  s->n = n;
  s->x = (double *)malloc(sizeof(double) * n);
  s->y = (double *)malloc(sizeof(double) * n);
  s->c = (double *)calloc(n, sizeof(double));
  if (!s->x || !s->y || !s->c) { orc_spline_free(s); return 3; }
  memcpy(s->x, x, sizeof(double) * n);
  memcpy(s->y, y, sizeof(double) * n);
  int m = n - 2;                               /* interior unknowns c_1..c_{n-2} */
  double *diag = (double *)malloc(sizeof(double) * m);
  double *rhs = (double *)malloc(sizeof(double) * m);
  double *off = (double *)malloc(sizeof(double) * m);
  for (int i = 0; i < m; i++) {
    double h0 = x[i + 1] - x[i], h1 = x[i + 2] - x[i + 1];
    diag[i] = 2.0 * (h0 + h1);
    off[i] = h1;                               /* coupling c_{i+1} <-> c_{i+2} */
    rhs[i] = 3.0 * ((y[i + 2] - y[i + 1]) / h1 - (y[i + 1] - y[i]) / h0);
  }
  /* forward elimination of the symmetric tridiagonal system */
  for (int i = 1; i < m; i++) {
    double w = off[i - 1] / diag[i - 1];
    diag[i] = diag[i] - w * off[i - 1];
    rhs[i] = rhs[i] - w * rhs[i - 1];
  }
  if (m > 0) s->c[m] = rhs[m - 1] / diag[m - 1];
  for (int i = m - 2; i >= 0; i--) s->c[i + 1] = (rhs[i] - off[i] * s->c[i + 2]) / diag[i];
  free(diag); free(rhs); free(off);
  return 0;
}

void orc_spline_free(orc_spline *s) {
  free(s->x); free(s->y); free(s->c);
  memset(s, 0, sizeof(*s));
}

double orc_spline_eval(const orc_spline *s, double x, int *status) {
  if (x < s->x[0] || x > s->x[s->n - 1]) { if (status) *status = 1; return NAN; }
  /* interval search: largest i with x_i <= x, clamped to n-2 */
  size_t lo = 0, hi = (size_t)s->n - 1;
  while (hi > lo + 1) {
    size_t mid = (hi + lo) / 2;
    if (s->x[mid] > x) hi = mid; else lo = mid;
  }
  double xl = s->x[lo], dx = s->x[lo + 1] - xl;
  double dy = s->y[lo + 1] - s->y[lo];
  double c0 = s->c[lo], c1 = s->c[lo + 1];
  double b = dy / dx - dx * (c1 + 2.0 * c0) / 3.0;
  double d = (c1 - c0) / (3.0 * dx);
  double t = x - xl;
  return s->y[lo] + t * (b + t * (c0 + t * d));
}
