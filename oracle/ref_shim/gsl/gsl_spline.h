/* REFERENCE BUILD — test infrastructure only.  Stand-in for the GSL spline
 * interface the reference calls (src/exshalos/density_grid.c:79-82,157;
 * find_halos.c:33-41,88-89,472-474): natural cubic splines only
 * (oracle/orc_spline.c).  An evaluation outside the knots, where GSL's
 * default error handler aborts, returns NaN and is counted
 * (ref_gsl_domain_errors in oracle/ref_shim.c). */
#ifndef EXH_REF_GSL_SPLINE_H
#define EXH_REF_GSL_SPLINE_H
#include <stddef.h>

typedef struct ref_gsl_interp_type { const char *name; } gsl_interp_type;
typedef struct ref_gsl_interp_accel gsl_interp_accel;
typedef struct ref_gsl_spline gsl_spline;

extern const gsl_interp_type *gsl_interp_cspline;

gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t size);
int gsl_spline_init(gsl_spline *spline, const double xa[], const double ya[], size_t size);
double gsl_spline_eval(const gsl_spline *spline, double x, gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *spline);

#endif
