/* REFERENCE BUILD — test infrastructure only.  Stand-in for the GSL random
 * distributions the reference calls (src/exshalos/density_grid.c:173-184):
 * the polar-method Gaussian and the flat distribution (oracle/orc_rng.c). */
#ifndef EXH_REF_GSL_RANDIST_H
#define EXH_REF_GSL_RANDIST_H
#include "gsl_rng.h"

double gsl_ran_gaussian(const gsl_rng *r, double sigma);
double gsl_ran_flat(const gsl_rng *r, double a, double b);

#endif
