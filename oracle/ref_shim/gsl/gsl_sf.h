/* REFERENCE BUILD — test infrastructure only.  Stand-in for the GSL special
 * function the reference calls (src/spectrum/powermodule.c:68,178):
 * Legendre polynomials P_l(x) by the upward three-term recurrence. */
#ifndef EXH_REF_GSL_SF_H
#define EXH_REF_GSL_SF_H
double gsl_sf_legendre_Pl(const int l, const double x);
#endif
