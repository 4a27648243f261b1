/* REFERENCE BUILD — test infrastructure only.  Stand-in for the GSL random
 * number interface the reference calls (src/exshalos/density_grid.c:89-91,
 * find_halos.c:464-472): gsl_rng_taus only, restated in oracle/orc_rng.c
 * (L'Ecuyer 1996 with GSL's documented LCG(69069) seeding). */
#ifndef EXH_REF_GSL_RNG_H
#define EXH_REF_GSL_RNG_H

typedef struct ref_gsl_rng_type { const char *name; } gsl_rng_type;
typedef struct ref_gsl_rng gsl_rng;

extern const gsl_rng_type *gsl_rng_taus;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long seed);
void gsl_rng_free(gsl_rng *r);
unsigned long gsl_rng_get(const gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);
double gsl_rng_uniform_pos(const gsl_rng *r);

#endif
