/* Declarations of the GSL random-number API that the reference's MC layer calls
 * (src/Replica.cpp:302-336, src/Simulation.cpp:5-7, src/Molecule.cpp:210-464), for
 * building that layer as a checker.  TEST INFRASTRUCTURE ONLY.  GSL itself is not used:
 * oracle/ref_rng.cpp implements these calls so that they hand the reference code the
 * draws of the GB300 engine's Philox protocol (see that file). */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gsl_rng_type gsl_rng_type;
typedef struct gsl_rng gsl_rng;

extern const gsl_rng_type *gsl_rng_mt19937;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long int s);
void gsl_rng_free(gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);
unsigned long int gsl_rng_uniform_int(const gsl_rng *r, unsigned long int n);

#ifdef __cplusplus
}
#endif
