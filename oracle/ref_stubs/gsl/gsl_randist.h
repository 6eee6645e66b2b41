/* Declarations of the GSL distributions the reference's MC layer calls
 * (src/Molecule.cpp:420-461, src/Replica.cpp:317-345).  TEST INFRASTRUCTURE ONLY;
 * implemented in oracle/ref_rng.cpp. */
#pragma once

#include <stddef.h>

#include "gsl_rng.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gsl_ran_discrete_t gsl_ran_discrete_t;

unsigned int gsl_ran_bernoulli(const gsl_rng *r, double p);
gsl_ran_discrete_t *gsl_ran_discrete_preproc(size_t K, const double *P);
size_t gsl_ran_discrete(const gsl_rng *r, const gsl_ran_discrete_t *g);
void gsl_ran_discrete_free(gsl_ran_discrete_t *g);

#ifdef __cplusplus
}
#endif
