/* Oracle compat shim (test infrastructure): the subset of GSL's gsl_rng API that
 * genetIC calls (genetIC/src/simulation/field/randomfieldgenerator.hpp:29-45,64-83,115,228-241).
 * Backed by the RANLUX restatement in oracle/rng/oracle_rng.c. */
#ifndef COMPAT_GSL_RNG_H
#define COMPAT_GSL_RNG_H
#include <stddef.h>
#include "../../rng/oracle_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_rng_type {
  const char *name;
  unsigned long int max;
  unsigned long int min;
  unsigned int luxury;
} gsl_rng_type;
typedef struct gsl_rng {
  const gsl_rng_type *type;
  oracle_ranlux state;
} gsl_rng;
extern const gsl_rng_type *gsl_rng_ranlxs2;
extern const gsl_rng_type *gsl_rng_ranlxd2;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long int seed);
void gsl_rng_free(gsl_rng *r);
unsigned long int gsl_rng_get(const gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);
#ifdef __cplusplus
}
#endif
#endif
