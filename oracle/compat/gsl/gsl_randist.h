/* Oracle compat shim: gsl_ran_gaussian_ziggurat (randomfieldgenerator.hpp:149-150,191). */
#ifndef COMPAT_GSL_RANDIST_H
#define COMPAT_GSL_RANDIST_H
#include "gsl_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
double gsl_ran_gaussian_ziggurat(const gsl_rng *r, double sigma);
#ifdef __cplusplus
}
#endif
#endif
