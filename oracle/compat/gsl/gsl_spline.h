/* Oracle compat shim: natural cubic spline subset of GSL's gsl_spline API, as called by
 * genetIC/src/tools/numerics/interpolation.hpp:27-75 (gsl_interp_cspline + gsl_spline_eval
 * with a null accelerator). */
#ifndef COMPAT_GSL_SPLINE_H
#define COMPAT_GSL_SPLINE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_interp_type { const char *name; } gsl_interp_type;
extern const gsl_interp_type *gsl_interp_cspline;
typedef struct gsl_interp_accel { size_t cache; } gsl_interp_accel;
typedef struct gsl_spline {
  size_t size;
  double *x, *y, *c;   /* knots, values, half second derivatives */
} gsl_spline;
gsl_interp_accel *gsl_interp_accel_alloc(void);
void gsl_interp_accel_free(gsl_interp_accel *a);
gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t size);
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], size_t size);
double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a);
void gsl_spline_free(gsl_spline *s);
#ifdef __cplusplus
}
#endif
#endif
