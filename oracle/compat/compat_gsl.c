/* Oracle compat shim (test infrastructure): GSL subset used by genetIC, restated.
 *  - gsl_rng ranlxs2 -> oracle_ranlux (RANLUX luxury 2, 24-bit outputs, max 2^24-1)
 *  - gsl_ran_gaussian_ziggurat -> oracle_gaussian_ziggurat scaled by sigma
 *  - gsl_spline cspline -> natural cubic spline (second-derivative form, Thomas solve)
 * Call sites: genetIC/src/simulation/field/randomfieldgenerator.hpp:43-45,149-150,191,228-241;
 * genetIC/src/tools/numerics/interpolation.hpp:49-75. */
#include "gsl/gsl_rng.h"
#include "gsl/gsl_randist.h"
#include "gsl/gsl_spline.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static const gsl_rng_type ranlxs2_type = {"ranlxs2", 0xFFFFFFUL, 0UL, 397u};
const gsl_rng_type *gsl_rng_ranlxs2 = &ranlxs2_type;
const gsl_rng_type *gsl_rng_ranlxd2 = &ranlxs2_type; /* named in a comment only */

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) {
  gsl_rng *r = (gsl_rng *)calloc(1, sizeof(gsl_rng));
  r->type = T;
  oracle_ranlux_seed(&r->state, 0, T->luxury);
  return r;
}
void gsl_rng_set(const gsl_rng *r, unsigned long int seed) {
  oracle_ranlux_seed((oracle_ranlux *)&r->state, seed, r->type->luxury);
}
void gsl_rng_free(gsl_rng *r) { free(r); }
unsigned long int gsl_rng_get(const gsl_rng *r) {
  return oracle_ranlux_next((oracle_ranlux *)&r->state);
}
double gsl_rng_uniform(const gsl_rng *r) {
  return oracle_ranlux_uniform((oracle_ranlux *)&r->state);
}
double gsl_ran_gaussian_ziggurat(const gsl_rng *r, double sigma) {
  return sigma * oracle_gaussian_ziggurat((oracle_ranlux *)&r->state);
}

static const gsl_interp_type cspline_type = {"cspline"};
const gsl_interp_type *gsl_interp_cspline = &cspline_type;

gsl_interp_accel *gsl_interp_accel_alloc(void) { return (gsl_interp_accel *)calloc(1, sizeof(gsl_interp_accel)); }
void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }

gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t size) {
  (void)T;
  gsl_spline *s = (gsl_spline *)calloc(1, sizeof(gsl_spline));
  s->size = size;
  s->x = (double *)calloc(size, sizeof(double));
  s->y = (double *)calloc(size, sizeof(double));
  s->c = (double *)calloc(size, sizeof(double));
  return s;
}

/* Natural cubic spline: c_0 = c_{n-1} = 0 and, for 0<i<n-1,
 * h_{i-1} c_{i-1} + 2 (h_{i-1}+h_i) c_i + h_i c_{i+1} = 3 (dy_i/h_i - dy_{i-1}/h_{i-1}). */
int gsl_spline_init(gsl_spline *s, const double xa[], const double ya[], size_t n) {
  memcpy(s->x, xa, n * sizeof(double));
  memcpy(s->y, ya, n * sizeof(double));
  for (size_t i = 0; i < n; ++i) s->c[i] = 0.0;
  if (n < 3) return 0;
  size_t m = n - 2;
  double *diag = (double *)malloc(m * sizeof(double));
  double *off = (double *)malloc(m * sizeof(double));
  double *rhs = (double *)malloc(m * sizeof(double));
  for (size_t i = 0; i < m; ++i) {
    double h0 = xa[i + 1] - xa[i], h1 = xa[i + 2] - xa[i + 1];
    double g0 = h0 != 0.0 ? 1.0 / h0 : 0.0, g1 = h1 != 0.0 ? 1.0 / h1 : 0.0;
    off[i] = h1;
    diag[i] = 2.0 * (h0 + h1);
    rhs[i] = 3.0 * ((ya[i + 2] - ya[i + 1]) * g1 - (ya[i + 1] - ya[i]) * g0);
  }
  /* symmetric tridiagonal solve (forward elimination, back substitution) */
  for (size_t i = 1; i < m; ++i) {
    double w = off[i - 1] / diag[i - 1];
    diag[i] -= w * off[i - 1];
    rhs[i] -= w * rhs[i - 1];
  }
  s->c[m] = rhs[m - 1] / diag[m - 1];
  for (size_t i = m - 1; i-- > 0;)
    s->c[i + 1] = (rhs[i] - off[i] * s->c[i + 2]) / diag[i];
  free(diag); free(off); free(rhs);
  return 0;
}

double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a) {
  (void)a;
  size_t lo = 0, hi = s->size - 1;
  if (x < s->x[0] || x > s->x[hi]) return NAN;
  while (hi > lo + 1) {
    size_t mid = (lo + hi) / 2;
    if (s->x[mid] > x) hi = mid; else lo = mid;
  }
  double h = s->x[lo + 1] - s->x[lo];
  double dx = x - s->x[lo];
  double dy = s->y[lo + 1] - s->y[lo];
  double ci = s->c[lo], ci1 = s->c[lo + 1];
  double b = dy / h - h * (ci1 + 2.0 * ci) / 3.0;
  double d = (ci1 - ci) / (3.0 * h);
  return s->y[lo] + dx * (b + dx * (ci + dx * d));
}

void gsl_spline_free(gsl_spline *s) {
  if (!s) return;
  free(s->x); free(s->y); free(s->c); free(s);
}
