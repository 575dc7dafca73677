/* Oracle (test infrastructure only): CPU restatement of the white-noise
 * random stream genetIC draws from.
 *
 * genetIC allocates GSL's `ranlxs2` generator and samples it with
 * `gsl_ran_gaussian_ziggurat` (genetIC/src/simulation/field/randomfieldgenerator.hpp:43-45,
 * 149-150, 191, 228-229).  GSL is a third-party dependency that is not part of
 * the reference tree (unpinned: CI installs the distribution's libgsl-dev,
 * .github/workflows/build-test.yaml).  This file restates the published
 * algorithms:
 *   - RANLUX, M. Luescher, Comput. Phys. Commun. 79 (1994) 100: the
 *     subtract-with-borrow x_n = x_{n-5} - x_{n-12} - c_{n-1} mod 2^48 on 48-bit
 *     words (equivalently base 2^24 with lags 10, 24), luxury level 2 = 397 word
 *     steps per block of 12 delivered words; each word delivered as two
 *     24-bit numbers; seeded through Luescher's 31-bit shift register.
 *   - the ziggurat of Marsaglia & Tsang, J. Stat. Softw. 5(8) (2000), 128-layer
 *     variant with the exponential-wedge base strip (tables: zig_tables.h).
 * Nothing in the shipped library uses this code; it is the checker.
 */
#ifndef ORACLE_RNG_H
#define ORACLE_RNG_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  uint64_t x[12];     /* ring of 48-bit words */
  unsigned ir;        /* slot holding the oldest word (next overwritten) */
  unsigned carry;     /* borrow from the previous step */
  unsigned lux;       /* word steps per delivered block */
  unsigned pos;       /* next index into out[]; 24 means "block exhausted" */
  uint32_t out[24];   /* current block of 24-bit outputs */
  uint64_t drawn;     /* number of 24-bit outputs delivered so far */
} oracle_ranlux;

/* 0: C library log in the ziggurat tail (as GSL on glibc); 1: correctly rounded log. */
void oracle_rng_set_cr_log(int on);
void oracle_ranlux_seed(oracle_ranlux *r, unsigned long seed, unsigned lux);
uint32_t oracle_ranlux_next(oracle_ranlux *r);       /* integer in [0, 2^24) */
double oracle_ranlux_uniform(oracle_ranlux *r);      /* next / 2^24 */
double oracle_gaussian_ziggurat(oracle_ranlux *r);   /* unit variance */

/* Fill `out` with n consecutive 24-bit outputs of the stream of `seed`. */
void oracle_ranlux_stream(unsigned long seed, uint32_t *out, uint64_t n);
/* Fill `out` with n consecutive unit gaussians of the stream of `seed`;
 * returns the number of 24-bit numbers consumed. */
uint64_t oracle_gaussian_stream(unsigned long seed, double *out, uint64_t n);

/* Draw white noise for one N^3 grid exactly as genetIC does, into a
 * half-spectrum array of (N, N, N/2+1) complex doubles (interleaved re,im;
 * kz fastest).  mode: 0 = real space (`random_seed_real_space`; out receives
 * N^3 real gaussians in index order instead), 1 = Fourier serial
 * (`random_seed_serial`), 2 = Fourier parallel shells (`random_seed`),
 * 3 = Fourier serial with swapped (re,im) (`seedfourier_reverse`).
 * Returns 0 on success. */
int oracle_draw_white_noise(int n, unsigned long seed, int mode, double *out);
/* The same for nlev levels of sizes ns[] (real-space mode: outs[l] receives
 * ns[l]^3 gaussians; Fourier modes: half spectra), continuing one stream across
 * levels where genetIC does. */
int oracle_draw_white_noise_levels(int nlev, const int *ns, unsigned long seed, int mode, double **outs);

#ifdef __cplusplus
}
#endif
#endif
