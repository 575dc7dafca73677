/* Oracle (test infrastructure only): see oracle_rng.h for what this restates. */
#include "oracle_rng.h"
#include "zig_tables.h"
#include <math.h>
#include <string.h>
#include <stdlib.h>
#if !defined(__aarch64__)
#include <quadmath.h>
#endif

/* log() for the ziggurat tail.  Mode 0 (default): the C library's log, as GSL
 * calls it -- what genetIC gets on a glibc system.  Mode 1: the correctly
 * rounded value, from a quad-precision log rounded once (glibc's log is one
 * ulp off for about 0.08% of the 2^24 possible arguments).  The GPU parity
 * tests use mode 1. */
static int g_cr_log = 0;
void oracle_rng_set_cr_log(int on) { g_cr_log = on; }
static double tail_log(double u) {
  if (!g_cr_log) return log(u);
#if defined(__aarch64__)
  return (double)logl((long double)u);  /* binary128 on this target */
#else
  return (double)logq((__float128)u);
#endif
}

#define W48 ((uint64_t)1 << 48)
#define M24 0xFFFFFFu

/* Luescher's seeding: 31-bit shift register x_k = x_{k-31} ^ x_{k-13}
 * produces 48 bits per word, most significant first. */
void oracle_ranlux_seed(oracle_ranlux *r, unsigned long seed, unsigned lux) {
  int bits[31];
  long s = (long)(seed == 0 ? 1 : seed);
  int v = (int)(s & 0xFFFFFFFFL);
  for (int k = 0; k < 31; ++k) { bits[k] = v % 2; v /= 2; }
  int ib = 0, jb = 18;
  for (int k = 0; k < 12; ++k) {
    uint64_t w = 0;
    for (int m = 0; m < 48; ++m) {
      w = 2 * w + (uint64_t)bits[ib];
      bits[ib] = (bits[ib] + bits[jb]) % 2;
      ib = (ib + 1) % 31;
      jb = (jb + 1) % 31;
    }
    r->x[k] = w;
  }
  r->ir = 0;
  r->carry = 0;
  r->lux = lux;
  r->pos = 24;
  r->drawn = 0;
}

/* lux steps of the 48-bit subtract-with-borrow, then split the 12 newest words
 * (oldest first) into 24-bit halves, low half first. */
static void ranlux_block(oracle_ranlux *r) {
  unsigned ir = r->ir, c = r->carry;
  for (unsigned k = 0; k < r->lux; ++k) {
    unsigned jr = (ir + 7) % 12;               /* x_{n-5} lives 7 slots after x_{n-12} */
    int64_t d = (int64_t)r->x[jr] - (int64_t)r->x[ir] - (int64_t)c;
    c = d < 0;
    if (d < 0) d += (int64_t)W48;
    r->x[ir] = (uint64_t)d;
    ir = (ir + 1) % 12;
  }
  r->ir = ir;
  r->carry = c;
  for (unsigned k = 0; k < 12; ++k) {
    uint64_t w = r->x[(ir + k) % 12];
    r->out[2 * k] = (uint32_t)(w & M24);
    r->out[2 * k + 1] = (uint32_t)(w >> 24);
  }
  r->pos = 0;
}

uint32_t oracle_ranlux_next(oracle_ranlux *r) {
  if (r->pos >= 24) ranlux_block(r);
  r->drawn++;
  return r->out[r->pos++];
}

double oracle_ranlux_uniform(oracle_ranlux *r) {
  return (double)oracle_ranlux_next(r) / 16777216.0;
}

double oracle_gaussian_ziggurat(oracle_ranlux *r) {
  for (;;) {
    uint32_t k1 = oracle_ranlux_next(r);
    uint32_t k2 = oracle_ranlux_next(r);
    unsigned i = k1 & 0xFFu;
    uint32_t j = k2 & M24;
    int sign = (i & 0x80u) ? 1 : -1;
    i &= 0x7Fu;
    double x = (double)j * gic_zig_wtab[i];
    if (j < gic_zig_ktab[i])
      return (double)sign * x;
    double y;
    if (i < 127) {
      double y0 = gic_zig_ytab[i], y1 = gic_zig_ytab[i + 1];
      double u1 = oracle_ranlux_uniform(r);
      y = y1 + (y0 - y1) * u1;
    } else {
      double u1 = 1.0 - oracle_ranlux_uniform(r);
      double u2 = oracle_ranlux_uniform(r);
      x = GIC_ZIG_R - tail_log(u1) / GIC_ZIG_R;
      y = exp(-GIC_ZIG_R * (x - 0.5 * GIC_ZIG_R)) * u2;
    }
    if (y < exp(-0.5 * x * x))
      return (double)sign * x;
  }
}

void oracle_ranlux_stream(unsigned long seed, uint32_t *out, uint64_t n) {
  oracle_ranlux r;
  oracle_ranlux_seed(&r, seed, 397);
  for (uint64_t i = 0; i < n; ++i) out[i] = oracle_ranlux_next(&r);
}

uint64_t oracle_gaussian_stream(unsigned long seed, double *out, uint64_t n) {
  oracle_ranlux r;
  oracle_ranlux_seed(&r, seed, 397);
  for (uint64_t i = 0; i < n; ++i) out[i] = oracle_gaussian_ziggurat(&r);
  return r.drawn;
}

/* --- draw order (randomfieldgenerator.hpp:144-171, 181-197, 203-260) --- */

/* Store a complex value for integer mode (kx,ky,kz) of a real field's
 * half-spectrum, folding kz<0 onto the conjugate (fourier.hpp:300-319,439-453). */
static void set_coeff(double *f, int n, int kx, int ky, int kz, double re, double im) {
  if (kz < 0) { kx = -kx; ky = -ky; kz = -kz; im = -im; }
  if (ky < 0) ky += n;
  if (kx < 0) kx += n;
  size_t nz = (size_t)n / 2 + 1;
  size_t idx = (size_t)kz + nz * ((size_t)ky + (size_t)n * (size_t)kx);
  f[2 * idx] = re;
  f[2 * idx + 1] = im;
}

static void draw_mode(double *f, int n, int k1, int k2, int k3, double norm,
                      oracle_ranlux *r, int reverse) {
  double a = norm * oracle_gaussian_ziggurat(r);
  double b = norm * oracle_gaussian_ziggurat(r);
  double re = reverse ? b : a, im = reverse ? a : b;
  set_coeff(f, n, k1, k2, k3, re, im);
  int nyq = n / 2;
  if (k1 == 0 || k1 == nyq || k2 == 0 || k2 == nyq || k3 == 0 || k3 == nyq)
    set_coeff(f, n, -k1, -k2, -k3, re, -im);
}

static void draw_shell(double *f, int n, int ks, double norm, oracle_ranlux *r, int reverse) {
  for (int k1 = -ks; k1 < ks; ++k1)
    for (int k2 = -ks; k2 < ks; ++k2) {
      draw_mode(f, n, ks, k1, k2, norm, r, reverse);
      draw_mode(f, n, k1, ks, k2, norm, r, reverse);
      draw_mode(f, n, k1, k2, ks, norm, r, reverse);
    }
}

/* Several levels, as RandomFieldGenerator::draw loops over them
 * (randomfieldgenerator.hpp:122-139): real-space and serial Fourier modes keep
 * drawing from one stream, the parallel mode reseeds each shell on each level. */
int oracle_draw_white_noise_levels(int nlev, const int *ns, unsigned long seed, int mode, double **outs) {
  oracle_ranlux r;
  const double norm = 1.0 / sqrt(2.0);
  if (mode == 2) {
    for (int l = 0; l < nlev; ++l)
      if (oracle_draw_white_noise(ns[l], seed, 2, outs[l])) return -1;
    return 0;
  }
  oracle_ranlux_seed(&r, seed, 397);
  for (int l = 0; l < nlev; ++l) {
    int n = ns[l];
    if (mode == 0) {
      size_t m = (size_t)n * n * n;
      for (size_t i = 0; i < m; ++i) outs[l][i] = oracle_gaussian_ziggurat(&r);
    } else if (mode == 1 || mode == 3) {
      memset(outs[l], 0, 2 * (size_t)n * n * (n / 2 + 1) * sizeof(double));
      for (int ks = 0; ks < n / 2; ++ks) draw_shell(outs[l], n, ks, norm, &r, mode == 3);
    } else {
      return -1;
    }
  }
  return 0;
}

int oracle_draw_white_noise(int n, unsigned long seed, int mode, double *out) {
  if (n <= 0) return -1;
  oracle_ranlux r;
  const double norm = 1.0 / sqrt(2.0);
  size_t ncomplex = (size_t)n * n * (n / 2 + 1);
  if (mode == 0) {
    oracle_ranlux_seed(&r, seed, 397);
    size_t m = (size_t)n * n * n;
    for (size_t i = 0; i < m; ++i) out[i] = oracle_gaussian_ziggurat(&r);
    return 0;
  }
  memset(out, 0, 2 * ncomplex * sizeof(double));
  if (mode == 1 || mode == 3) {
    oracle_ranlux_seed(&r, seed, 397);
    for (int ks = 0; ks < n / 2; ++ks) draw_shell(out, n, ks, norm, &r, mode == 3);
    return 0;
  }
  if (mode == 2) {
    for (int ks = 0; ks < n / 2; ++ks) {
      oracle_ranlux_seed(&r, seed + (unsigned long)ks, 397);
      draw_shell(out, n, ks, norm, &r, 0);
    }
    return 0;
  }
  return -1;
}
