// Natural log of u = k / 2^24 (k = 1 .. 2^24) rounded to nearest double, for the
// exponential tail of the ziggurat sampler (x = R - log(u)/R).  The value is
// evaluated in double-double arithmetic (about 100 correct bits) and rounded
// once, so host and device agree bit for bit, and with a correctly rounded libm
// log.  Method: u = 2^e f with f in [sqrt(1/2), sqrt(2)), ln f = 2 atanh(s),
// s = (f-1)/(f+1), atanh(s) = s + s^3/3 + s^5/5 + ...  (|s| < 0.1716).
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define GIC_DD __host__ __device__ __forceinline__
#else
#define GIC_DD inline
#endif

struct dd {
  double hi, lo;
};

GIC_DD dd dd_two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double err = (a - (s - bb)) + (b - bb);
  return dd{s, err};
}
GIC_DD dd dd_fast_two_sum(double a, double b) {
  double s = a + b;
  return dd{s, b - (s - a)};
}
GIC_DD dd dd_two_prod(double a, double b) {
  double p = a * b;
  return dd{p, fma(a, b, -p)};
}
GIC_DD dd dd_add(dd a, dd b) {
  dd s = dd_two_sum(a.hi, b.hi);
  dd t = dd_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = dd_fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return dd_fast_two_sum(s.hi, s.lo);
}
GIC_DD dd dd_mul(dd a, dd b) {
  dd p = dd_two_prod(a.hi, b.hi);
  p.lo = fma(a.hi, b.lo, p.lo);
  p.lo = fma(a.lo, b.hi, p.lo);
  return dd_fast_two_sum(p.hi, p.lo);
}
GIC_DD dd dd_div_d(dd a, double b) {
  double q1 = a.hi / b;
  dd p = dd_two_prod(q1, b);
  double r = (a.hi - p.hi - p.lo + a.lo) / b;
  return dd_fast_two_sum(q1, r);
}

// ln(k / 2^24), k in [1, 2^24]
GIC_DD double gic_log_k24(uint32_t k) {
  if (k >= 16777216u) return 0.0;
  // k = 2^e2 * f, f in [1,2)
  int e2 = 31 - (int)(
#if defined(__CUDA_ARCH__)
      __clz(k)
#else
      __builtin_clz(k)
#endif
  );
  double f = (double)k / (double)(1u << e2);  // exact
  int e = e2 - 24;
  if (f > 1.4142135623730951) {
    f *= 0.5;
    e += 1;
  }
  // s = (f-1)/(f+1) in double-double; f-1 and f+1 are exact
  dd num{f - 1.0, 0.0};
  double den = f + 1.0;
  dd s = dd_div_d(num, den);
  dd s2 = dd_mul(s, s);
  // atanh series sum_{j>=0} s^(2j) / (2j+1), Horner from the tail
  dd acc{1.0 / 41.0, 0.0};
  for (int j = 19; j >= 0; --j) {
    acc = dd_mul(acc, s2);
    dd inv = dd_div_d(dd{1.0, 0.0}, (double)(2 * j + 1));
    acc = dd_add(acc, inv);
  }
  dd lnf = dd_mul(acc, s);
  lnf.hi *= 2.0;
  lnf.lo *= 2.0;
  const dd ln2{0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56};
  dd el = dd_mul(ln2, dd{(double)e, 0.0});
  dd r = dd_add(el, lnf);
  return r.hi + r.lo;
}
