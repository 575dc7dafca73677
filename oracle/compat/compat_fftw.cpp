// Oracle compat shim (test infrastructure): FFTW3 subset restated as a plain
// mixed-radix Cooley-Tukey DFT.  genetIC's call sites:
// genetIC/src/tools/numerics/fourier.hpp:479-518 (r2c/c2r, in place, padded rows,
// normalised by the caller), :600-624 (complex 3-D).  c2r treats each last-axis
// line as Hermitian: the imaginary parts of its zero and Nyquist entries do not
// contribute, as for any real-output inverse DFT.
#include "fftw3.h"
#include <cmath>
#include <complex>
#include <vector>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T>
struct Line1D {
  int n;
  int sign;
  std::vector<int> factors;            // radices, product = n
  std::vector<std::complex<T>> tw;     // e^{sign 2 pi i k / n}, k < n

  Line1D(int n_, int sign_) : n(n_), sign(sign_) {
    int m = n, p = 4;
    while (m > 1) {
      while (m % p) {
        if (p == 4) p = 2; else if (p == 2) p = 3; else p += 2;
        if (p * p > m) p = m;
      }
      factors.push_back(p);
      m /= p;
    }
    tw.resize(n);
    for (int k = 0; k < n; ++k) {
      long double a = (long double)sign * 2.0L * 3.14159265358979323846264338327950288L * k / n;
      tw[k] = std::complex<T>((T)cosl(a), (T)sinl(a));
    }
  }

  // out[k] = sum_j in[j*stride] w^{jk}, recursive decimation in time
  void work(std::complex<T> *out, const std::complex<T> *in, int fstride, int istride, int level) const {
    int p = factors[level];
    int m = 1;
    for (size_t l = level + 1; l < factors.size(); ++l) m *= factors[l];
    if (m == 1) {
      for (int q = 0; q < p; ++q) out[q] = in[(size_t)q * fstride * istride];
    } else {
      for (int q = 0; q < p; ++q)
        work(out + (size_t)q * m, in + (size_t)q * fstride * istride, fstride * p, istride, level + 1);
    }
    // radix-p butterflies over the p sub-transforms of length m
    std::complex<T> tmp[64];
    std::vector<std::complex<T>> big;
    std::complex<T> *scratch = tmp;
    if (p > 64) { big.resize(p); scratch = big.data(); }
    for (int u = 0; u < m; ++u) {
      for (int q = 0; q < p; ++q) {
        std::complex<T> v = out[(size_t)q * m + u];
        scratch[q] = q ? v * tw[(size_t)q * u * fstride % n] : v;
      }
      for (int r = 0; r < p; ++r) {
        std::complex<T> acc = scratch[0];
        for (int q = 1; q < p; ++q)
          acc += scratch[q] * tw[((size_t)q * r * m * fstride) % n];
        out[(size_t)r * m + u] = acc;
      }
    }
  }

  void run(std::complex<T> *buf, std::complex<T> *tmp) const {
    if (n == 1) return;
    work(tmp, buf, 1, 1, 0);
    std::memcpy((void *)buf, (void *)tmp, sizeof(std::complex<T>) * n);
  }
};

}  // namespace

enum class Kind { R2C, C2R, C2C };

struct compat_fft_plan {
  Kind kind;
  bool single;
  int n0, n1, n2, sign;
  void *data;
};

namespace {

int g_threads = 1;

// transform along axis `ax` of a complex array of shape (a0, a1, a2)
template <typename T>
void axis_pass(std::complex<T> *d, int a0, int a1, int a2, int ax, int sign) {
  int len = ax == 0 ? a0 : ax == 1 ? a1 : a2;
  size_t stride = ax == 0 ? (size_t)a1 * a2 : ax == 1 ? (size_t)a2 : 1;
  size_t nlines = (size_t)a0 * a1 * a2 / len;
  Line1D<T> plan(len, sign);
#pragma omp parallel num_threads(g_threads)
  {
    std::vector<std::complex<T>> line(len), tmp(len);
#pragma omp for schedule(static)
    for (long long li = 0; li < (long long)nlines; ++li) {
      size_t base;
      if (ax == 2) base = (size_t)li * a2;
      else if (ax == 1) base = ((size_t)li / a2) * (size_t)a1 * a2 + ((size_t)li % a2);
      else base = (size_t)li;
      for (int k = 0; k < len; ++k) line[k] = d[base + k * stride];
      plan.run(line.data(), tmp.data());
      for (int k = 0; k < len; ++k) d[base + k * stride] = line[k];
    }
  }
}

template <typename T>
void r2c(T *data, int n0, int n1, int n2) {
  int nc = n2 / 2 + 1;
  size_t rows = (size_t)n0 * n1;
  Line1D<T> plan(n2, -1);
#pragma omp parallel num_threads(g_threads)
  {
    std::vector<std::complex<T>> line(n2), tmp(n2);
#pragma omp for schedule(static)
    for (long long r = 0; r < (long long)rows; ++r) {
      T *row = data + (size_t)r * 2 * nc;
      for (int k = 0; k < n2; ++k) line[k] = std::complex<T>(row[k], 0);
      plan.run(line.data(), tmp.data());
      for (int k = 0; k < nc; ++k) { row[2 * k] = line[k].real(); row[2 * k + 1] = line[k].imag(); }
    }
  }
  auto *c = reinterpret_cast<std::complex<T> *>(data);
  axis_pass(c, n0, n1, nc, 1, -1);
  axis_pass(c, n0, n1, nc, 0, -1);
}

template <typename T>
void c2r(T *data, int n0, int n1, int n2) {
  int nc = n2 / 2 + 1;
  auto *c = reinterpret_cast<std::complex<T> *>(data);
  axis_pass(c, n0, n1, nc, 0, +1);
  axis_pass(c, n0, n1, nc, 1, +1);
  size_t rows = (size_t)n0 * n1;
  Line1D<T> plan(n2, +1);
#pragma omp parallel num_threads(g_threads)
  {
    std::vector<std::complex<T>> line(n2), tmp(n2);
#pragma omp for schedule(static)
    for (long long r = 0; r < (long long)rows; ++r) {
      T *row = data + (size_t)r * 2 * nc;
      for (int k = 0; k < nc; ++k) line[k] = std::complex<T>(row[2 * k], row[2 * k + 1]);
      line[0] = std::complex<T>(line[0].real(), 0);
      if (n2 % 2 == 0) line[n2 / 2] = std::complex<T>(line[n2 / 2].real(), 0);
      for (int k = nc; k < n2; ++k) line[k] = std::conj(line[n2 - k]);
      plan.run(line.data(), tmp.data());
      for (int k = 0; k < n2; ++k) row[k] = line[k].real();
    }
  }
}

compat_fft_plan *make(Kind k, bool single, int n0, int n1, int n2, int sign, void *data) {
  auto *p = new compat_fft_plan;
  p->kind = k; p->single = single; p->n0 = n0; p->n1 = n1; p->n2 = n2; p->sign = sign; p->data = data;
  return p;
}

}  // namespace

extern "C" {

int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int nthreads) { g_threads = nthreads > 0 ? nthreads : 1; }

fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *, unsigned) {
  return make(Kind::R2C, false, n0, n1, n2, -1, in);
}
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *, unsigned) {
  return make(Kind::C2R, false, n0, n1, n2, +1, in);
}
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *, int sign, unsigned) {
  return make(Kind::C2C, false, n0, n1, n2, sign, in);
}
fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float *in, fftwf_complex *, unsigned) {
  return make(Kind::R2C, true, n0, n1, n2, -1, in);
}
fftwf_plan fftwf_plan_dft_c2r_3d(int n0, int n1, int n2, fftwf_complex *in, float *, unsigned) {
  return make(Kind::C2R, true, n0, n1, n2, +1, in);
}

static void execute(const compat_fft_plan *p) {
  if (p->single) {
    float *d = (float *)p->data;
    if (p->kind == Kind::R2C) r2c(d, p->n0, p->n1, p->n2);
    else if (p->kind == Kind::C2R) c2r(d, p->n0, p->n1, p->n2);
  } else {
    double *d = (double *)p->data;
    if (p->kind == Kind::R2C) r2c(d, p->n0, p->n1, p->n2);
    else if (p->kind == Kind::C2R) c2r(d, p->n0, p->n1, p->n2);
    else {
      auto *c = reinterpret_cast<std::complex<double> *>(d);
      for (int ax = 2; ax >= 0; --ax) axis_pass(c, p->n0, p->n1, p->n2, ax, p->sign);
    }
  }
}
void fftw_execute(const fftw_plan p) { execute(p); }
void fftwf_execute(const fftwf_plan p) { execute(p); }
void fftw_destroy_plan(fftw_plan p) { delete p; }
void fftwf_destroy_plan(fftwf_plan p) { delete p; }

}  // extern "C"
