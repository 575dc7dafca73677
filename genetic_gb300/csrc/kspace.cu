// Power spectrum and fused k-space kernels.
//
// Transfer function: genetIC reads a CAMB table, normalises each species column
// by the first row's column 1 and interpolates ln T against ln k with a natural
// cubic spline, returning 0 outside the table
// (genetIC/src/cosmology/camb.hpp:224-268, genetIC/src/tools/numerics/interpolation.hpp:81-110).
// P(k) = A k^ns T(k)^2 with A = (sigma8 / sigma8_pre * D(a)/D(1))^2, sigma8_pre
// from a 50 000-step Riemann sum over a top-hat window of radius 8 Mpc/h
// (camb.hpp:289-328).  On a grid: P_grid = P(k) (2 pi / L)^3 / (2 pi)^3 N^3
// (camb.hpp:101-139) and the field is multiplied by P_grid^0.5 (field.hpp:394-412).
//
// GB300 layout choice: P_grid depends on k only through the integer
// q = kx^2 + ky^2 + kz^2 <= 3 (N/2)^2, so sqrt(P_grid) is tabulated once per
// grid by q (196 609 doubles at N = 512, resident in L2) and every k-space
// kernel reads it with one lookup instead of evaluating the spline per cell.
#include "gic_internal.h"
#include <cmath>
#include <vector>

namespace gic {
namespace {

// Natural cubic spline (second-derivative form): c[i] (= y''/2) at the knots from the
// tridiagonal system, solved on the host (n ~ 10^3: microseconds) and uploaded.
void spline_solve_host(const std::vector<double> &x, const std::vector<double> &y, std::vector<double> &c) {
  const int n = (int)x.size();
  c.assign(n, 0.0);
  if (n < 3) return;
  const int m = n - 2;
  std::vector<double> diag(m), off(m), rhs(m);
  for (int i = 0; i < m; ++i) {
    double h0 = x[i + 1] - x[i], h1 = x[i + 2] - x[i + 1];
    double g0 = h0 != 0.0 ? 1.0 / h0 : 0.0, g1 = h1 != 0.0 ? 1.0 / h1 : 0.0;
    off[i] = h1;
    diag[i] = 2.0 * (h0 + h1);
    rhs[i] = 3.0 * ((y[i + 2] - y[i + 1]) * g1 - (y[i + 1] - y[i]) * g0);
  }
  for (int i = 1; i < m; ++i) {
    double w = off[i - 1] / diag[i - 1];
    diag[i] -= w * off[i - 1];
    rhs[i] -= w * rhs[i - 1];
  }
  c[m] = rhs[m - 1] / diag[m - 1];
  for (int i = m - 1; i-- > 0;) c[i + 1] = (rhs[i] - off[i] * c[i + 2]) / diag[i];
}

uint64_t fnv1a(uint64_t h, const void *data, size_t bytes) {
  const unsigned char *p = static_cast<const unsigned char *>(data);
  for (size_t i = 0; i < bytes; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

__device__ double spline_eval(const double *x, const double *y, const double *c, int n, double v) {
  if (v < x[0] || v > x[n - 1]) return 0.0;
  int lo = 0, hi = n - 1;
  while (hi > lo + 1) {
    int mid = (lo + hi) >> 1;
    if (x[mid] > v) hi = mid; else lo = mid;
  }
  double h = x[lo + 1] - x[lo];
  double dx = v - x[lo];
  double dy = y[lo + 1] - y[lo];
  double ci = c[lo], ci1 = c[lo + 1];
  double b = dy / h - h * (ci1 + 2.0 * ci) / 3.0;
  double d = (ci1 - ci) / (3.0 * h);
  return y[lo] + dx * (b + dx * (ci + dx * d));
}

// T(k) from the log-log spline, zero outside the table
__device__ double transfer_at(const double *lx, const double *ly, const double *c, int n, double k) {
  double l = log(k);
  if (l < lx[0] || l > lx[n - 1]) return 0.0;
  return exp(spline_eval(lx, ly, c, n, l));
}

// terms of calculateLinearVarianceInSphere's sum (camb.hpp:300-328) at the host-accumulated k_i
__global__ void k_sigma8_terms(const double *ks, int cnt, double ns, double radius, const double *lx,
                               const double *ly, const double *c, int n, double *partial) {
  __shared__ double red[256];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
    double k = ks[i];
    double t = transfer_at(lx, ly, c, n, k);
    double kr = k * radius;
    double w = (sin(kr) - kr * cos(kr)) / (kr * kr * kr);
    acc += pow(k, ns + 2.) * w * w * t * t;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// P_grid^power by q (applyTransferFunction, field.hpp:394-412: cov^power where cov != 0);
// fundamental_one: the k = 0 value set to 1 first, as spliceOneLevel's preconditioner
__global__ void k_sqrtp_table(double *tab, long long nq, double kmin, double amplitude, double ns, double norm,
                              const double *lx, const double *ly, const double *c, int n, double power = 0.5,
                              int fundamental_one = 0) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  double k = sqrt((double)q) * kmin;
  double p = 0.0;
  if (k != 0.0) {
    double t = transfer_at(lx, ly, c, n, k);
    p = amplitude * pow(k, ns) * t * t;
  }
  double spec = p * norm;
  if (q == 0 && fundamental_one) spec = 1.0;
  if (spec != 0.0 && power != 1.0) spec = pow(spec, power);
  tab[q] = spec;
}

template <typename T> struct V2;
template <> struct V2<float> { using type = float2; };
template <> struct V2<double> { using type = double2; };

// delta = w sqrt(P); psi_i = i k_i delta / k^2, zero at k = 0 and at the
// positive Nyquist component (zeldovich.hpp:155-181)
// (outputs: delta may be null; px, py, pz are all null or all set)
template <typename T>
__global__ void k_za_fields(const typename V2<T>::type *noise, const T *tab, int n, T kmin,
                            typename V2<T>::type *delta, typename V2<T>::type *px, typename V2<T>::type *py,
                            typename V2<T>::type *pz) {
  using C = typename V2<T>::type;
  const int H = n / 2, S = H + 1;
  unsigned row;
  int iz;
  if (!hs_cell(n, row, iz)) return;
  int ix = (int)(row / (unsigned)n), iy = (int)(row % (unsigned)n);
  size_t id = (size_t)row * S + iz;
  int kx = ix > H ? ix - n : ix;
  int ky = iy > H ? iy - n : iy;
  int kz = iz;
  long long q = (long long)kx * kx + (long long)ky * ky + (long long)kz * kz;
  T s = (T)tab[q];
  C w = noise[id];
  C d;
  d.x = w.x * s;
  d.y = w.y * s;
  if (delta) delta[id] = d;
  if (!px) return;
  T fx = (T)kx * kmin, fy = (T)ky * kmin, fz = (T)kz * kmin;
  T kk = fx * fx + fy * fy + fz * fz;
  C base;
  base.x = -d.y / kk;
  base.y = d.x / kk;
  C z;
  z.x = 0;
  z.y = 0;
  C rx = z, ry = z, rz = z;
  if (q != 0) {
    if (kx != H) { rx.x = base.x * fx; rx.y = base.y * fx; }
    if (ky != H) { ry.x = base.x * fy; ry.y = base.y * fy; }
    if (kz != H) { rz.x = base.x * fz; rz.y = base.y * fz; }
  }
  px[id] = rx;
  py[id] = ry;
  pz[id] = rz;
}

// Second derivatives of the potential (nabla^2 phi = delta): phi_ab = k_a k_b delta / k^2
// for ab = xx, yy, zz, xy, xz, yz, delta = src * tab[q]; zero at k = 0, and the
// mixed ones where either component is the Nyquist mode.
template <typename C>
struct SixFields {
  C *p[6];
};
template <typename T>
__global__ void k_hessian_fields(const typename V2<T>::type *src, const T *tab, int n, T kmin,
                                 SixFields<typename V2<T>::type> out) {
  using C = typename V2<T>::type;
  const int H = n / 2, S = H + 1;
  unsigned row;
  int iz;
  if (!hs_cell(n, row, iz)) return;
  int ix = (int)(row / (unsigned)n), iy = (int)(row % (unsigned)n);
  size_t id = (size_t)row * S + iz;
  int kc[3] = {ix > H ? ix - n : ix, iy > H ? iy - n : iy, iz};
  long long q = (long long)kc[0] * kc[0] + (long long)kc[1] * kc[1] + (long long)kc[2] * kc[2];
  T f[3] = {(T)kc[0] * kmin, (T)kc[1] * kmin, (T)kc[2] * kmin};
  T kk = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
  C w = src[id];
  T s = q == 0 ? (T)0 : (T)tab[q] / kk;
  const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    int a = pa[c], b = pb[c];
    T m = s * f[a] * f[b];
    if (a != b && (kc[a] == H || kc[b] == H)) m = 0;
    C o;
    o.x = w.x * m;
    o.y = w.y * m;
    out.p[c][id] = o;
  }
}

// S = xx yy + xx zz + yy zz - xy^2 - xz^2 - yz^2 over padded real rows, into xx
template <typename T>
__global__ void k_lpt2_source(T *xx, const T *yy, const T *zz, const T *xy, const T *xz, const T *yz, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T a = xx[i], b = yy[i], c = zz[i], d = xy[i], e = xz[i], f = yz[i];
  xx[i] = a * b + a * c + b * c - d * d - e * e - f * f;
}

__global__ void k_table_to_float(float *out, const double *in, long long nq) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq) out[q] = (float)in[q];
}

__global__ void k_table_scale(double *t, long long nq, double s) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nq) t[q] *= s;
}

// Per-|k|^2 tables: out[q] = base[q] * f(sqrt(q) kmin), f = 1, the low-pass Fermi
// filter 1/(1 + exp((k - kcut)/T)) with T = 0.1 kcut, or the complementary
// high-pass sqrt(1 - LP^2) (genetIC/src/simulation/filters/filter.hpp:208-275,
// filterfamily.hpp:106-140 with FRACTIONAL_K_SPLIT = 0.3, FRACTIONAL_FILTER_TEMPERATURE = 0.1).
__global__ void k_filter_table(double *out, const double *base, long long nq, double kmin, double kcut, int kind) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  double f = 1.0;
  if (kind != 0) {
    double k = sqrt((double)q) * kmin;
    double temperature = kcut * 0.1;
    double lp = 1. / (1. + exp((k - kcut) / temperature));
    f = kind == 1 ? lp : sqrt(1. - lp * lp);
  }
  out[q] = (base ? base[q] : 1.0) * f;
}

// multiply a half spectrum by tab[|k|^2]
inline dim3 hs_grid(int n) { return dim3((unsigned)((hs_elements(n) + 255) / 256)); }
inline dim3 hs_block() { return dim3(256); }

template <typename T>
__global__ void k_scale_table(typename V2<T>::type *c, int n, const double *tab) {
  const int H = n / 2, S = H + 1;
  unsigned row;
  int iz;
  if (!hs_cell(n, row, iz)) return;
  int ix = (int)(row / (unsigned)n), iy = (int)(row % (unsigned)n);
  size_t id = (size_t)row * S + iz;
  long long kx = ix > H ? ix - n : ix, ky = iy > H ? iy - n : iy;
  T s = (T)tab[kx * kx + ky * ky + (long long)iz * iz];
  c[id].x *= s;
  c[id].y *= s;
}

// Carroll, Press & Turner growth-factor fit, as genetIC evaluates it
// (genetIC/src/cosmology/parameters.hpp:55-70), on the host: a scalar.
double growth_factor(double a, double Om, double Ol) {
  double Hsq = Om / powf((float)a, 3.0f) + (1. - Om - Ol) / a / a + Ol;
  double d = 2.5 * a * Om / pow(a, 3.0) / Hsq /
             (pow(Om / Hsq / a / a / a, 4.f / 7.f) - Ol / Hsq + (1. + 0.5 * Om / pow(a, 3.0) / Hsq) * (1. + 1. / 70. * Ol / Hsq));
  return d;
}

}  // namespace

double Level::kmin() const { return 2. * M_PI / box; }

void transfer_setup(Context &ctx, const double *table, int nrows, int ncols) {
  if (!ctx.have_cosmo) fail(GIC_ERR_NOT_READY, "set the cosmology before the transfer function");
  if (ncols != 7 && ncols != 13) fail(GIC_ERR_INVALID_ARG, "CAMB transfer file doesn't have a sensible number of columns");
  if (nrows < 2) fail(GIC_ERR_INVALID_ARG, "transfer table too short");
  Transfer &T = ctx.transfer;
  // an unchanged table and cosmology leave the state as it is (callers re-upload the
  // same table once per realisation)
  uint64_t h = 1469598103934665603ull;
  h = fnv1a(h, &nrows, sizeof nrows);
  h = fnv1a(h, &ncols, sizeof ncols);
  h = fnv1a(h, table, (size_t)nrows * ncols * sizeof(double));
  h = fnv1a(h, &ctx.cosmo, sizeof ctx.cosmo);
  if (T.ready && T.inputs_hash == h) return;
  T.ready = false;
  // species columns: dm -> 1, all -> 6; normalised by the first row's column 1
  double tnorm = table[1];
  std::vector<double> k, tall, tdm;
  for (int j = 0; j < nrows; ++j) {
    if (table[(size_t)ncols * j] > 0) {
      k.push_back(table[(size_t)ncols * j]);
      tdm.push_back(table[(size_t)ncols * j + 1] / tnorm);
      tall.push_back(table[(size_t)ncols * j + 6] / tnorm);
    }
  }
  auto logs = [](const std::vector<double> &x, const std::vector<double> &y, std::vector<double> &lx,
                 std::vector<double> &ly) {
    for (size_t i = 0; i < x.size(); ++i) {
      double a = std::log(x[i]), b = std::log(y[i]);
      if (std::isfinite(a) && std::isfinite(b)) {
        lx.push_back(a);
        ly.push_back(b);
      }
    }
  };
  std::vector<double> lx_all, ly_all, lx_dm, ly_dm;
  logs(k, tall, lx_all, ly_all);
  logs(k, tdm, lx_dm, ly_dm);
  if (lx_all.size() < 2 || lx_dm.size() < 2)
    fail(GIC_ERR_INVALID_ARG, "Could not find enough valid values in the transfer function");
  if (lx_all.size() != lx_dm.size()) fail(GIC_ERR_INVALID_ARG, "transfer columns with invalid entries are not supported");
  int n = (int)lx_all.size();
  T.nrows = n;
  cudaStream_t s = ctx.stream;
  // the spline's second derivatives: a serial recurrence, solved on the host
  std::vector<double> c_all, c_dm;
  spline_solve_host(lx_all, ly_all, c_all);
  spline_solve_host(lx_dm, ly_dm, c_dm);
  T.lnk.ensure(n * sizeof(double));
  T.lnT_all.ensure(n * sizeof(double));
  T.c_all.ensure(n * sizeof(double));
  T.lnT_dm.ensure(n * sizeof(double));
  T.c_dm.ensure(n * sizeof(double));
  GIC_CUDA(cudaMemcpyAsync(T.lnk.ptr, lx_all.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
  GIC_CUDA(cudaMemcpyAsync(T.lnT_all.ptr, ly_all.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
  GIC_CUDA(cudaMemcpyAsync(T.lnT_dm.ptr, ly_dm.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
  GIC_CUDA(cudaMemcpyAsync(T.c_all.ptr, c_all.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
  GIC_CUDA(cudaMemcpyAsync(T.c_dm.ptr, c_dm.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));

  // sigma8 before normalisation, radius 8 Mpc/h, species "all".  The k_i of
  // `for (k = kmin; k < kmax; k += dk)` are accumulated on the host exactly as written
  // (a serial recurrence); the terms are summed on the device.
  const double radius = 8.0;
  double kmax = std::min(k.back(), 200.0 / radius) * 0.999999;
  double kmin = k[0] * 1.000001;
  double dk = (kmax - kmin) / 50000.;
  const int cap = 50100;
  std::vector<double> hks;
  hks.reserve(cap);
  for (double kk = kmin; kk < kmax && (int)hks.size() < cap; kk += dk) hks.push_back(kk);
  const int count = (int)hks.size();
  DevBuf ks, partial;
  ks.ensure(std::max(count, 1) * sizeof(double));
  const int blocks = 64;
  partial.ensure(blocks * sizeof(double));
  if (count) GIC_CUDA(cudaMemcpyAsync(ks.ptr, hks.data(), count * sizeof(double), cudaMemcpyHostToDevice, s));
  k_sigma8_terms<<<blocks, 256, 0, s>>>(ks.as<double>(), count, ctx.cosmo.ns, radius, T.lnk.as<double>(),
                                        T.lnT_all.as<double>(), T.c_all.as<double>(), n, partial.as<double>());
  launched(1);
  std::vector<double> hp(blocks);
  read_small(ctx, partial.ptr, blocks * sizeof(double), hp.data());
  double sum = 0;
  for (double v : hp) sum += v;
  double amp = 9. / 2. / M_PI / M_PI;
  double sigma8_pre = std::sqrt(sum * amp * dk);
  const Cosmo &c = ctx.cosmo;
  double d_here = growth_factor(c.a, c.om, c.ol);
  double d_today = growth_factor(1. / (1. + (double)(float)0), c.om, c.ol);
  double renorm = (c.s8 / sigma8_pre) * (d_here / d_today);
  T.sigma8_pre = sigma8_pre;
  T.amplitude = renorm * renorm;
  T.lnk_min = lx_all.front();
  T.lnk_max = lx_all.back();
  T.ready = true;
  T.inputs_hash = h;
  ctx.drop_col_tables(false);
  ctx.table_cache.clear();
  for (auto &L : ctx.levels) {
    L->sqrtp.release();
    L->sqrtp_dm.release();
    L->tab_main.release();
    L->tab_lp_src.release();
    L->tab_lp.release();
    L->tab_main_f.release();
    L->tab_lp_src_f.release();
    L->tab_lp_f.release();
  }
}

void build_sqrtp_table(Context &ctx, Level &L) { build_sqrtp_table_species(ctx, L, 0); }

// sqrt(P_grid) by |k|^2 for the "all" transfer column (dm = 0) or the dark-matter column
void build_sqrtp_table_species(Context &ctx, Level &L, int dm) {
  if (!ctx.transfer.ready) fail(GIC_ERR_NOT_READY, "no transfer function");
  DevBuf &tab = dm ? L.sqrtp_dm : L.sqrtp;
  if (tab.ptr) return;
  long long half = L.n / 2;
  long long nq = 3 * half * half + 1;
  tab.ensure(nq * sizeof(double));
  double kw = 2. * M_PI / L.box;
  double norm = kw * kw * kw / pow(2.f * M_PI, 3.f) * (double)L.ncells();
  k_sqrtp_table<<<(unsigned)((nq + 255) / 256), 256, 0, ctx.stream>>>(
      tab.as<double>(), nq, L.kmin(), ctx.transfer.amplitude, ctx.cosmo.ns, norm, ctx.transfer.lnk.as<double>(),
      dm ? ctx.transfer.lnT_dm.as<double>() : ctx.transfer.lnT_all.as<double>(),
      dm ? ctx.transfer.c_dm.as<double>() : ctx.transfer.c_all.as<double>(), ctx.transfer.nrows);
  launched();
}

// k_cut of the filter between level l-1 and l: 0.3 * N_{l-1} * kmin_{l-1}
static double level_kcut(const Level &coarse) { return 0.3 * ((double)coarse.n * coarse.kmin()); }

// tab_main = sqrt(P) (level 0) or sqrt(P) * HP(k_cut of the level above) (zoom levels)
static void build_level_tables(Context &ctx, int li) {
  Level &L = *ctx.levels[li];
  build_sqrtp_table(ctx, L);
  if (L.tab_main.ptr) return;
  long long half = L.n / 2, nq = 3 * half * half + 1;
  L.tab_main.ensure(nq * sizeof(double));
  double kcut = li > 0 ? level_kcut(*ctx.levels[li - 1]) : 1.0;
  k_filter_table<<<(unsigned)((nq + 255) / 256), 256, 0, ctx.stream>>>(L.tab_main.as<double>(), L.sqrtp.as<double>(),
                                                                       nq, L.kmin(), kcut, li > 0 ? 2 : 0);
  L.tab_main_f.ensure(nq * sizeof(float));
  k_table_to_float<<<(unsigned)((nq + 255) / 256), 256, 0, ctx.stream>>>(L.tab_main_f.as<float>(), L.tab_main.as<double>(),
                                                                         nq);
  launched(2);
}

// on the coarse level l-1: sqrt(P) * LP and LP alone, for the copy into level l
static void build_lowpass_tables(Context &ctx, int coarse_index) {
  Level &C = *ctx.levels[coarse_index];
  build_sqrtp_table(ctx, C);
  if (C.tab_lp_src.ptr) return;
  long long half = C.n / 2, nq = 3 * half * half + 1;
  C.tab_lp_src.ensure(nq * sizeof(double));
  C.tab_lp.ensure(nq * sizeof(double));
  double kcut = level_kcut(C);
  unsigned blocks = (unsigned)((nq + 255) / 256);
  k_filter_table<<<blocks, 256, 0, ctx.stream>>>(C.tab_lp_src.as<double>(), C.sqrtp.as<double>(), nq, C.kmin(), kcut, 1);
  k_filter_table<<<blocks, 256, 0, ctx.stream>>>(C.tab_lp.as<double>(), nullptr, nq, C.kmin(), kcut, 1);
  C.tab_lp_src_f.ensure(nq * sizeof(float));
  C.tab_lp_f.ensure(nq * sizeof(float));
  k_table_to_float<<<blocks, 256, 0, ctx.stream>>>(C.tab_lp_src_f.as<float>(), C.tab_lp_src.as<double>(), nq);
  k_table_to_float<<<blocks, 256, 0, ctx.stream>>>(C.tab_lp_f.as<float>(), C.tab_lp.as<double>(), nq);
  launched(4);
  // the low-pass multiplies the coarse level's x passes (zoom combination)
  ctx.register_col_table(C.tab_lp.ptr, C.n, (int)sizeof(double), false);
  ctx.register_col_table(C.tab_lp_f.ptr, C.n, (int)sizeof(float), false);
}

template <>
const double *tab_main<double>(const Level &L) { return L.tab_main.as<double>(); }
template <>
const float *tab_main<float>(const Level &L) { return L.tab_main_f.as<float>(); }
template <>
const double *tab_lp_src<double>(const Level &L) { return L.tab_lp_src.as<double>(); }
template <>
const float *tab_lp_src<float>(const Level &L) { return L.tab_lp_src_f.as<float>(); }
template <>
const double *tab_lp<double>(const Level &L) { return L.tab_lp.as<double>(); }
template <>
const float *tab_lp<float>(const Level &L) { return L.tab_lp_f.as<float>(); }

template <>
const double *typed_table<double>(Context &, DevBuf &, const double *tab, size_t) { return tab; }
template <>
const float *typed_table<float>(Context &ctx, DevBuf &shadow, const double *tab, size_t nq) {
  shadow.ensure(nq * sizeof(float));
  k_table_to_float<<<(unsigned)((nq + 255) / 256), 256, 0, ctx.stream>>>(shadow.as<float>(), tab, (long long)nq);
  launched();
  return shadow.as<float>();
}

// the fields of `mask` (bit f: field f; kFieldDelta, kFieldsPsi) of level li in real space
template <typename T>
static void za_fields_typed(Context &ctx, int li, unsigned mask) {
  using C = typename V2<T>::type;
  Level &L = *ctx.levels[li];
  size_t nc = L.ncomplex();
  for (int f = 0; f < 4; ++f) L.field[f].ensure(nc * sizeof(C));
  build_level_tables(ctx, li);
  auto out = [&](int f) { return (mask >> f) & 1u ? L.field[f].as<C>() : nullptr; };
  k_za_fields<T><<<hs_grid(L.n), hs_block(), 0, ctx.stream>>>(L.noise.as<C>(), tab_main<T>(L), L.n, (T)L.kmin(),
                                                 out(0), out(1), out(2), out(3));
  launched();
  double scale = 1.0 / std::pow((double)L.n, 1.5);
  for (int f = 0; f < 4; ++f)
    if ((mask >> f) & 1u) fft_c2r_3d<T>(ctx, L.field[f].as<T>(), L.n, scale);
  if (mask & kFieldsPsi) {
    L.have_fields = true;
    L.have_delta = false;
  }
  if (mask & kFieldDelta) L.have_delta = true;
}

template <typename T>
void interp_add_fields(Context &ctx, const Level &coarse, T *const src[4], Level &fine, unsigned mask);

// low-passed level li-1 (the fields of `mask`) in real space, interpolated into level li
template <typename T>
static void zoom_combine_typed(Context &ctx, int li, unsigned mask) {
  using C = typename V2<T>::type;
  Level &Cl = *ctx.levels[li - 1];
  Level &F = *ctx.levels[li];
  size_t nc = Cl.ncomplex();
  for (int f = 0; f < 4; ++f) ctx.zoom_scratch[f].ensure(nc * sizeof(C));
  T *src[4];
  for (int f = 0; f < 4; ++f) src[f] = ctx.zoom_scratch[f].as<T>();
  build_lowpass_tables(ctx, li - 1);
  double scale = 1.0 / std::pow((double)Cl.n, 1.5);
  if (li - 1 == 0) {
    // level 0 is unfiltered: its low-passed fields come straight from its noise
    auto out = [&](int f) { return (mask >> f) & 1u ? reinterpret_cast<C *>(src[f]) : nullptr; };
    k_za_fields<T><<<hs_grid(Cl.n), hs_block(), 0, ctx.stream>>>(Cl.noise.as<C>(), tab_lp_src<T>(Cl), Cl.n, (T)Cl.kmin(),
                                                   out(0), out(1), out(2), out(3));
    launched();
  } else {
    // the combined real fields of level li-1, back to Fourier space, low-passed
    for (int f = 0; f < 4; ++f) {
      if (!((mask >> f) & 1u)) continue;
      GIC_CUDA(cudaMemcpyAsync(src[f], Cl.field[f].ptr, nc * sizeof(C), cudaMemcpyDeviceToDevice, ctx.stream));
      fft_r2c_3d<T>(ctx, src[f], Cl.n, scale, tab_lp<T>(Cl));  // low-passed on the way out
    }
  }
  // the interpolation reads the coarse cells around the fine level only
  const CellBox fp = footprint_box(F, Cl, 3);
  for (int f = 0; f < 4; ++f)
    if ((mask >> f) & 1u) fft_c2r_3d<T>(ctx, src[f], Cl.n, scale, nullptr, &fp);
  interp_add_fields<T>(ctx, Cl, src, F, mask);
}

// ---- second-order LPT ------------------------------------------------------------
// No counterpart in genetIC.  psi2 = (3/7) i k S_k / k^2 with nabla^2 phi = delta and
// S = sum_{a<b} (phi_aa phi_bb - phi_ab^2) (Scoccimarro 1998; Crocce, Pueblas &
// Scoccimarro 2006, Einstein-de Sitter growth D2 = -3/7 D1^2).  On a zoom level both
// the Hessian and psi2 are combined like the first-order fields: the level's own
// part times the high-pass filter plus the coarser level's combined field
// low-passed and interpolated in.

// out[q] = scalar * (1, HP or LP filter of cut kcut)
static void filter_table(Context &ctx, DevBuf &out, const Level &L, double kcut, int kind, double scalar) {
  long long half = L.n / 2, nq = 3 * half * half + 1;
  out.ensure(nq * sizeof(double));
  unsigned blocks = (unsigned)((nq + 255) / 256);
  k_filter_table<<<blocks, 256, 0, ctx.stream>>>(out.as<double>(), nullptr, nq, L.kmin(), kcut, kind);
  launched();
  if (scalar != 1.0) {
    k_table_scale<<<blocks, 256, 0, ctx.stream>>>(out.as<double>(), nq, scalar);
    launched();
  }
}

// real fields of level li-1 (combined), low-passed, added into level li's real fields
template <typename T>
static void add_lowpassed_coarse(Context &ctx, int li, T *const *coarse, T *const *fine, int nf) {
  using C = typename V2<T>::type;
  Level &Cl = *ctx.levels[li - 1];
  Level &F = *ctx.levels[li];
  build_lowpass_tables(ctx, li - 1);
  const size_t bytes = Cl.ncomplex() * sizeof(C);
  const double scale = 1.0 / std::pow((double)Cl.n, 1.5);
  auto tmp = ctx.pool.take(bytes);
  T *t = tmp->as<T>();
  for (int f = 0; f < nf; ++f) {
    GIC_CUDA(cudaMemcpyAsync(t, coarse[f], bytes, cudaMemcpyDeviceToDevice, ctx.stream));
    fft_r2c_3d<T>(ctx, t, Cl.n, scale);
    fft_c2r_3d<T>(ctx, t, Cl.n, scale, tab_lp<T>(Cl));  // low-passed on the way back
    const T *src[1] = {t};
    T *dst[1] = {fine[f]};
    interp_add<T, 1>(ctx, Cl, src, F, dst);
  }
  ctx.pool.give(std::move(tmp));
}

template <typename T>
static void lpt2_typed(Context &ctx) {
  using C = typename V2<T>::type;
  const int nl = (int)ctx.levels.size();
  std::vector<std::vector<std::unique_ptr<DevBuf>>> hess(nl);
  std::vector<std::unique_ptr<DevBuf>> source(nl);
  // the psi2 multiplier tables are kept by the context: nothing is allocated or freed
  // per call once they have grown (a batch captures this in a CUDA graph that holds
  // the pointers)
  DevBuf &tab = ctx.lpt2_tab, &tabt = ctx.lpt2_tabt;
  // combined Hessian and the source S of every level
  for (int li = 0; li < nl; ++li) {
    Level &L = *ctx.levels[li];
    const size_t bytes = L.ncomplex() * sizeof(C);
    const double scale = 1.0 / std::pow((double)L.n, 1.5);
    build_level_tables(ctx, li);
    SixFields<C> hp{};
    for (int c = 0; c < 6; ++c) {
      hess[li].push_back(ctx.pool.take(bytes));
      hp.p[c] = hess[li][c]->as<C>();
    }
    k_hessian_fields<T><<<hs_grid(L.n), hs_block(), 0, ctx.stream>>>(L.noise.as<C>(), tab_main<T>(L), L.n,
                                                                     (T)L.kmin(), hp);
    launched();
    T *real[6];
    for (int c = 0; c < 6; ++c) {
      real[c] = hess[li][c]->as<T>();
      fft_c2r_3d<T>(ctx, real[c], L.n, scale);
    }
    if (li > 0) {
      T *coarse[6];
      for (int c = 0; c < 6; ++c) coarse[c] = hess[li - 1][c]->as<T>();
      add_lowpassed_coarse<T>(ctx, li, coarse, real, 6);
      for (auto &b : hess[li - 1]) ctx.pool.give(std::move(b));
      hess[li - 1].clear();
    }
    source[li] = ctx.pool.take(bytes);
    GIC_CUDA(cudaMemcpyAsync(source[li]->ptr, real[0], bytes, cudaMemcpyDeviceToDevice, ctx.stream));
    const size_t nreal = 2 * L.ncomplex();
    k_lpt2_source<T><<<(unsigned)((nreal + 255) / 256), 256, 0, ctx.stream>>>(
        source[li]->as<T>(), real[1], real[2], real[3], real[4], real[5], nreal);
    launched();
  }
  for (auto &b : hess[nl - 1]) ctx.pool.give(std::move(b));
  // psi2 of every level from its S, combined across levels
  for (int li = 0; li < nl; ++li) {
    Level &L = *ctx.levels[li];
    const size_t bytes = L.ncomplex() * sizeof(C);
    const double scale = 1.0 / std::pow((double)L.n, 1.5);
    for (int f = 0; f < 3; ++f) L.field2[f].ensure(bytes);
    T *sk = source[li]->as<T>();
    fft_r2c_3d<T>(ctx, sk, L.n, scale);
    double kcut = li > 0 ? level_kcut(*ctx.levels[li - 1]) : 1.0;
    filter_table(ctx, tab, L, kcut, li > 0 ? 2 : 0, 3.0 / 7.0);
    const long long nq_l = 3ll * (L.n / 2) * (L.n / 2) + 1;
    k_za_fields<T><<<hs_grid(L.n), hs_block(), 0, ctx.stream>>>(reinterpret_cast<C *>(sk),
                                                                typed_table<T>(ctx, tabt, tab.as<double>(), nq_l), L.n,
                                                                (T)L.kmin(), reinterpret_cast<C *>(sk),
                                                                L.field2[0].as<C>(), L.field2[1].as<C>(),
                                                                L.field2[2].as<C>());
    launched();
    T *real[3];
    for (int f = 0; f < 3; ++f) {
      real[f] = L.field2[f].as<T>();
      fft_c2r_3d<T>(ctx, real[f], L.n, scale);
    }
    if (li > 0) {
      Level &Cl = *ctx.levels[li - 1];
      T *coarse[3] = {Cl.field2[0].as<T>(), Cl.field2[1].as<T>(), Cl.field2[2].as<T>()};
      add_lowpassed_coarse<T>(ctx, li, coarse, real, 3);
    }
    L.have_lpt2 = true;
  }
  if (!ctx.defer_checks) GIC_CUDA(cudaStreamSynchronize(ctx.stream));
  for (auto &b : source) ctx.pool.give(std::move(b));
}

void lpt2_fields(Context &ctx) {
  for (auto &L : ctx.levels)
    if (!L->have_fields) fail(GIC_ERR_NOT_READY, "first-order fields have not been computed");
  if (ctx.dbl())
    lpt2_typed<double>(ctx);
  else
    lpt2_typed<float>(ctx);
}

// ---- operations on the drawn white noise (ic.hpp:1342-1344, 1652-1705) ----------
// op 0: w -> -w (reverse, multilevelfield.hpp:182-191); op 1: -w where 0 < k^2 < kmax^2,
// k^2 in the grid's physical units as the reference forms it (reverseSmallK);
// op 2: w -> w / |w| (enforcePowerSpectrumOneGrid, multilevelfield.hpp:498-510)
template <typename T>
__global__ void k_noise_op(typename V2<T>::type *w, int n, double kmin, int op, double k2max) {
  const int H = n / 2, S = H + 1;
  unsigned row;
  int iz;
  if (!hs_cell(n, row, iz)) return;
  int ix = (int)(row / (unsigned)n), iy = (int)(row % (unsigned)n);
  size_t id = (size_t)row * S + iz;
  typename V2<T>::type v = w[id];
  if (op == 0) {
    v.x = -v.x;
    v.y = -v.y;
  } else if (op == 1) {
    double kx = (double)(ix > H ? ix - n : ix) * kmin, ky = (double)(iy > H ? iy - n : iy) * kmin,
           kz = (double)iz * kmin;
    double k2 = kx * kx + ky * ky + kz * kz;
    if (k2 < k2max && k2 != 0) {
      v.x = -v.x;
      v.y = -v.y;
    }
  } else {
    T a = hypot(v.x, v.y);
    if (a != 0) {
      v.x /= a;
      v.y /= a;
    }
  }
  w[id] = v;
}

template <typename T>
static void noise_op_typed(Context &ctx, int op, double param) {
  using C = typename V2<T>::type;
  for (auto &Lp : ctx.levels) {
    Level &L = *Lp;
    k_noise_op<T><<<hs_grid(L.n), hs_block(), 0, ctx.stream>>>(L.noise.as<C>(), L.n, L.kmin(), op, param * param);
    launched();
    L.have_fields = L.have_lpt2 = false;
  }
  GIC_CUDA(cudaStreamSynchronize(ctx.stream));
}

void noise_op(Context &ctx, int op, double param) {
  for (auto &L : ctx.levels)
    if (!L->have_noise) fail(GIC_ERR_NOT_READY, "white noise has not been drawn");
  if (ctx.dbl()) noise_op_typed<double>(ctx, op, param);
  else noise_op_typed<float>(ctx, op, param);
}

void level_tables(Context &ctx, int li) { build_level_tables(ctx, li); }

// P_grid^power of a level ("all" transfer column), k = 0 set to 1 first (splicing)
void preconditioner_table(Context &ctx, const Level &L, double power, DevBuf &out) {
  if (!ctx.transfer.ready) fail(GIC_ERR_NOT_READY, "no transfer function");
  long long half = L.n / 2, nq = 3 * half * half + 1;
  out.ensure(nq * sizeof(double));
  double kw = 2. * M_PI / L.box;
  double norm = kw * kw * kw / pow(2.f * M_PI, 3.f) * (double)L.ncells();
  k_sqrtp_table<<<(unsigned)((nq + 255) / 256), 256, 0, ctx.stream>>>(
      out.as<double>(), nq, L.kmin(), ctx.transfer.amplitude, ctx.cosmo.ns, norm, ctx.transfer.lnk.as<double>(),
      ctx.transfer.lnT_all.as<double>(), ctx.transfer.c_all.as<double>(), ctx.transfer.nrows, power, 1);
  launched();
}
void lowpass_tables(Context &ctx, int coarse_index) { build_lowpass_tables(ctx, coarse_index); }

void za_fields(Context &ctx, int li, unsigned mask) {
  Level &L = *ctx.levels[li];
  if (!L.have_noise) fail(GIC_ERR_NOT_READY, "white noise has not been drawn");
  if (ctx.dbl())
    za_fields_typed<double>(ctx, li, mask);
  else
    za_fields_typed<float>(ctx, li, mask);
}

void zoom_combine(Context &ctx, int li, unsigned mask) {
  if (li < 1) return;
  if (ctx.dbl())
    zoom_combine_typed<double>(ctx, li, mask);
  else
    zoom_combine_typed<float>(ctx, li, mask);
}

void ensure_delta(Context &ctx) {
  bool all = true;
  for (auto &L : ctx.levels) {
    if (!L->have_fields) fail(GIC_ERR_NOT_READY, "fields have not been computed");
    all = all && L->have_delta;
  }
  if (all) return;
  const int nl = (int)ctx.levels.size();
  for (int l = 0; l < nl; ++l) za_fields(ctx, l, kFieldDelta);
  for (int l = 1; l < nl; ++l) zoom_combine(ctx, l, kFieldDelta);
}

}  // namespace gic
