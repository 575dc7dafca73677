// Linear modifications (constraints) on the white noise, as genetIC applies them
// (genetIC/src/simulation/modifications/modificationmanager.hpp:90-125, 199-217, 288-331,
//  linearmodification.hpp, multilevelgrid.hpp:245-321, multilevelfield.hpp:248-384,
//  field.hpp:752-849).
//
//  - covector of a modification: a top-hat (overdensity) or 4th-order gradient
//    stencil (velocity) over the flagged cells of the finest level, transformed
//    to Fourier space; carried to coarser levels by the transpose of the tricubic
//    interpolation (separable: three one-axis passes), weighted by the cell-volume
//    ratio, filtered by the level's filter of the zoom filter family, and
//    multiplied by sqrt(P_dm) (and by -v/k^2 for velocities);
//  - metric C (covector <-> vector): per level f_l^2 (or, towards a covector, the
//    filter applied inside/outside the next level's window) plus cross-level terms
//    f_t f_s sqrt(w_t/w_s) interpolated up or block-averaged down;
//  - inner products <a|b> = sum_l sum_k Re(conj(a) b) with Hermitian weights,
//    accumulated in double on the device;
//  - Gram-Schmidt of the covectors: the same sequence of projections as the
//    reference, evaluated through the Gram matrix G_ij = <a_i|C|a_j> (C is
//    linear), which needs one metric conversion per covector instead of one per
//    inner product; the correction sum_i d_i C a'_i is then one combination of
//    the converted covectors.
#include "gic_internal.h"
#include <atomic>
#include <cmath>
#include <algorithm>

namespace gic {
namespace {

template <typename T> struct V2m;
template <> struct V2m<float> { using type = float2; };
template <> struct V2m<double> { using type = double2; };

// --- per-|k|^2 tables ---------------------------------------------------------

// table[q] = scalar * (prod_i HP(k; hp_cut_i) * prod_j LP(k; lp_cut_j))^power
//            [* sqrtp[q]] [* -vel / k^2], k = sqrt(q) kmin
struct TableSpec {
  double kmin;
  int nhp;
  double hp_cut[8];
  int nlp;
  double lp_cut[4];
  int power;
  double scalar;
  const double *sqrtp;
  double vel;
  double var_cut;  // > 0: times 1 - LP(k; var_cut), the variance high-pass
  double offset;   // added last
};

__device__ __forceinline__ double fermi_lp(double k, double kcut) {
  double temperature = kcut * 0.1;
  return 1. / (1. + exp((k - kcut) / temperature));
}

// out: the table; outf (optional): its float copy, for float fields
__global__ void k_mod_table(double *out, float *outf, long long nq, TableSpec sp) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  double k = sqrt((double)q) * sp.kmin;
  double f = 1.0;
  for (int i = 0; i < sp.nhp; ++i) {
    double lp = fermi_lp(k, sp.hp_cut[i]);
    f *= sqrt(1. - lp * lp);
  }
  for (int i = 0; i < sp.nlp; ++i) f *= fermi_lp(k, sp.lp_cut[i]);
  if (sp.var_cut > 0) f *= 1. - fermi_lp(k, sp.var_cut);
  if (sp.power == 2) f = f * f;
  f *= sp.scalar;
  if (sp.sqrtp) f *= sp.sqrtp[q];
  if (sp.vel != 0.0) f = q == 0 ? 0.0 : -sp.vel * f / (k * k);
  f += sp.offset;
  out[q] = f;
  if (outf) outf[q] = (float)f;
}

// Half-spectrum kernels run on a 2-D grid: x over rows (kx, ky), y over 32-wide
// kz chunks, so no 64-bit division per element.
constexpr int kKzChunk = 32, kRowsPerBlock = 8;
// elementwise half-spectrum kernels: one thread per coefficient, flat (hs_cell)
inline dim3 hs_grid(int n) { return dim3((unsigned)((hs_elements(n) + 255) / 256)); }
inline dim3 hs_block() { return dim3(256); }
// reductions: warps of kKzChunk lanes walking rows, kRowsPerBlock warps per CTA
inline dim3 red_block() { return dim3(kKzChunk, kRowsPerBlock); }

template <typename T>
__global__ void k_mul_table(typename V2m<T>::type *c, int n, const T *tab) {
  const int H = n / 2, S = H + 1;
  unsigned row;
  int iz;
  if (!hs_cell(n, row, iz)) return;
  int ix = (int)(row / (unsigned)n), iy = (int)(row % (unsigned)n);
  long long kx = ix > H ? ix - n : ix, ky = iy > H ? iy - n : iy;
  T s = (T)tab[kx * kx + ky * ky + (long long)iz * iz];
  size_t id = (size_t)row * S + iz;
  c[id].x *= s;
  c[id].y *= s;
}

// out = tab[q] x (+ add): the metric's level term f^2 X plus its transformed cross terms
template <typename T>
__global__ void k_mul_table_add(typename V2m<T>::type *out, const typename V2m<T>::type *x, int n, const T *tab,
                                const typename V2m<T>::type *add) {
  const int H = n / 2, S = H + 1;
  unsigned row;
  int iz;
  if (!hs_cell(n, row, iz)) return;
  int ix = (int)(row / (unsigned)n), iy = (int)(row % (unsigned)n);
  long long kx = ix > H ? ix - n : ix, ky = iy > H ? iy - n : iy;
  T s = (T)tab[kx * kx + ky * ky + (long long)iz * iz];
  size_t id = (size_t)row * S + iz;
  typename V2m<T>::type v = x[id];
  v.x *= s;
  v.y *= s;
  if (add) {
    v.x += add[id].x;
    v.y += add[id].y;
  }
  out[id] = v;
}

// a += sum_k c[k] b[k] over n values (up to 8 sources in one pass)
constexpr int kMaxAxpy = 8;
template <typename T>
struct AxpySources {
  const T *b[kMaxAxpy];
  T c[kMaxAxpy];  // rounded to the field precision on the host (a per-element double->float
                  // conversion would occupy the FP64 pipe)
  int nb;
  const T *cdev;  // or, when set, the coefficients in device memory (already rounded)
};
template <typename T>
__global__ void k_axpy_multi(T *a, AxpySources<T> src, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T v = a[i];
  for (int k = 0; k < src.nb; ++k) v += (src.cdev ? src.cdev[k] : src.c[k]) * src.b[k][i];
  a[i] = v;
}
// the same with NB sources known at compile time and 16-byte vectors (4 floats or 2
// doubles per thread): every source's load is in flight before the sums, which run in
// the order above
template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int W = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int W = 2; };
template <typename T, int NB>
__global__ void k_axpy_multi_vec(T *a, AxpySources<T> src, size_t nvec) {
  using V = typename Vec16<T>::type;
  constexpr int W = Vec16<T>::W;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvec) return;
  V v = reinterpret_cast<V *>(a)[i];
  V b[NB];
#pragma unroll
  for (int k = 0; k < NB; ++k) b[k] = reinterpret_cast<const V *>(src.b[k])[i];
  T *pv = reinterpret_cast<T *>(&v);
#pragma unroll
  for (int k = 0; k < NB; ++k) {
    const T *pb = reinterpret_cast<const T *>(&b[k]);
    const T ck = src.cdev ? src.cdev[k] : src.c[k];
#pragma unroll
    for (int w = 0; w < W; ++w) pv[w] += ck * pb[w];
  }
  reinterpret_cast<V *>(a)[i] = v;
}

// Gram-Schmidt of n covectors through their Gram matrix, in the order of
// modificationmanager.hpp:288-312, and the correction's coefficients on the covectors
// converted to vectors (applyLinearModif, :199-217), as the host form in apply_mods:
// one thread, so that a realisation needs no host round trip (a batch captures it in a
// CUDA graph).  M: n x (n + 1) doubles, M[i][0] = <a_i|W>, M[i][1 + j] = <a_i|C a_j>.
constexpr int kDevGramMax = 16;
struct GramTargets {
  int n;
  double t[kDevGramMax];
};
template <typename T>
__global__ void k_gram_coefficients(const double *M, GramTargets tg, T *coef) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int n = tg.n;
  double L[kDevGramMax * kDevGramMax], t[kDevGramMax], c[kDevGramMax];
  auto G = [&](int i, int j) { return M[(size_t)i * (n + 1) + 1 + j]; };
  auto ip = [&](const double *x, const double *y) {
    double s = 0;
    for (int k = 0; k < n; ++k)
      for (int m = 0; m < n; ++m) s += x[k] * y[m] * G(k, m);
    return s;
  };
  for (int i = 0; i < n; ++i) {
    t[i] = tg.t[i];
    c[i] = 0;
    for (int k = 0; k < n; ++k) L[i * kDevGramMax + k] = 0;
  }
  for (int i = 0; i < n; ++i) {
    double *li = &L[i * kDevGramMax];
    li[i] = 1.0;
    for (int j = 0; j < i; ++j) {
      const double *lj = &L[j * kDevGramMax];
      const double r = ip(li, lj);
      for (int k = 0; k < n; ++k) li[k] -= r * lj[k];
      t[i] -= r * t[j];
    }
    const double nrm = sqrt(ip(li, li));
    for (int k = 0; k < n; ++k) li[k] /= nrm;
    t[i] /= nrm;
  }
  for (int i = 0; i < n; ++i) {
    double existing = 0;
    for (int k = 0; k < n; ++k) existing += L[i * kDevGramMax + k] * M[(size_t)k * (n + 1)];
    const double d = t[i] - existing;
    for (int k = 0; k < n; ++k) c[k] += d * L[i * kDevGramMax + k];
  }
  for (int k = 0; k < n; ++k) coef[k] = (T)c[k];
}

// all products <a_i|b_j> (i < na <= 4, j < nb <= 5) of half spectra in one pass over the
// fields, Hermitian-weighted; the partial sum of each block for product
// g = (ia0 + i) nb_total + jb0 + j goes to partial[g * pstride + block]
constexpr int kBlockA = 4, kBlockB = 5;
template <typename T>
struct BlockFields {
  const T *a[kBlockA];
  const T *b[kBlockB];
  int na, nb;
};
// Sums of one row's products in the field's precision, then rows accumulated in a
// compensated float pair (float fields) or a double: float fields carry 6e-8
// relative rounding already, and a row holds at most N/2 + 1 products.
template <typename T>
struct RowAcc;
template <>
struct RowAcc<float> {
  float s, e;
  __device__ __forceinline__ void zero() { s = e = 0.f; }
  __device__ __forceinline__ void add(float x) {
    const float t = s + x, bb = t - s;
    e += (s - (t - bb)) + (x - bb);
    s = t;
  }
  __device__ __forceinline__ double get() const { return (double)s + (double)e; }
};
template <>
struct RowAcc<double> {
  double s;
  __device__ __forceinline__ void zero() { s = 0; }
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double get() const { return s; }
};

template <typename T>
__global__ void __launch_bounds__(256, 3) k_inner_block(BlockFields<T> f, int n, double *partial, int ia0, int jb0,
                                                     int nb_total, size_t pstride) {
  __shared__ double red[256];
  // the row accumulators live in shared memory (one column per thread, touched once
  // per row), which keeps the registers for the loads in flight
  __shared__ RowAcc<T> acc[kBlockA * kBlockB][kKzChunk * kRowsPerBlock];
  const int H = n / 2, S = H + 1;
  const unsigned rows = (unsigned)n * (unsigned)n;
  const int tid = threadIdx.y * kKzChunk + threadIdx.x;
#pragma unroll
  for (int p = 0; p < kBlockA * kBlockB; ++p) acc[p][tid].zero();
  // a warp walks whole rows (one contiguous span of S coefficients per field), rows
  // strided over the grid
  for (unsigned r = blockIdx.x * kRowsPerBlock + threadIdx.y; r < rows; r += gridDim.x * kRowsPerBlock) {
    T row[kBlockA * kBlockB];
#pragma unroll
    for (int p = 0; p < kBlockA * kBlockB; ++p) row[p] = 0;
    for (int iz = threadIdx.x; iz < S; iz += kKzChunk) {
      const T w = (iz == 0 || iz == H) ? (T)1 : (T)2;
      const size_t id = 2 * ((size_t)r * S + iz);
      T br[kBlockB], bi[kBlockB];
#pragma unroll
      for (int j = 0; j < kBlockB; ++j)
        if (j < f.nb) {
          br[j] = f.b[j][id];
          bi[j] = f.b[j][id + 1];
        }
#pragma unroll
      for (int i = 0; i < kBlockA; ++i)
        if (i < f.na) {
          const T ar = f.a[i][id], ai = f.a[i][id + 1];
#pragma unroll
          for (int j = 0; j < kBlockB; ++j)
            if (j < f.nb) row[i * kBlockB + j] += w * (ar * br[j] + ai * bi[j]);
        }
    }
#pragma unroll
    for (int p = 0; p < kBlockA * kBlockB; ++p) acc[p][tid].add(row[p]);
  }
  for (int i = 0; i < f.na; ++i)
    for (int j = 0; j < f.nb; ++j) {
      red[tid] = acc[i * kBlockB + j][tid].get();
      __syncthreads();
      for (int s2 = 128; s2 > 0; s2 >>= 1) {
        if (tid < s2) red[tid] += red[tid + s2];
        __syncthreads();
      }
      if (tid == 0) partial[(size_t)((ia0 + i) * nb_total + jb0 + j) * pstride + blockIdx.x] = red[0];
      __syncthreads();
    }
}

// The same products for a full NA x NB block, walking the half spectra as one flat
// array of 16-byte vectors (two float or one double coefficient): every coefficient
// summed with weight 1, and the kz = 0 and kz = N/2 planes (weight 1 in the Hermitian
// sum, 2 elsewhere) counted again with weight -1/2, so twice the sum is the weighted one.
// Each thread sums four vectors in the field's precision, then into its compensated
// shared-memory accumulators.
__device__ __forceinline__ float vdot(const float4 &a, const float4 &b) {
  return fmaf(a.x, b.x, fmaf(a.y, b.y, fmaf(a.z, b.z, a.w * b.w)));
}
__device__ __forceinline__ double vdot(const double2 &a, const double2 &b) { return a.x * b.x + a.y * b.y; }

template <typename T, int NA, int NB>
__global__ void __launch_bounds__(256, 2) k_inner_block_flat(BlockFields<T> f, int n, double *partial, int ia0,
                                                          int jb0, int nb_total, size_t pstride) {
  using V = typename Vec16<T>::type;
  __shared__ double red[256];
  __shared__ RowAcc<T> acc[NA * NB][256];
  const int tid = threadIdx.x;
#pragma unroll
  for (int p = 0; p < NA * NB; ++p) acc[p][tid].zero();
  const int H = n / 2, S = H + 1;
  // n is even, so n^2 (n/2 + 1) coefficients fill whole vectors
  const size_t nv = (size_t)n * n * S * 2 / Vec16<T>::W;
  const size_t step = (size_t)gridDim.x * blockDim.x;
  size_t q = (size_t)blockIdx.x * blockDim.x + tid;
  while (q < nv) {
    T part[NA * NB];
#pragma unroll
    for (int p = 0; p < NA * NB; ++p) part[p] = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (q < nv) {
        V b[NB];
#pragma unroll
        for (int j = 0; j < NB; ++j) b[j] = __ldg(reinterpret_cast<const V *>(f.b[j]) + q);
#pragma unroll
        for (int i = 0; i < NA; ++i) {
          const V a = __ldg(reinterpret_cast<const V *>(f.a[i]) + q);
#pragma unroll
          for (int j = 0; j < NB; ++j) part[i * NB + j] += vdot(a, b[j]);
        }
      }
      q += step;
    }
#pragma unroll
    for (int p = 0; p < NA * NB; ++p) acc[p][tid].add(part[p]);
  }
  // the kz = 0 and kz = N/2 planes once more, weight -1/2
  const unsigned rows = (unsigned)n * (unsigned)n;
  for (unsigned r = blockIdx.x * blockDim.x + tid; r < rows; r += (unsigned)step) {
    T part[NA * NB];
#pragma unroll
    for (int p = 0; p < NA * NB; ++p) part[p] = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const size_t id = 2 * ((size_t)r * S + (h ? H : 0));
      T br[NB], bi[NB];
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        br[j] = f.b[j][id];
        bi[j] = f.b[j][id + 1];
      }
#pragma unroll
      for (int i = 0; i < NA; ++i) {
        const T ar = f.a[i][id], ai = f.a[i][id + 1];
#pragma unroll
        for (int j = 0; j < NB; ++j) part[i * NB + j] += ar * br[j] + ai * bi[j];
      }
    }
#pragma unroll
    for (int p = 0; p < NA * NB; ++p) acc[p][tid].add((T)-0.5 * part[p]);
  }
  for (int p = 0; p < NA * NB; ++p) {
    red[tid] = 2.0 * acc[p][tid].get();
    __syncthreads();
    for (int s2 = 128; s2 > 0; s2 >>= 1) {
      if (tid < s2) red[tid] += red[tid + s2];
      __syncthreads();
    }
    if (tid == 0) partial[(size_t)((ia0 + p / NB) * nb_total + jb0 + p % NB) * pstride + blockIdx.x] = red[0];
    __syncthreads();
  }
}

// --- elementwise ----------------------------------------------------------------

template <typename T>
__global__ void k_axpy(T *a, const T *b, T c, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] += c * b[i];
}

template <typename T>
__global__ void k_scale(T *a, T c, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] *= c;
}

// Window combinations on padded real fields (in = cell inside the window):
//   op 0: r = (in ? 0 : r) + s      op 1: r = in ? s : r      op 2: r = in ? s : 0
template <typename T>
__global__ void k_window_op(T *r, const T *s, int n, const unsigned char *mx, const unsigned char *my,
                            const unsigned char *mz, int op, int x0, int y0, int ny) {
  // a CTA per row of n cells of the rows x0 + i, y0 + j (cyclic; blockIdx.x = i ny + j):
  // the row's x and y window tests once, then its cells
  const int x = (x0 + (int)(blockIdx.x / (unsigned)ny)) % n, y = (y0 + (int)(blockIdx.x % (unsigned)ny)) % n;
  const unsigned row = (unsigned)x * (unsigned)n + (unsigned)y;
  const bool row_in = mx[x] && my[y];
  const size_t base = (size_t)row * (size_t)(2 * (n / 2 + 1));
  for (int z = threadIdx.x; z < n; z += blockDim.x) {
    const bool in = row_in && mz[z];
    const size_t id = base + z;
    if (op == 0) r[id] = (in ? (T)0 : r[id]) + s[id];
    else if (op == 1) { if (in) r[id] = s[id]; }
    else r[id] = in ? s[id] : (T)0;
  }
}
inline dim3 real_block(int n) { return dim3((unsigned)std::min(256, (n + 31) / 32 * 32)); }

// Hermitian-weighted Re(conj(a) b) over a half spectrum, partial sums per block.
// Float fields: every product is split exactly (fma) and accumulated in a
// compensated float pair per thread, converted to double once -- a double-grade
// sum without double arithmetic per element.  Double fields: plain doubles.
__device__ __forceinline__ void acc2(float &s, float &e, float x) {
  float t = s + x;
  float bb = t - s;
  e += (s - (t - bb)) + (x - bb);
  s = t;
}
__device__ __forceinline__ double thread_inner_col(const float *a, const float *b, unsigned rows, int S, int iz,
                                                   float w, unsigned r0, unsigned rstep) {
  float s = 0.f, e = 0.f;
  for (unsigned r = r0; r < rows; r += rstep) {
    size_t id = (size_t)r * S + iz;
    float ar = a[2 * id], ai = a[2 * id + 1], br = b[2 * id], bi = b[2 * id + 1];
    float p1 = ar * br, p2 = ai * bi;
    float e1 = fmaf(ar, br, -p1), e2 = fmaf(ai, bi, -p2);
    acc2(s, e, w * p1);
    acc2(s, e, w * p2);
    e += w * (e1 + e2);
  }
  return (double)s + (double)e;
}
__device__ __forceinline__ double thread_inner_col(const double *a, const double *b, unsigned rows, int S, int iz,
                                                   float w, unsigned r0, unsigned rstep) {
  double acc = 0;
  for (unsigned r = r0; r < rows; r += rstep) {
    size_t id = (size_t)r * S + iz;
    acc += (double)w * (a[2 * id] * b[2 * id] + a[2 * id + 1] * b[2 * id + 1]);
  }
  return acc;
}

// sum over the n^3 cells of two padded real fields (Parseval: equals the
// Hermitian-weighted spectral sum of their unitary transforms)
__device__ __forceinline__ double thread_dot_col(const float *a, const float *b, unsigned rows, size_t rs, int z,
                                                 unsigned r0, unsigned rstep) {
  float s = 0.f, e = 0.f;
  for (unsigned r = r0; r < rows; r += rstep) {
    size_t id = (size_t)r * rs + z;
    float p = a[id] * b[id];
    e += fmaf(a[id], b[id], -p);
    acc2(s, e, p);
  }
  return (double)s + (double)e;
}
__device__ __forceinline__ double thread_dot_col(const double *a, const double *b, unsigned rows, size_t rs, int z,
                                                 unsigned r0, unsigned rstep) {
  double acc = 0;
  for (unsigned r = r0; r < rows; r += rstep) acc += a[(size_t)r * rs + z] * b[(size_t)r * rs + z];
  return acc;
}

template <typename T>
__global__ void k_inner_real(const T *a, const T *b, int n, double *partial) {
  __shared__ double red[256];
  const unsigned rows = (unsigned)n * (unsigned)n;
  const size_t rs = (size_t)(2 * (n / 2 + 1));
  const int tid = threadIdx.y * kKzChunk + threadIdx.x;
  double acc = 0;
  for (int z = threadIdx.x; z < n; z += kKzChunk)
    acc += thread_dot_col(a, b, rows, rs, z, blockIdx.x * kRowsPerBlock + threadIdx.y, gridDim.x * kRowsPerBlock);
  red[tid] = acc;
  __syncthreads();
  for (int s2 = 128; s2 > 0; s2 >>= 1) {
    if (tid < s2) red[tid] += red[tid + s2];
    __syncthreads();
  }
  if (tid == 0) partial[blockIdx.x] = red[0];
}

// sum over the cells of a box (cyclic ranges per axis) of two padded real fields
template <typename T>
__global__ void k_inner_real_box(const T *a, const T *b, int n, CellBox box, double *partial) {
  __shared__ double red[256];
  const size_t rs = (size_t)(2 * (n / 2 + 1));
  const int tid = threadIdx.y * kKzChunk + threadIdx.x;
  const unsigned ny = (unsigned)box.len[1], rows = (unsigned)box.len[0] * ny;
  double acc = 0;
  for (unsigned r = blockIdx.x * kRowsPerBlock + threadIdx.y; r < rows; r += gridDim.x * kRowsPerBlock) {
    const int x = (box.start[0] + (int)(r / ny)) % n, y = (box.start[1] + (int)(r % ny)) % n;
    const size_t base = ((size_t)x * (size_t)n + (size_t)y) * rs;
    for (int j = threadIdx.x; j < box.len[2]; j += kKzChunk) {
      const size_t id = base + (size_t)((box.start[2] + j) % n);
      acc += (double)a[id] * (double)b[id];
    }
  }
  red[tid] = acc;
  __syncthreads();
  for (int s2 = 128; s2 > 0; s2 >>= 1) {
    if (tid < s2) red[tid] += red[tid + s2];
    __syncthreads();
  }
  if (tid == 0) partial[blockIdx.x] = red[0];
}

template <typename T>
__global__ void k_inner(const T *a, const T *b, int n, double *partial) {
  __shared__ double red[256];
  const int H = n / 2, S = H + 1;
  const unsigned rows = (unsigned)n * (unsigned)n;
  const int tid = threadIdx.y * kKzChunk + threadIdx.x;
  double acc = 0;
  // grid-stride over rows; each thread owns a kz column chunk of its rows
  for (int iz = threadIdx.x; iz < S; iz += kKzChunk) {
    float wf = (iz == 0 || iz == H) ? 1.f : 2.f;
    acc += thread_inner_col(a, b, rows, S, iz, wf, blockIdx.x * kRowsPerBlock + threadIdx.y,
                            gridDim.x * kRowsPerBlock);
  }
  red[tid] = acc;
  __syncthreads();
  for (int s2 = 128; s2 > 0; s2 >>= 1) {
    if (tid < s2) red[tid] += red[tid + s2];
    __syncthreads();
  }
  if (tid == 0) partial[blockIdx.x] = red[0];
}

// partial dot products of two flat arrays (grid-stride, one value per block)
template <typename T>
__global__ void k_dot_flat(const T *a, const T *b, size_t n, double *partial) {
  __shared__ double red[256];
  double acc = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    acc += (double)a[i] * (double)b[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// the tail of genetIC's real-space buffer after an inverse transform: padded positions
// [n^3, n^2 (n + 2)) of the c2r output -- the last rows' values, and their padding
// slots (the kz = n/2 coefficient after the x and y passes, which this library's c2r
// leaves unscaled) -- divided by n^1.5 (fourier.hpp:388-404, 479-518)
template <typename T>
__global__ void k_extract_tail(const T *padded, T *tail, int n, T scale) {
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t n3 = (size_t)n * n * n, len = (size_t)n * n * (n + 2) - n3;
  if (t >= len) return;
  size_t p = n3 + t;
  T v = padded[p];
  if ((int)(p % (size_t)(n + 2)) >= n) v *= scale;
  tail[t] = v;
}

// sums of consecutive runs of n doubles in a fixed order, one block per run
__global__ void k_sum(const double *in, int n, double *out) {
  __shared__ double red[256];
  in += (size_t)blockIdx.x * n;
  out += blockIdx.x;
  double acc = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += in[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// flagged cells (compact linear indices (x n + y) n + z) of a padded real field
__device__ __forceinline__ size_t padded_index(unsigned long long c, int n) {
  unsigned long long row = c / (unsigned)n;
  return (size_t)row * (size_t)(2 * (n / 2 + 1)) + (size_t)(c - row * (unsigned)n);
}
template <typename T>
__global__ void k_gather_cells(const T *real, int n, const unsigned long long *cells, size_t count, T *out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) out[i] = real[padded_index(cells[i], n)];
}
template <typename T>
__global__ void k_scatter_cells(const T *in, int n, const unsigned long long *cells, size_t count, T *real) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) real[padded_index(cells[i], n)] = in[i];
}
// zero the flagged cells of a padded real field
template <typename T>
__global__ void k_zero_cells(T *real, int n, const unsigned long long *cells, size_t count) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) real[padded_index(cells[i], n)] = (T)0;
}

// the variance operator on the flagged values: v = (v - mean) / count, the mean
// summed in double in one block (quadraticmodification.hpp:199-218)
template <typename T>
__global__ void k_center_cells(T *v, size_t count) {
  __shared__ double red[1024];
  __shared__ double mean;
  double acc = 0;
  for (size_t i = threadIdx.x; i < count; i += blockDim.x) acc += (double)v[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) mean = red[0] / (double)count;
  __syncthreads();
  const T m = (T)mean, c = (T)(double)count;
  for (size_t i = threadIdx.x; i < count; i += blockDim.x) v[i] = (v[i] - m) / c;
}

// Localisation covectors on the finest grid (padded real layout).  genetIC builds them
// cell by cell in the order of its sorted flagged-cell list, adding the stencil values
// into the output (linearmodification.hpp:223-233, 344-374); where stencils overlap, a
// cell's value is a sum whose rounding depends on that order.  Each kernel here writes
// every reached cell once, from the thread of the contribution that comes first, as the
// double sum of all its contributions in the reference's order, so the FP64 covector has
// the reference's bits (the mixed form rounds that sum once) and nothing depends on
// thread scheduling.  cells: sorted, unique.

// The list position of a cell: from a dense map of the flagged cells' box (start, len per
// axis, cyclic on n cells; -1 = not flagged, and every cell outside the box is unflagged),
// or, without a map, by binary search of the sorted list.
struct FlagLookup {
  const int *map;
  int n, start[3], len[3];
};
__device__ __forceinline__ long long find_flagged(const unsigned long long *cells, size_t count,
                                                  unsigned long long id);
__device__ __forceinline__ long long find_flagged(const FlagLookup &fl, const unsigned long long *cells, size_t count,
                                                  unsigned long long id) {
  if (!fl.map) return find_flagged(cells, count, id);
  const int n = fl.n;
  const int p[3] = {(int)(id / ((unsigned long long)n * n)), (int)((id / n) % n), (int)(id % n)};
  int o[3];
  for (int a = 0; a < 3; ++a) {
    o[a] = ((p[a] - fl.start[a]) % n + n) % n;
    if (o[a] >= fl.len[a]) return -1;
  }
  return fl.map[((size_t)o[0] * fl.len[1] + o[1]) * fl.len[2] + o[2]];
}
__global__ void k_flag_map(const unsigned long long *cells, size_t count, FlagLookup fl, int *map) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const unsigned long long id = cells[i];
  const int n = fl.n;
  const int p[3] = {(int)(id / ((unsigned long long)n * n)), (int)((id / n) % n), (int)(id % n)};
  int o[3];
  for (int a = 0; a < 3; ++a) o[a] = ((p[a] - fl.start[a]) % n + n) % n;
  map[((size_t)o[0] * fl.len[1] + o[1]) * fl.len[2] + o[2]] = (int)i;
}

// the list position of cell id, or -1
__device__ __forceinline__ long long find_flagged(const unsigned long long *cells, size_t count,
                                                  unsigned long long id) {
  size_t lo = 0, hi = count;
  while (lo < hi) {
    const size_t mid = (lo + hi) / 2;
    if (cells[mid] < id) lo = mid + 1;
    else hi = mid;
  }
  return lo < count && cells[lo] == id ? (long long)lo : -1;
}
// the cell `step` cells from id along axis ax, periodically
__device__ __forceinline__ unsigned long long step_cell(unsigned long long id, int n, int ax, int step) {
  int p[3] = {(int)(id / ((unsigned long long)n * n)), (int)((id / n) % n), (int)(id % n)};
  p[ax] = ((p[ax] + step) % n + n) % n;
  return ((unsigned long long)p[0] * n + p[1]) * n + p[2];
}
__device__ __forceinline__ size_t padded_at(unsigned long long id, int n) {
  const unsigned long long z = id % n, r = id / n;
  return (size_t)r * (size_t)(2 * (n / 2 + 1)) + (size_t)z;
}

// kind 0: w on every flagged cell (OverdensityModification); kind 1: the 4th-order
// gradient stencil along dir with values a, b, -b, -a at -2, -1, +1, +2 (VelocityModification)
template <typename T>
__global__ void k_localise(T *real, int n, const unsigned long long *cells, size_t count, int kind, int dir,
                           double w, double a, double b, FlagLookup fl) {
  // kind 0: a thread per flagged cell; kind 1: a thread per (flagged cell, stencil position)
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (kind == 0) {
    if (tid < count) real[padded_at(cells[tid], n)] = (T)w;
    return;
  }
  const size_t i = tid >> 2;
  const int k = (int)(tid & 3);
  if (i >= count) return;
  const unsigned long long q = cells[i];
  const int off[4] = {-2, -1, 1, 2};
  const double val[4] = {a, b, -b, -a};
  const unsigned long long t = step_cell(q, n, dir, off[k]);
  // every contribution to t: the flagged cell -off[k2] away, its stencil value k2
  long long ci[4];
  int ck[4], nc = 0;
  for (int k2 = 0; k2 < 4; ++k2) {
    const long long i2 = find_flagged(fl, cells, count, step_cell(t, n, dir, -off[k2]));
    if (i2 < 0) continue;
    if (i2 < (long long)i || (i2 == (long long)i && k2 < k)) return;  // an earlier contribution writes t
    ci[nc] = i2;
    ck[nc++] = k2;
  }
  for (int u = 1; u < nc; ++u)  // by (list position, stencil position)
    for (int v = u; v > 0 && (ci[v] < ci[v - 1] || (ci[v] == ci[v - 1] && ck[v] < ck[v - 1])); --v) {
      const long long ti = ci[v]; ci[v] = ci[v - 1]; ci[v - 1] = ti;
      const int tk = ck[v]; ck[v] = ck[v - 1]; ck[v - 1] = tk;
    }
  double acc = 0;  // the reference's double sum; rounded once in the mixed form
  for (int u = 0; u < nc; ++u) acc += val[ck[u]];
  real[padded_at(t, n)] = (T)acc;
}

// angular-momentum localisation covector (AngMomentumModification::calculateLocalisationCovector,
// linearmodification.hpp:333-383): per flagged cell at centroid q, with dq = centre - q
// (wrapped), coefficients c[dir+2] = dq[dir+1], c[dir+1] = -dq[dir+2], and along each
// other axis (ascending) the 4th-order gradient stencil a, b, -b, -a scaled by that
// coefficient, summed in the reference's order (cell, axis, stencil position)
template <typename T>
__global__ void k_localise_am(T *real, int n, const unsigned long long *cells, size_t count, int dir, double dx,
                              double x0, double y0, double z0, double cx, double cy, double cz, double period,
                              double a, double b, FlagLookup fl) {
  // a thread per (flagged cell, axis, stencil position)
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t i = tid >> 3;
  if (i >= count) return;
  const int d1 = (dir + 1) % 3, d2 = (dir + 2) % 3;
  const int axes[2] = {d1 < d2 ? d1 : d2, d1 < d2 ? d2 : d1};
  const double org[3] = {x0, y0, z0}, cen[3] = {cx, cy, cz};
  // the stencil coefficient of a flagged cell along axis ax
  auto coeff = [&](unsigned long long id, int ax) {
    const int p[3] = {(int)(id / ((unsigned long long)n * n)), (int)((id / n) % n), (int)(id % n)};
    double dq[3];
    for (int k = 0; k < 3; ++k) {
      double v = cen[k] - (p[k] * dx + org[k] + dx / 2);
      if (v > period / 2) v -= period;
      if (v < -period / 2) v += period;
      dq[k] = v;
    }
    return ax == d2 ? dq[d1] : (ax == d1 ? -dq[d2] : 0.0);
  };
  const int off[4] = {-2, -1, 1, 2};
  const unsigned long long q = cells[i];
  const int xa = (int)((tid >> 2) & 1), k = (int)(tid & 3);
  const unsigned long long t = step_cell(q, n, axes[xa], off[k]);
  // every contribution to t, unless an earlier one (in the reference's order) writes it
  long long ci[8];
  int cx2[8], ck[8], nc = 0;
  for (int xb = 0; xb < 2; ++xb)
    for (int k2 = 0; k2 < 4; ++k2) {
      const long long i2 = find_flagged(fl, cells, count, step_cell(t, n, axes[xb], -off[k2]));
      if (i2 < 0) continue;
      if (i2 < (long long)i || (i2 == (long long)i && (xb < xa || (xb == xa && k2 < k)))) return;
      ci[nc] = i2;
      cx2[nc] = xb;
      ck[nc++] = k2;
    }
  for (int u = 1; u < nc; ++u)  // by (list position, axis, stencil position)
    for (int v = u; v > 0; --v) {
      const bool before = ci[v] < ci[v - 1] ||
                          (ci[v] == ci[v - 1] && (cx2[v] < cx2[v - 1] || (cx2[v] == cx2[v - 1] && ck[v] < ck[v - 1])));
      if (!before) break;
      const long long ti = ci[v]; ci[v] = ci[v - 1]; ci[v - 1] = ti;
      const int tx = cx2[v]; cx2[v] = cx2[v - 1]; cx2[v - 1] = tx;
      const int tk = ck[v]; ck[v] = ck[v - 1]; ck[v - 1] = tk;
    }
  double acc = 0;  // the reference's double sum; rounded once in the mixed form
  for (int u = 0; u < nc; ++u) {
    const double c = coeff(cells[ci[u]], axes[cx2[u]]);
    acc += ck[u] == 0 ? c * a : ck[u] == 1 ? c * b : ck[u] == 2 ? -(c * b) : -(c * a);
  }
  real[padded_at(t, n)] = (T)acc;
}

// cosmology::densityToPotential (cosmology/parameters.hpp:209-225): times -prefac / k^2.
// The reference's guard against k = 0 tests the y component of k, so every mode with
// ky = 0 is set to zero; that behaviour is kept.
template <typename T>
__global__ void k_density_to_potential(typename V2m<T>::type *c, int n, double kmin, double prefac) {
  const int H = n / 2, S = H + 1;
  unsigned row;
  int iz;
  if (!hs_cell(n, row, iz)) return;
  int ix = (int)(row / (unsigned)n), iy = (int)(row % (unsigned)n);
  double kx = (double)(ix > H ? ix - n : ix) * kmin, ky = (double)(iy > H ? iy - n : iy) * kmin,
         kz = (double)iz * kmin;
  double ksq = kx * kx + ky * ky + kz * kz;
  double inv = ky == 0.0 ? 0.0 : 1.0 / ksq;
  size_t id = (size_t)row * S + iz;
  typename V2m<T>::type v = c[id];
  v.x = (T)(-prefac * (double)v.x * inv);
  v.y = (T)(-prefac * (double)v.y * inv);
  c[id] = v;
}

template <typename T>
__device__ __forceinline__ void cr_weights(T t, T (&w)[4]) {
  T t2 = t * t, t3 = t2 * t;
  w[0] = -(t - 1) * (t - 1) * t / 2;
  w[1] = (2 - 5 * t2 + 3 * t3) / 2;
  w[2] = t * (1 + 4 * t - 3 * t2) / 2;
  w[3] = (t - 1) * t2 / 2;
}

// Transpose interpolation, one axis at a time.  `in` has dims (A0, A1, A2) with
// strides (s0, s1, 1); the pass contracts axis `ax` of nf fine cells into nout coarse
// cells starting at unwrapped coarse index c0: out[..c..] = sum over x of
// w_a(t_x) in[..x..] for c = ubase[x] - 1 + a, taken in increasing x, a thread per
// output element.  range[u - umin] = the first and last fine cell (whole
// axis) reaching unwrapped coarse index u; ubase and frac start at the line's first
// fine cell x0 (whole-axis index), nf cells.  Every output element is written.
template <typename T>
__global__ void k_deinterp_gather(const T *in, long long in_s0, long long in_s1, T *out, long long out_s0,
                                  long long out_s1, int ax, int n0, int n1, int n2, int nf, const int *ubase,
                                  const T *frac, const int2 *range, int umin, int ncu, int x0, int c0, int nout,
                                  T scale) {
  int d[3] = {n0, n1, n2};
  const int oa = ax == 0 ? 1 : 0, ob = ax == 2 ? 1 : 2;
  const long long lines = (long long)d[oa] * d[ob];
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= lines * nout) return;
  const long long line = tid % lines;
  const int cc = (int)(tid / lines);
  const int ib = (int)(line % d[ob]), ia = (int)(line / d[ob]);
  long long is[3] = {in_s0, in_s1, 1}, os[3] = {out_s0, out_s1, 1};
  const long long ibase = (long long)ia * is[oa] + (long long)ib * is[ob];
  const long long obase = (long long)ia * os[oa] + (long long)ib * os[ob];
  const int u = c0 + cc, ui = u - umin;
  T acc = 0;
  if (ui >= 0 && ui < ncu) {
    const int2 rg = range[ui];
    const int lo = max(rg.x - x0, 0), hi = min(rg.y - x0, nf - 1);
    for (int x = lo; x <= hi; ++x) {
      const int a = u - (ubase[x] - 1);
      if (a < 0 || a > 3) continue;
      const T v = in[ibase + (long long)x * is[ax]] * scale;
      T w[4];
      cr_weights<T>(frac[x], w);
      acc += w[a] * v;
    }
  }
  out[obase + (long long)cc * os[ax]] = acc;
}

// add a compact block (bx, by, bz) starting at unwrapped coarse (c0x, c0y, c0z) into a padded real coarse field
template <typename T>
__global__ void k_add_block(const T *blk, int bx, int by, int bz, int c0x, int c0y, int c0z, T *real, int n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t m = (size_t)bx * by * bz;
  if (i >= m) return;
  int z = (int)(i % bz);
  size_t r = i / bz;
  int y = (int)(r % by), x = (int)(r / by);
  int X = ((c0x + x) % n + n) % n, Y = ((c0y + y) % n + n) % n, Z = ((c0z + z) % n + n) % n;
  atomicAdd(real + ((size_t)X * n + Y) * (size_t)(2 * (n / 2 + 1)) + Z, blk[i]);
}

// coarse cells covered by the fine grid receive the mean of their r^3 fine cells
template <typename T>
__global__ void k_subsample_add(const T *fine, int nf, int r, int sx, int sy, int sz, T *coarse, int nc) {
  int m = nf / r;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)m * m * m) return;
  int k = (int)(i % m);
  size_t rr = i / m;
  int j = (int)(rr % m), ii = (int)(rr / m);
  const size_t frs = (size_t)(2 * (nf / 2 + 1));
  T s = 0;
  for (int a = 0; a < r; ++a)
    for (int b = 0; b < r; ++b)
      for (int c = 0; c < r; ++c)
        s += fine[((size_t)(ii * r + a) * nf + (j * r + b)) * frs + (k * r + c)];
  s /= (T)((double)r * r * r);
  int X = ((sx + ii) % nc + nc) % nc, Y = ((sy + j) % nc + nc) % nc, Z = ((sz + k) % nc + nc) % nc;
  coarse[((size_t)X * nc + Y) * (size_t)(2 * (nc / 2 + 1)) + Z] += s;
}

// Block means of an inverse transform, formed in Fourier space.  With unitary transforms,
// the mean over the r^3 fine cells of block X of f = IFFT_N(F) is IFFT_{N/r}(G)(X) with
//   G(K) = r^-1.5 sum_{m in [0,r)^3} F(K + m N/r) b(K_x + m_x N/r) b(..y) b(..z),
//   b(k) = (1/r) sum_{j<r} exp(+2 pi i k j / N)
// (a box filter, then decimation: the r^3 aliases of K fold onto it).  F = in * tab[q] on
// the fine half spectrum, completed by Hermitian symmetry; on the kz = 0 and N/2 planes
// the conjugate halves are taken from their partners, as the inverse transform's mirror
// does.  out: the (N/r)^3 half spectrum G.  btab: b(k), k < N.
// The r^2 (m_x, m_y) alias pairs of an output coefficient are spread over the warps of
// a CTA: a CTA owns 32 consecutive output coefficients (one per lane),
// warp w sums the pairs w, w + NW, ... over m_z, and the NW partial sums are added in
// shared memory: r^2 times the loads in flight of one thread per output coefficient, for
// a pass bound by its loads' latency.  R > 0: r known at compile time.
template <typename T, int R, int NW>
__global__ void __launch_bounds__(32 * NW) k_fold_block_means(typename V2m<T>::type *out,
                                                                    const typename V2m<T>::type *in, int N,
                                                                    int r_rt, const T *tab,
                                                                    const typename V2m<T>::type *btab, T fac,
                                                                    const T *tcol) {
  using C = typename V2m<T>::type;
  __shared__ C part[NW][32];
  const int r = R > 0 ? R : r_rt;
  const int nc = N / r, Sc = nc / 2 + 1, H = N / 2, S = H + 1;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const size_t id = (size_t)blockIdx.x * 32 + lane;
  const bool valid = id < (size_t)nc * nc * Sc;
  T ar = 0, ai = 0;
  if (valid) {
    const int KZ = (int)(id % Sc);
    const size_t rr = id / Sc;
    const int KY = (int)(rr % nc), KX = (int)(rr / nc);
    for (int pr = w; pr < r * r; pr += NW) {
      const int mx = pr / r, my = pr - mx * r;
      const int kx = KX + mx * nc, ky = KY + my * nc;
      const C bx = btab[kx], by = btab[ky];
      const T bxy_r = bx.x * by.x - bx.y * by.y, bxy_i = bx.x * by.y + bx.y * by.x;
      const long long sxk = kx > H ? kx - N : kx, syk = ky > H ? ky - N : ky;
      const long long qxy = sxk * sxk + syk * syk;
      constexpr int RU = R > 0 ? R : 1;
#pragma unroll
      for (int mz0 = 0; mz0 < (R > 0 ? R : r); mz0 += RU) {
        C f[RU];
        T t[RU];
#pragma unroll
        for (int u = 0; u < RU; ++u) {
          const int kz = KZ + (mz0 + u) * nc;
          // the stored coefficient, or the conjugate of its Hermitian partner
          const bool mir = kz > H || ((kz == 0 || kz == H) && (kx > H || ((kx == 0 || kx == H) && ky > H)));
          const int qx = mir ? (N - kx) % N : kx, qy = mir ? (N - ky) % N : ky, qz = kz > H ? N - kz : kz;
          f[u] = in[((size_t)qx * N + qy) * S + qz];
          if (mir) f[u].y = -f[u].y;
          // the filter from its per-coefficient layout (contiguous along a warp's kz) where there is one
          t[u] = tcol ? tcol[((size_t)(qx > H ? N - qx : qx) * N + qy) * S + qz] : tab[qxy + (long long)qz * qz];
        }
#pragma unroll
        for (int u = 0; u < RU; ++u) {
          const C bz = btab[KZ + (mz0 + u) * nc];
          const T b_r = bxy_r * bz.x - bxy_i * bz.y, b_i = bxy_r * bz.y + bxy_i * bz.x;
          const T fr = f[u].x * t[u], fi = f[u].y * t[u];
          ar += fr * b_r - fi * b_i;
          ai += fr * b_i + fi * b_r;
        }
      }
    }
  }
  C v;
  v.x = ar;
  v.y = ai;
  part[w][lane] = v;
  __syncthreads();
  if (w == 0 && valid) {
    T sr = 0, si = 0;
#pragma unroll
    for (int k = 0; k < NW; ++k) {
      sr += part[k][lane].x;
      si += part[k][lane].y;
    }
    C o;
    o.x = sr * fac;
    o.y = si * fac;
    out[id] = o;
  }
}

// mbarrier and bulk-copy helpers of k_fold_rows
__device__ __forceinline__ unsigned fold_smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool fold_mbar_wait(uint64_t *b, long long cycles) {
  const long long t0 = clock64();
  for (;;) {
    unsigned done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(fold_smem_u32(b)), "r"(0u)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > cycles) return false;
  }
}
// one bulk copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) completing on bar
__device__ __forceinline__ void fold_bulk(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   fold_smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(fold_smem_u32(bar))
               : "memory");
}
template <int BYTES>
__device__ __forceinline__ void fold_cp_async(void *smem, const void *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(fold_smem_u32(smem)), "l"(gmem), "n"(BYTES));
}

// Row geometry of k_fold_rows for N: a staged row of the half spectrum (N/2 + 1 complex) or
// of the filter's per-coefficient layout (N/2 + 1 real) starts on the 16-byte boundary at or
// below the row and covers it: the shared-memory row is that many bytes, the element at
// kz is at (row start mod 16) / element size + kz.
template <typename T>
struct FoldRowGeom {
  // bytes of a copy of `bytes` starting `shift` bytes after a 16-byte boundary
  __host__ __device__ static size_t span(size_t shift, size_t bytes) { return (shift + bytes + 15) & ~(size_t)15; }
  // the largest such copy: row starts are multiples of the element size
  __host__ __device__ static size_t data_bytes(int N) {
    const size_t e = 2 * sizeof(T);
    return span(e < 16 ? 16 - e : 0, (size_t)(N / 2 + 1) * e);
  }
  __host__ __device__ static size_t tab_bytes(int N) {
    const size_t e = sizeof(T);
    return span(e < 16 ? 16 - e : 0, (size_t)(N / 2 + 1) * e);
  }
  // shared memory: an mbarrier (16 bytes), 2 r^2 data rows, 2 r^2 filter rows, b(k) for k < N,
  // and the partial sums of up to 4 groups of alias pairs for the 2 (N/r/2 + 1) outputs
  static size_t smem(int r, int N) {
    return 16 + 2 * (size_t)r * r * (data_bytes(N) + tab_bytes(N)) + (size_t)N * 2 * sizeof(T) +
           4 * 2 * (size_t)(N / r / 2 + 1) * 2 * sizeof(T);
  }
};
constexpr size_t kFoldRowsSmem = 220 * 1024;

// per alias row of k_fold_rows: the staged rows' element offsets and b(kx) b(ky)
template <typename T>
struct FoldPair {
  int own, town, mir, tmir;  // the row and its Hermitian partner row (elements of g, tv)
  int noncanon;              // (kx, ky) takes the kz = 0, N/2 coefficients from its partner
  T bxy_r, bxy_i;
};

// The same G by fine rows.  A CTA owns a pair of coarse columns {K, K'} with
// K' = (-K_x, -K_y) mod N/r (a column equal to its partner alone): the r^2 fine rows
// (K_x + m_x N/r, K_y + m_y N/r) of each, the ones whose Hermitian partners the other
// column's mirrored aliases read, are copied once into shared memory with their filter
// values and b(k), by one bulk copy (cp.async.bulk) per row, all in flight together.  Then
// each output coefficient (side, K_z) sums its r^3 aliases from there with the products of
// k_fold_block_means: the alias pairs (m_x, m_y) fall in up to 4 equal groups in order,
// a thread sums a group (each pair's m_z terms first, then the pairs in order), and the
// groups' sums are added in order.  tcol: the filter's per-coefficient layout, or nullptr
// (tab by |k|^2, a gather of 4- or 8-byte cp.async).  The CTAs cover the columns with K <= K' (ids K_x nc + K_y):
// K_x in [1, nc/2) with every K_y, then K_x = 0 and nc/2 with K_y in [0, nc/2].
// err, wait_cycles: a wait for the bulk copies that gives up sets *err = 4 and the CTA
// returns after its copies have landed (or a second wait has given up).  N % 4 == 0.
template <typename T, int R, int NT>
__global__ void __launch_bounds__(NT) k_fold_rows(typename V2m<T>::type *out, const typename V2m<T>::type *in, int N,
                                                  const T *tab, const T *tcol, const typename V2m<T>::type *btab,
                                                  T fac, int *err, long long wait_cycles) {
  using C = typename V2m<T>::type;
  using G = FoldRowGeom<T>;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ FoldPair<T> pairs[2 * R * R];
  __shared__ int s_stop;
  constexpr int R2 = R * R;
  const int nc = N / R, Sc = nc / 2 + 1, H = N / 2, S = H + 1;
  int KX, KY;
  {
    const int p = (int)blockIdx.x, head = (nc / 2 - 1) * nc;
    if (p < head) {
      KX = 1 + p / nc;
      KY = p - (KX - 1) * nc;
    } else {
      const int q = p - head;
      KX = q < nc / 2 + 1 ? 0 : nc / 2;
      KY = q % (nc / 2 + 1);
    }
  }
  const int PX = (nc - KX) % nc, PY = (nc - KY) % nc;
  const int sides = (PX == KX && PY == KY) ? 1 : 2;
  const size_t DB = G::data_bytes(N), TB = G::tab_bytes(N);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smraw);
  unsigned char *drows = smraw + 16;
  unsigned char *trows = drows + 2 * R2 * DB;
  C *bt = reinterpret_cast<C *>(trows + 2 * R2 * TB);
  const int nrow = sides * R2;
  if (threadIdx.x == 0) {
    s_stop = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fold_smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // the bulk copies, spread over the first warp's lanes: each lane announces its bytes
  // before it issues them, and lane 0 arrives after the whole warp has announced, so the
  // phase completes only when every copy has landed.  A row's copy starts on the 16-byte
  // boundary at or below the row and ends on the one at or above its end: for the array
  // of N^2 rows (N % 4 == 0) and the per-coefficient layout of a power-of-two N, the
  // bytes before and after a row belong to its neighbouring rows, inside the buffer.
  if (threadIdx.x < 32) {
    unsigned mine = 0;
    for (int row = (int)threadIdx.x; row < nrow; row += 32) {
      const int sd = row / R2, pr = row - sd * R2;
      const int kx = (sd ? PX : KX) + (pr / R) * nc, ky = (sd ? PY : KY) + (pr % R) * nc;
      const uintptr_t a = (uintptr_t)(in + ((size_t)kx * N + ky) * S);
      mine += (unsigned)G::span(a & 15, (size_t)S * sizeof(C));
      if (tcol) {
        const uintptr_t b = (uintptr_t)(tcol + ((size_t)(kx > H ? N - kx : kx) * N + ky) * S);
        mine += (unsigned)G::span(b & 15, (size_t)S * sizeof(T));
      }
    }
    if (threadIdx.x == 0) mine += (unsigned)(N * sizeof(C));
    if (mine)
      asm volatile("mbarrier.expect_tx.shared::cta.b64 [%0], %1;" ::"r"(fold_smem_u32(bar)), "r"(mine) : "memory");
    __syncwarp();
    if (threadIdx.x == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(fold_smem_u32(bar)) : "memory");
    for (int row = (int)threadIdx.x; row < nrow; row += 32) {
      const int sd = row / R2, pr = row - sd * R2;
      const int kx = (sd ? PX : KX) + (pr / R) * nc, ky = (sd ? PY : KY) + (pr % R) * nc;
      const uintptr_t a = (uintptr_t)(in + ((size_t)kx * N + ky) * S);
      fold_bulk(drows + row * DB, (const void *)(a & ~(uintptr_t)15), (unsigned)G::span(a & 15, (size_t)S * sizeof(C)),
                bar);
      if (tcol) {
        const uintptr_t b = (uintptr_t)(tcol + ((size_t)(kx > H ? N - kx : kx) * N + ky) * S);
        fold_bulk(trows + row * TB, (const void *)(b & ~(uintptr_t)15),
                  (unsigned)G::span(b & 15, (size_t)S * sizeof(T)), bar);
      }
    }
    if (threadIdx.x == 0) fold_bulk(bt, btab, (unsigned)(N * sizeof(C)), bar);
  }
  if (!tcol) {
    // the filter by |k|^2: a gather, element by element (no shift: rows start aligned)
    const int warp = (int)threadIdx.x >> 5, lane = (int)threadIdx.x & 31;
    for (int row = warp; row < nrow; row += NT / 32) {
      const int sd = row / R2, pr = row - sd * R2;
      const int kx = (sd ? PX : KX) + (pr / R) * nc, ky = (sd ? PY : KY) + (pr % R) * nc;
      const long long sx = kx > H ? kx - N : kx, sy = ky > H ? ky - N : ky, qxy = sx * sx + sy * sy;
      T *dst = reinterpret_cast<T *>(trows + row * TB);
      for (int kz = lane; kz < S; kz += 32) fold_cp_async<sizeof(T)>(dst + kz, tab + qxy + (long long)kz * kz);
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
  }
  if (threadIdx.x == 0 && !fold_mbar_wait(bar, wait_cycles)) {
    s_stop = 1;
    atomicExch(err, 4);
    fold_mbar_wait(bar, wait_cycles);  // the copies still in flight write this CTA's shared memory
  }
  __syncthreads();
  if (s_stop) return;
  // per alias row: offsets of the row and of its partner, in elements
  if ((int)threadIdx.x < nrow) {
    const int row = (int)threadIdx.x, sd = row / R2, pr = row - sd * R2;
    const int kx = (sd ? PX : KX) + (pr / R) * nc, ky = (sd ? PY : KY) + (pr % R) * nc;
    const int qx = (N - kx) % N, qy = (N - ky) % N;
    const int prow = (sides == 2 ? 1 - sd : 0) * R2 + (qx / nc) * R + qy / nc;
    auto dshift = [&](int x, int y) {
      return (int)(((uintptr_t)(in + ((size_t)x * N + y) * S) & 15) / sizeof(C));
    };
    auto tshift = [&](int x, int y) {
      return tcol ? (int)(((uintptr_t)(tcol + ((size_t)(x > H ? N - x : x) * N + y) * S) & 15) / sizeof(T)) : 0;
    };
    FoldPair<T> fp;
    fp.own = (int)(row * (DB / sizeof(C))) + dshift(kx, ky);
    fp.town = (int)(row * (TB / sizeof(T))) + tshift(kx, ky);
    fp.mir = (int)(prow * (DB / sizeof(C))) + dshift(qx, qy);
    fp.tmir = (int)(prow * (TB / sizeof(T))) + tshift(qx, qy);
    fp.noncanon = kx > H || ((kx == 0 || kx == H) && ky > H);
    const C bx = bt[kx], by = bt[ky];
    fp.bxy_r = bx.x * by.x - bx.y * by.y;
    fp.bxy_i = bx.x * by.y + bx.y * by.x;
    pairs[row] = fp;
  }
  __syncthreads();
  const C *g = reinterpret_cast<const C *>(drows);
  const T *tv = reinterpret_cast<const T *>(trows);
  // the alias pairs in NQ groups of PQ: a work item sums one group for one output
  // coefficient into part[group][output]
  constexpr int NQ = R2 < 4 ? R2 : 4, PQ = R2 / NQ;
  static_assert(R2 % NQ == 0, "equal groups of alias pairs");
  const int nout = sides * Sc;
  C *part = bt + N;
  for (int item = threadIdx.x; item < NQ * nout; item += NT) {
    const int q = item / nout, o = item - q * nout;
    const int side = o / Sc, KZ = o - side * Sc;
    T sr = 0, si = 0;
    for (int pr = q * PQ; pr < (q + 1) * PQ; ++pr) {
      const FoldPair<T> P = pairs[side * R2 + pr];
      T ar = 0, ai = 0;
#pragma unroll
      for (int mz = 0; mz < R; ++mz) {
        const int kz = KZ + mz * nc;
        const bool mir = kz > H || ((kz == 0 || kz == H) && P.noncanon);
        C f;
        T t;
        if (mir) {
          const int at = kz > H ? N - kz : kz;
          f = g[P.mir + at];
          f.y = -f.y;
          t = tv[P.tmir + at];
        } else {
          f = g[P.own + kz];
          t = tv[P.town + kz];
        }
        const C bz = bt[kz];
        const T b_r = P.bxy_r * bz.x - P.bxy_i * bz.y, b_i = P.bxy_r * bz.y + P.bxy_i * bz.x;
        const T fr = f.x * t, fi = f.y * t;
        ar += fr * b_r - fi * b_i;
        ai += fr * b_i + fi * b_r;
      }
      sr += ar;
      si += ai;
    }
    C v;
    v.x = sr;
    v.y = si;
    part[q * nout + o] = v;
  }
  __syncthreads();
  for (int o = threadIdx.x; o < nout; o += NT) {
    const int side = o / Sc, KZ = o - side * Sc;
    T sr = 0, si = 0;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      sr += part[q * nout + o].x;
      si += part[q * nout + o].y;
    }
    C res;
    res.x = sr * fac;
    res.y = si * fac;
    out[((size_t)(side ? PX : KX) * nc + (side ? PY : KY)) * Sc + KZ] = res;
  }
}

// coarse[(s + X) mod nc] += means[X] for X in [0, m)^3 (means: padded real layout of m^3)
template <typename T>
__global__ void k_block_add(const T *means, int m, int sx, int sy, int sz, T *coarse, int nc) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)m * m * m) return;
  const int k = (int)(i % m);
  const size_t rr = i / m;
  const int j = (int)(rr % m), ii = (int)(rr / m);
  const T v = means[((size_t)ii * m + j) * (size_t)(2 * (m / 2 + 1)) + k];
  int X = ((sx + ii) % nc + nc) % nc, Y = ((sy + j) % nc + nc) % nc, Z = ((sz + k) % nc + nc) % nc;
  coarse[((size_t)X * nc + Y) * (size_t)(2 * (nc / 2 + 1)) + Z] += v;
}

// transpose of k_subsample_add: every fine cell takes its coarse cell's value / r^3
template <typename T>
__global__ void k_subsample_transpose(const T *coarse, int nc, int r, int sx, int sy, int sz, T *fine, int nf) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)nf * nf * nf) return;
  int z = (int)(i % nf);
  size_t rr = i / nf;
  int y = (int)(rr % nf), x = (int)(rr / nf);
  int X = ((sx + x / r) % nc + nc) % nc, Y = ((sy + y / r) % nc + nc) % nc, Z = ((sz + z / r) % nc + nc) % nc;
  fine[((size_t)x * nf + y) * (size_t)(2 * (nf / 2 + 1)) + z] =
      coarse[((size_t)X * nc + Y) * (size_t)(2 * (nc / 2 + 1)) + Z] / (T)((double)r * r * r);
}

template <typename T>
__global__ void k_axes_geom(int nf, double dxf, double f0, double f1, double f2, double o0, double o1, double o2,
                            double dxc, double period, int nc, int *ubase, T *frac) {
  int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= 3 * nf) return;
  int a = id / nf, x = id % nf;
  double fo = a == 0 ? f0 : (a == 1 ? f1 : f2);
  double co = a == 0 ? o0 : (a == 1 ? o1 : o2);
  double lu = (double)x * dxf + fo + dxf / 2 - co;
  double l = fmod(lu, period);
  if (l < 0) l += period;
  double u = l / dxc - 0.5;
  double f = floor(u);
  frac[id] = (T)(u - f);
  ubase[id] = (int)f + (int)floor(lu / period) * nc;
}

// compact N^3 real arrays <-> padded real layout (rows of 2(N/2+1))
template <typename T>
__global__ void k_pad(const T *compact, T *padded, int n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)n * n * n) return;
  size_t row = i / n;
  padded[row * (size_t)(2 * (n / 2 + 1)) + (i - row * n)] = compact[i];
}
template <typename T>
__global__ void k_unpad(const T *padded, T *compact, int n, T scale) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)n * n * n) return;
  size_t row = i / n;
  compact[i] = padded[row * (size_t)(2 * (n / 2 + 1)) + (i - row * n)] * scale;
}

// multiply a half spectrum by the map of field `what` (0: delta = tab[q] w; 1-3:
// psi_a = i k_a tab[q] w / k^2, zero at k = 0 and where k_a is the Nyquist mode,
// zeldovich.hpp:155-181), or by its complex conjugate (the adjoint)
template <typename T>
__global__ void k_field_mult(typename V2m<T>::type *c, int n, const T *tab, T kmin, int what, int conj) {
  const int H = n / 2, S = H + 1;
  unsigned row;
  int iz;
  if (!hs_cell(n, row, iz)) return;
  int ix = (int)(row / (unsigned)n), iy = (int)(row % (unsigned)n);
  int kc[3] = {ix > H ? ix - n : ix, iy > H ? iy - n : iy, iz};
  long long q = (long long)kc[0] * kc[0] + (long long)kc[1] * kc[1] + (long long)kc[2] * kc[2];
  size_t id = (size_t)row * S + iz;
  typename V2m<T>::type v = c[id];
  T t = (T)tab[q];
  if (what == 0) {
    v.x *= t;
    v.y *= t;
  } else {
    int a = what - 1;
    T f[3] = {(T)kc[0] * kmin, (T)kc[1] * kmin, (T)kc[2] * kmin};
    T kk = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    T m = (q == 0 || kc[a] == H) ? (T)0 : t * f[a] / kk;
    T x = v.x, y = v.y;
    if (conj) {
      v.x = m * y;
      v.y = -m * x;
    } else {
      v.x = -m * y;
      v.y = m * x;
    }
  }
  c[id] = v;
}

inline unsigned nblk(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// axis a of `box`: the shortest cyclic range of n coordinates holding every occupied
// one (the complement of the longest run of empty ones), widened by `margin`
void cyclic_cover(CellBox &box, int a, const unsigned char *occupied, int n, int margin) {
  int best = 0, best_start = 0, run = 0;
  for (int k = 0; k < 2 * n; ++k) {
    if (occupied[k % n]) {
      run = 0;
      continue;
    }
    ++run;
    if (run > best && run <= n) {
      best = run;
      best_start = k - run + 1;
    }
  }
  if (best == n) {  // nothing occupied: an empty range stands for "no cells"; keep the whole axis
    box.start[a] = 0;
    box.len[a] = n;
    return;
  }
  box.set_axis(a, (long long)best_start + best, (long long)best_start + n, margin, n);
}

// box of a list of cells (x n + y) n + z of an n^3 grid, widened by `margin` cells
CellBox cells_box(const unsigned long long *cells, size_t count, int n, int margin) {
  CellBox b = CellBox::whole(n);
  if (count == 0) return b;
  std::vector<unsigned char> occ(3 * (size_t)n, 0);
  for (size_t i = 0; i < count; ++i) {
    unsigned long long c = cells[i];
    occ[2 * (size_t)n + c % n] = 1;
    c /= n;
    occ[(size_t)n + c % n] = 1;
    occ[c / n] = 1;
  }
  for (int a = 0; a < 3; ++a) cyclic_cover(b, a, &occ[(size_t)a * n], n, margin);
  return b;
}

}  // namespace

// --- the multi-level field algebra ------------------------------------------------

template <typename T>
struct ModEngine {
  using C = typename V2m<T>::type;
  Context &ctx;
  ModScratch &S;
  explicit ModEngine(Context &c) : ctx(c), S(c.modscratch) {}

  int nl() const { return (int)ctx.levels.size(); }
  Level &lev(int l) { return *ctx.levels[l]; }
  size_t elems(int l) { return 2 * lev(l).ncomplex(); }
  double scale(int l) { return 1.0 / std::pow((double)lev(l).n, 1.5); }

  // one half-spectrum (or padded real) buffer per level, taken from the context's pool
  struct Field {
    BufPool *pool = nullptr;
    std::vector<std::unique_ptr<DevBuf>> b;
    std::vector<char> fourier;
    Field() = default;
    Field(Field &&) = default;
    Field &operator=(Field &&) = delete;
    ~Field() {
      if (pool)
        for (auto &x : b) pool->give(std::move(x));
    }
  };

  void alloc(Field &f) {
    f.pool = &ctx.pool;
    f.b.resize(nl());
    f.fourier.assign(nl(), 1);
    for (int l = 0; l < nl(); ++l)
      if (!f.b[l] || f.b[l]->bytes < elems(l) * sizeof(T)) {
        ctx.pool.give(std::move(f.b[l]));
        f.b[l] = ctx.pool.take(elems(l) * sizeof(T));
      }
  }
  T *ptr(Field &f, int l) { return f.b[l]->template as<T>(); }
  void zero(Field &f, int l) { GIC_CUDA(cudaMemsetAsync(f.b[l]->ptr, 0, elems(l) * sizeof(T), ctx.stream)); }
  void copy(Field &dst, const Field &src) {
    alloc(dst);
    for (int l = 0; l < nl(); ++l) {
      GIC_CUDA(cudaMemcpyAsync(dst.b[l]->ptr, src.b[l]->ptr, elems(l) * sizeof(T), cudaMemcpyDeviceToDevice,
                               ctx.stream));
      dst.fourier[l] = src.fourier[l];
    }
  }
  void copy_level(DevBuf &dst, const DevBuf &src, int l) {
    dst.ensure(elems(l) * sizeof(T));
    GIC_CUDA(cudaMemcpyAsync(dst.ptr, src.ptr, elems(l) * sizeof(T), cudaMemcpyDeviceToDevice, ctx.stream));
  }
  // box: the forward transform's input is zero outside it / only the inverse
  // transform's output inside it is used (the transforms skip the rest)
  void to_fourier(T *p, int l, const CellBox *box = nullptr) { fft_r2c_3d<T>(ctx, p, lev(l).n, scale(l), nullptr, box); }
  void to_real(T *p, int l) { fft_c2r_3d<T>(ctx, p, lev(l).n, scale(l)); }
  // times the current table, then to real space: the multiply rides on the
  // transform's first pass (bit-identical to mul_table followed by to_real)
  void to_real_times_table(T *p, int l, const CellBox *box = nullptr) {
    fft_c2r_3d<T>(ctx, p, lev(l).n, scale(l), tabT(), box);
  }
  // cells of level c that the fine level f covers (margin: extra cells each side), cyclic
  CellBox footprint(int f, int c, int margin) { return footprint_box(lev(f), lev(c), margin); }
  void to_fourier(Field &f, int l) {
    if (!f.fourier[l]) to_fourier(ptr(f, l), l);
    f.fourier[l] = 1;
  }
  void to_real(Field &f, int l) {
    if (f.fourier[l]) to_real(ptr(f, l), l);
    f.fourier[l] = 0;
  }

  // family filter of level l (filterfamily.hpp:106-140) evaluated on grid g
  void add_filter_factors(TableSpec &sp, int l) {
    for (int m = 0; m < l; ++m) sp.hp_cut[sp.nhp++] = kcut(m);
    if (l < nl() - 1) sp.lp_cut[sp.nlp++] = kcut(l);
  }
  double kcut(int l) { return 0.3 * ((double)lev(l).n * lev(l).kmin()); }

  // the table of `sp0` on grid g becomes the current one: from the context's cache, or
  // built (k_mod_table, double with a float copy) and cached
  void table(const TableSpec &sp0, int g) {
    long long half = lev(g).n / 2, nq = 3 * half * half + 1;
    TableSpec sp = sp0;
    sp.kmin = lev(g).kmin();
    std::vector<unsigned char> key;
    auto put = [&key](const void *p, size_t n) {
      const unsigned char *b = static_cast<const unsigned char *>(p);
      key.insert(key.end(), b, b + n);
    };
    const int dims[6] = {g, lev(g).n, sp.nhp, sp.nlp, sp.power, (int)sizeof(T)};
    put(dims, sizeof(dims));
    put(&sp.kmin, sizeof(double));
    put(sp.hp_cut, sp.nhp * sizeof(double));
    put(sp.lp_cut, sp.nlp * sizeof(double));
    put(&sp.scalar, sizeof(double));
    put(&sp.sqrtp, sizeof(sp.sqrtp));
    put(&sp.vel, sizeof(double));
    put(&sp.var_cut, sizeof(double));
    put(&sp.offset, sizeof(double));
    for (auto &e : ctx.table_cache)
      if (e->key == key) {
        cur_tab = e.get();
        return;
      }
    if (ctx.table_cache.size() >= 128) ctx.clear_table_cache();
    auto e = std::make_unique<CachedTable>();
    e->key = std::move(key);
    e->d.ensure(nq * sizeof(double));
    if (sizeof(T) == 4) e->f.ensure(nq * sizeof(float));
    k_mod_table<<<nblk(nq), 256, 0, ctx.stream>>>(e->d.template as<double>(),
                                                 sizeof(T) == 4 ? e->f.template as<float>() : nullptr, nq, sp);
    launched();
    cur_tab = e.get();
    ctx.register_col_table(tabT(), lev(g).n, (int)sizeof(T), true);
    ctx.table_cache.push_back(std::move(e));
  }
  CachedTable *cur_tab = nullptr;
  // the current table in the fields' precision
  const T *tabT() const {
    if constexpr (sizeof(T) == 4) return cur_tab->f.template as<float>();
    else return cur_tab->d.template as<double>();
  }

  void mul_table(T *p, int g) {
    k_mul_table<T><<<hs_grid(lev(g).n), hs_block(), 0, ctx.stream>>>(reinterpret_cast<C *>(p), lev(g).n, tabT());
    launched();
  }
  void axpy(T *a, const T *b, double c, int l) {
    k_axpy<T><<<nblk(elems(l)), 256, 0, ctx.stream>>>(a, b, (T)c, elems(l));
    launched();
  }
  void scale_by(T *a, double c, int l) {
    k_scale<T><<<nblk(elems(l)), 256, 0, ctx.stream>>>(a, c, elems(l));
    launched();
  }

  // one term of an inner product: two half spectra or two padded real fields of level
  // l, or two flat arrays of `count` values
  // kRealBox: two padded real fields of level l over the cells of `box` only
  enum TermKind { kFourier = 0, kReal = 1, kFlat = 2, kRealBox = 3 };
  struct Term {
    const T *a, *b;
    int l;
    int kind;
    size_t count = 0;
    CellBox box{};
  };
  // sum of each group's terms; every group has the same number of terms, and all
  // groups are read back together
  std::vector<double> inner_groups(const std::vector<std::vector<Term>> &groups) {
    const int blocks = 152 * 8;
    const int np = (int)groups.size(), nt = np ? (int)groups[0].size() : 0;
    if (np == 0) return {};
    const size_t per = (size_t)nt * blocks;
    S.reduce.ensure((per * np + np) * sizeof(double));
    double *part = S.reduce.template as<double>();
    for (int p = 0; p < np; ++p)
      for (int i = 0; i < nt; ++i) {
        const Term &t = groups[p][i];
        double *dst = part + per * p + (size_t)i * blocks;
        if (t.kind == kReal)
          k_inner_real<T><<<blocks, red_block(), 0, ctx.stream>>>(t.a, t.b, lev(t.l).n, dst);
        else if (t.kind == kFlat)
          k_dot_flat<T><<<blocks, 256, 0, ctx.stream>>>(t.a, t.b, t.count, dst);
        else if (t.kind == kRealBox)
          k_inner_real_box<T><<<blocks, red_block(), 0, ctx.stream>>>(t.a, t.b, lev(t.l).n, t.box, dst);
        else if (reinterpret_cast<uintptr_t>(t.a) % 16 == 0 && reinterpret_cast<uintptr_t>(t.b) % 16 == 0) {
          BlockFields<T> bf{};
          bf.a[0] = t.a;
          bf.b[0] = t.b;
          bf.na = bf.nb = 1;
          k_inner_block_flat<T, 1, 1><<<blocks, 256, 0, ctx.stream>>>(bf, lev(t.l).n, dst, 0, 0, 1, 0);
        } else
          k_inner<T><<<blocks, red_block(), 0, ctx.stream>>>(t.a, t.b, lev(t.l).n, dst);
        launched();
      }
    k_sum<<<np, 256, 0, ctx.stream>>>(part, (int)per, part + per * np);
    launched();
    std::vector<double> out(np);
    read_small(ctx, part + per * np, np * sizeof(double), out.data());
    return out;
  }
  // <a_i|b_i> for every pair, summed over levels, in Fourier space
  std::vector<double> inner_many(const std::vector<std::pair<Field *, Field *>> &pairs) {
    std::vector<std::vector<Term>> groups;
    for (auto &pr : pairs) {
      std::vector<Term> g;
      for (int l = 0; l < nl(); ++l) {
        to_fourier(*pr.first, l);
        to_fourier(*pr.second, l);
        g.push_back({ptr(*pr.first, l), ptr(*pr.second, l), l, kFourier});
      }
      groups.push_back(std::move(g));
    }
    return inner_groups(groups);
  }
  double inner(Field &a, Field &b) { return inner_many({{&a, &b}})[0]; }

  // M[i][j] = <A_i|B_j> summed over levels (Fourier), each field read once per level
  // for every 4 x 5 block of products, left in device scratch (inner_block reads it back)
  const double *inner_block_dev(const std::vector<Field *> &A, const std::vector<Field *> &B) {
    // one wave of resident CTAs
    static std::atomic<int> per_sm{0};
    if (per_sm.load() == 0) {
      int nb = 0;
      GIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_inner_block<T>, kKzChunk * kRowsPerBlock, 0));
      per_sm.store(std::max(nb, 1));
    }
    static std::atomic<int> per_sm_flat{0};
    if (per_sm_flat.load() == 0) {
      int nb = 0;
      GIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_inner_block_flat<T, kBlockA, kBlockB>, 256, 0));
      per_sm_flat.store(std::max(nb, 1));
    }
    int nsm = 0;
    GIC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx.device));
    const int nb_row = per_sm.load() * nsm, blocks_flat = per_sm_flat.load() * nsm;
    const int blocks = std::max(nb_row, blocks_flat);
    const int L = nl(), na = (int)A.size(), nbt = (int)B.size(), np = na * nbt;
    if (np == 0) return nullptr;
    const size_t pstride = (size_t)L * blocks;
    S.reduce.ensure((pstride * np + np) * sizeof(double));
    double *part = S.reduce.template as<double>();
    // each product has `blocks` slots per level; a kernel with fewer CTAs leaves zeros
    if (nb_row != blocks_flat) GIC_CUDA(cudaMemsetAsync(part, 0, pstride * np * sizeof(double), ctx.stream));
    for (Field *f : A)
      for (int l = 0; l < L; ++l) to_fourier(*f, l);
    for (Field *f : B)
      for (int l = 0; l < L; ++l) to_fourier(*f, l);
    for (int ia = 0; ia < na; ia += kBlockA)
      for (int jb = 0; jb < nbt; jb += kBlockB)
        for (int l = 0; l < L; ++l) {
          BlockFields<T> bf{};
          bf.na = std::min(kBlockA, na - ia);
          bf.nb = std::min(kBlockB, nbt - jb);
          bool aligned = true;
          for (int i = 0; i < bf.na; ++i) {
            bf.a[i] = ptr(*A[ia + i], l);
            aligned = aligned && (reinterpret_cast<uintptr_t>(bf.a[i]) % 16 == 0);
          }
          for (int j = 0; j < bf.nb; ++j) {
            bf.b[j] = ptr(*B[jb + j], l);
            aligned = aligned && (reinterpret_cast<uintptr_t>(bf.b[j]) % 16 == 0);
          }
          // slots [l blocks, (l + 1) blocks) of each product; unused ones are zeroed
          double *slot = part + (size_t)l * blocks;
          if (aligned && bf.na == kBlockA && bf.nb == kBlockB) {
            k_inner_block_flat<T, kBlockA, kBlockB><<<blocks_flat, 256, 0, ctx.stream>>>(bf, lev(l).n, slot, ia, jb, nbt,
                                                                                        pstride);
          } else {
            k_inner_block<T><<<nb_row, red_block(), 0, ctx.stream>>>(bf, lev(l).n, slot, ia, jb, nbt, pstride);
          }
          launched();
        }
    k_sum<<<np, 256, 0, ctx.stream>>>(part, (int)pstride, part + pstride * np);
    launched();
    return part + pstride * np;
  }
  std::vector<double> inner_block(const std::vector<Field *> &A, const std::vector<Field *> &B) {
    const size_t np = A.size() * B.size();
    if (np == 0) return {};
    const double *d = inner_block_dev(A, B);
    std::vector<double> out(np);
    read_small(ctx, d, np * sizeof(double), out.data());
    return out;
  }

  // a += sum_k c[k] b[k] over a level's half spectrum, up to kMaxAxpy sources per pass;
  // the coefficients from c (host) or, when cdev is set, from device memory
  void axpy_many(T *a, const std::vector<const T *> &b, const std::vector<double> &c, int l,
                 const T *cdev = nullptr) {
    for (size_t k0 = 0; k0 < b.size(); k0 += kMaxAxpy) {
      AxpySources<T> src{};
      src.nb = (int)std::min<size_t>(kMaxAxpy, b.size() - k0);
      src.cdev = cdev ? cdev + k0 : nullptr;
      for (int k = 0; k < src.nb; ++k) {
        src.b[k] = b[k0 + k];
        src.c[k] = cdev ? (T)0 : (T)c[k0 + k];
      }
      constexpr int W = Vec16<T>::W;
      const size_t n = elems(l);
      bool aligned = n % W == 0 && (uintptr_t)a % 16 == 0;
      for (int k = 0; k < src.nb; ++k) aligned = aligned && (uintptr_t)src.b[k] % 16 == 0;
      if (aligned) {
        const size_t nv = n / W;
        switch (src.nb) {
          case 1: k_axpy_multi_vec<T, 1><<<nblk(nv), 256, 0, ctx.stream>>>(a, src, nv); break;
          case 2: k_axpy_multi_vec<T, 2><<<nblk(nv), 256, 0, ctx.stream>>>(a, src, nv); break;
          case 3: k_axpy_multi_vec<T, 3><<<nblk(nv), 256, 0, ctx.stream>>>(a, src, nv); break;
          case 4: k_axpy_multi_vec<T, 4><<<nblk(nv), 256, 0, ctx.stream>>>(a, src, nv); break;
          case 5: k_axpy_multi_vec<T, 5><<<nblk(nv), 256, 0, ctx.stream>>>(a, src, nv); break;
          case 6: k_axpy_multi_vec<T, 6><<<nblk(nv), 256, 0, ctx.stream>>>(a, src, nv); break;
          case 7: k_axpy_multi_vec<T, 7><<<nblk(nv), 256, 0, ctx.stream>>>(a, src, nv); break;
          default: k_axpy_multi_vec<T, 8><<<nblk(nv), 256, 0, ctx.stream>>>(a, src, nv); break;
        }
      } else {
        k_axpy_multi<T><<<nblk(n), 256, 0, ctx.stream>>>(a, src, n);
      }
      launched();
    }
  }

  // window of level wl on the cells of level l, per axis (window.hpp)
  // the cached geometry entry of `key` (created empty when new)
  GeomEntry &geom_entry(const std::vector<double> &key, bool &fresh) {
    for (auto &e : S.geom_cache)
      if (e->key == key) {
        fresh = false;
        return *e;
      }
    if (S.geom_cache.size() >= 64)  // keep the masks in use; cudaFree orders after pending work
      for (size_t i = S.geom_cache.size(); i-- > 0;)
        if (S.geom_cache[i]->dev.ptr != (const void *)S.cur_masks) S.geom_cache.erase(S.geom_cache.begin() + i);
    S.geom_cache.push_back(std::make_unique<GeomEntry>());
    S.geom_cache.back()->key = key;
    fresh = true;
    return *S.geom_cache.back();
  }

  void window_masks(int l, int wl) {
    const Level &L = lev(l), &W = lev(wl);
    bool fresh = false;
    GeomEntry &g = geom_entry({1.0, (double)l, (double)wl, (double)L.n, L.dx, L.x0[0], L.x0[1], L.x0[2], L.periodic,
                               W.box, W.x0[0], W.x0[1], W.x0[2]},
                              fresh);
    if (!fresh) {
      S.cur_masks = g.dev.template as<unsigned char>();
      win_box = g.box;
      return;
    }
    double P = L.periodic;
    std::vector<unsigned char> m(3 * (size_t)L.n);
    for (int a = 0; a < 3; ++a) {
      auto wrap = [P](double v) {
        if (v < 0) v += P;
        if (v >= P) v -= P;
        return v;
      };
      double lo = wrap(W.x0[a]), hi = wrap(W.x0[a] + W.box);
      for (int i = 0; i < L.n; ++i) {
        double c = (double)i * L.dx + L.x0[a] + L.dx / 2;
        bool in = lo <= hi ? (c < hi && c >= lo) : (c < hi || c >= lo);
        m[(size_t)a * L.n + i] = in ? 1 : 0;
      }
    }
    g.dev.ensure(m.size());
    GIC_CUDA(cudaMemcpyAsync(g.dev.ptr, m.data(), m.size(), cudaMemcpyHostToDevice, ctx.stream));
    GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    g.box = CellBox::whole(L.n);
    for (int a = 0; a < 3; ++a) cyclic_cover(g.box, a, &m[(size_t)a * L.n], L.n, 0);
    S.cur_masks = g.dev.template as<unsigned char>();
    win_box = g.box;
  }
  CellBox win_box;  // cells inside the last window_masks' window
  // rows: only these rows (x and y ranges of the box) are combined; null: all
  void window_op(T *r, const T *src, int l, int op, const CellBox *rows = nullptr) {
    int n = lev(l).n;
    const unsigned char *m = S.cur_masks;
    const int x0 = rows ? rows->start[0] : 0, nx = rows ? rows->len[0] : n;
    const int y0 = rows ? rows->start[1] : 0, ny = rows ? rows->len[1] : n;
    k_window_op<T><<<(unsigned)((size_t)nx * ny), real_block(n), 0, ctx.stream>>>(r, src, n, m, m + n, m + 2 * n, op,
                                                                                   x0, ny > 0 ? y0 : 0, ny);
    launched();
  }

  // f_l applied in Fourier space
  void apply_family(T *p, int l, int power) {
    family_table(l, power);
    mul_table(p, l);
  }
  void family_table(int l, int power) {
    TableSpec sp{};
    sp.power = power;
    sp.scalar = 1.0;
    add_filter_factors(sp, l);
    table(sp, l);
  }

  double level_weight(int l) {
    double r = lev(l).dx / lev(0).dx;
    return r * r * r;
  }

  // The block means of the finer level s (spectrum source_k times the current table), added
  // into the coarse real field of level t, formed in Fourier space (k_fold_block_means)
  // and inverse-transformed on the (n_s/r)^3 grid: one pass over the fine spectrum
  // instead of its n_s^3 inverse transform.  False when the geometry does not allow it.
  bool fold_block_means(T *target_real, int t, const T *source_k, int s) {
    const Level &F = lev(s), &Cl = lev(t);
    const int r = (int)std::lround(Cl.dx / F.dx);
    if (r < 2 || F.n % r || (F.n / r) % 2 || F.n / r < 8) return false;
    const int nc = F.n / r;
    // b(k) = (1/r) sum_j exp(+2 pi i k j / N), cached per (N, r)
    if (S.btab_n != F.n || S.btab_r != r) {
      std::vector<C> hb(F.n);
      for (int k = 0; k < F.n; ++k) {
        long double sr = 0, si = 0;
        for (int j = 0; j < r; ++j) {
          const long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)k * j / (long double)F.n;
          sr += cosl(a);
          si += sinl(a);
        }
        hb[k].x = (T)(sr / r);
        hb[k].y = (T)(si / r);
      }
      S.btab.ensure(F.n * sizeof(C));
      GIC_CUDA(cudaMemcpyAsync(S.btab.ptr, hb.data(), F.n * sizeof(C), cudaMemcpyHostToDevice, ctx.stream));
      GIC_CUDA(cudaStreamSynchronize(ctx.stream));
      S.btab_n = F.n;
      S.btab_r = r;
    }
    const size_t ncomplex = (size_t)nc * nc * (nc / 2 + 1);
    S.fold.ensure(ncomplex * sizeof(C));
    C *g = S.fold.template as<C>();
    const T fac = (T)std::pow((double)r, -1.5);
    const C *src = reinterpret_cast<const C *>(source_k);
    const C *bt = S.btab.template as<C>();
    // 32 coefficients per CTA, the r^2 alias pairs over its warps
    const unsigned ctas = nblk(ncomplex, 32);
    const T *tc = coefficient_table<T>(ctx, tabT(), F.n);
    // by fine rows where a CTA's 2 r^2 rows, their filter values and b(k) fit in shared memory
    const size_t rows_smem = FoldRowGeom<T>::smem(r, F.n);
    const bool aligned = (((uintptr_t)src | (uintptr_t)tc | (uintptr_t)bt) & 15) == 0;
    if ((r == 2 || r == 4) && F.n % 4 == 0 && aligned && rows_smem <= kFoldRowsSmem) {
      static std::atomic<int> done2{0}, done4{0};
      const void *fn = r == 2 ? (const void *)k_fold_rows<T, 2, 256> : (const void *)k_fold_rows<T, 4, 256>;
      std::atomic<int> &done = r == 2 ? done2 : done4;
      if (!(done.load() & (1 << (ctx.device & 31)))) {
        GIC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFoldRowsSmem));
        done.fetch_or(1 << (ctx.device & 31));
      }
      // the column pairs: K_x in [1, nc/2) with every K_y, K_x = 0 and nc/2 with K_y <= nc/2
      const unsigned cols = (unsigned)((nc / 2 - 1) * nc + 2 * (nc / 2 + 1));
      int *err = ctx.fft.wait_flag();
      const long long wait_cycles = 1ll << 31;
      if (r == 2)
        k_fold_rows<T, 2, 256><<<cols, 256, rows_smem, ctx.stream>>>(g, src, F.n, tabT(), tc, bt, fac, err, wait_cycles);
      else
        k_fold_rows<T, 4, 256><<<cols, 256, rows_smem, ctx.stream>>>(g, src, F.n, tabT(), tc, bt, fac, err, wait_cycles);
    } else if (r == 2) k_fold_block_means<T, 2, 4><<<ctas, 128, 0, ctx.stream>>>(g, src, F.n, r, tabT(), bt, fac, tc);
    else if (r == 4) k_fold_block_means<T, 4, 16><<<ctas, 512, 0, ctx.stream>>>(g, src, F.n, r, tabT(), bt, fac, tc);
    else if (r == 8) k_fold_block_means<T, 8, 16><<<ctas, 512, 0, ctx.stream>>>(g, src, F.n, r, tabT(), bt, fac, tc);
    else k_fold_block_means<T, 0, 8><<<ctas, 256, 0, ctx.stream>>>(g, src, F.n, r, tabT(), bt, fac, tc);
    launched();
    fft_c2r_3d<T>(ctx, reinterpret_cast<T *>(g), nc, std::pow((double)nc, -1.5));
    const int sx = (int)std::lround((F.x0[0] - Cl.x0[0]) / Cl.dx), sy = (int)std::lround((F.x0[1] - Cl.x0[1]) / Cl.dx),
              sz = (int)std::lround((F.x0[2] - Cl.x0[2]) / Cl.dx);
    const size_t m3 = (size_t)nc * nc * nc;
    k_block_add<T><<<nblk(m3), 256, 0, ctx.stream>>>(reinterpret_cast<const T *>(g), nc, sx, sy, sz, target_real, Cl.n);
    launched();
    return true;
  }

  // assign: a coarser source's interpolation replaces target_real (every cell of the
  // finer level is written) instead of adding to it
  void cross_term_impl(T *target_real, int t, const T *source_k, int s, bool assign = false) {
    TableSpec sp{};
    sp.power = 1;
    add_filter_factors(sp, t);
    add_filter_factors(sp, s);
    sp.scalar = std::sqrt(level_weight(t) / level_weight(s));
    table(sp, s);
    if (s > t && fold_block_means(target_real, t, source_k, s)) return;
    S.tmp_src.ensure(elems(s) * sizeof(T));
    // source (Fourier, unchanged) times the table, to real space in tmp_src; the
    // interpolation up reads the coarse cells around the fine level only
    const CellBox fp = footprint(t, s, 3);
    fft_c2r_3d_from<T>(ctx, S.tmp_src.template as<T>(), source_k, lev(s).n, scale(s), tabT(), s < t ? &fp : nullptr);
    if (s < t) {
      const T *src[1] = {S.tmp_src.template as<T>()};
      T *dst[1] = {target_real};
      interp_add<T, 1>(ctx, lev(s), src, lev(t), dst, assign);
    } else {
      const Level &F = lev(s), &Cl = lev(t);
      int r = (int)std::lround(Cl.dx / F.dx);
      int sx = (int)std::lround((F.x0[0] - Cl.x0[0]) / Cl.dx), sy = (int)std::lround((F.x0[1] - Cl.x0[1]) / Cl.dx),
          sz = (int)std::lround((F.x0[2] - Cl.x0[2]) / Cl.dx);
      size_t m = (size_t)(F.n / r);
      k_subsample_add<T><<<nblk(m * m * m), 256, 0, ctx.stream>>>(S.tmp_src.template as<T>(), F.n, r, sx, sy, sz, target_real,
                                                                  Cl.n);
      launched();
    }
  }

  // MultiLevelField::applyMetric (multilevelfield.hpp:344-384): X in Fourier space
  void apply_metric(Field &X, Field &out, bool to_covector) {
    for (int l = 0; l < nl(); ++l) to_fourier(X, l);
    alloc(out);
    DevBuf &inw = S.win;
    for (int t = 0; t < nl(); ++t) {
      T *R = ptr(out, t);
      if (to_covector && t < nl() - 1) {
        fft_c2r_3d_from<T>(ctx, R, ptr(X, t), lev(t).n, scale(t));
        windowed_covector_real(X, t, R);
        to_fourier(R, t);
      } else {
        // f_t^2 X_t stays in Fourier space; the cross-level terms are summed in real
        // space and transformed once: R = f_t^2 X_t + FFT(sum_s cross_s), in one pass
        const C *add = nullptr;
        if (nl() > 1) {
          inw.ensure(elems(t) * sizeof(T));
          T *Cr = inw.template as<T>();
          // with no coarser source (t = 0) the block means of the finer levels fill only
          // the next level's footprint: only its planes are zeroed (the transform reads
          // those only); otherwise the coarser source's interpolation assigns every cell
          const CellBox fp = footprint(std::min(t + 1, nl() - 1), t, 1);
          bool first = true;
          if (t == 0) {
            if (fft_prunes(ctx, lev(0).n)) zero_planes(Cr, 0, fp);
            else GIC_CUDA(cudaMemsetAsync(Cr, 0, elems(t) * sizeof(T), ctx.stream));
            first = false;
          }
          for (int s = 0; s < nl(); ++s)
            if (s != t) {
              cross_term_impl(Cr, t, ptr(X, s), s, first && s < t);
              first = false;
            }
          // R = f_t^2 X_t + FFT(Cr), the sum formed by the transform's last pass
          family_table(t, 2);
          fft_r2c_3d_add<T>(ctx, Cr, lev(t).n, scale(t), nullptr, t == 0 ? &fp : nullptr, R, ptr(X, t), tabT());
        } else {
          family_table(t, 2);
          k_mul_table_add<T><<<hs_grid(lev(t).n), hs_block(), 0, ctx.stream>>>(
              reinterpret_cast<C *>(R), reinterpret_cast<const C *>(ptr(X, t)), lev(t).n, tabT(), add);
          launched();
        }
      }
      out.fourier[t] = 1;
    }
  }

  // Towards a covector on a level t with a finer level inside it: R (real, holding
  // X_t in real space on entry) becomes, in real space,
  //   g = f (W x) + (1 - W) x            applyFilterInWindow(f, window, true)
  //   R = W f g + (1 - W) g              applyFilterInWindow(f, window, false)
  // plus the cross-level terms (field.hpp:752-775, multilevelfield.hpp:344-384).
  // The reference transforms after each masking; the sums are formed here in real
  // space, which needs four transforms instead of six.
  void windowed_covector_real(Field &X, int t, T *R) {
    windowed_self_real(t, R);
    for (int s = 0; s < nl(); ++s)
      if (s != t) cross_term_impl(R, t, ptr(X, s), s);
  }
  // the level's own part P1^T P1 x, P1 = f W + (1 - W): symmetric
  void windowed_self_real(int t, T *R) {
    window_masks(t, t + 1);
    S.win.ensure(elems(t) * sizeof(T));
    T *I = S.win.template as<T>();
    const CellBox wb = win_box;
    // I = W x, zero outside the window.  The box-restricted transform reads the window's
    // x planes and the row tiles (at most 32 rows) around its y range only, so only those
    // rows are written (the whole field when the transform is not box-restricted)
    CellBox rows_wide = wb;
    rows_wide.set_axis(1, wb.start[1], (long long)wb.start[1] + wb.len[1], 32, lev(t).n);
    window_op(I, R, t, 2, fft_prunes(ctx, lev(t).n) ? &rows_wide : nullptr);
    to_fourier(I, t, &wb);
    family_table(t, 1);
    to_real_times_table(I, t);
    window_op(R, I, t, 0);  // g = (1 - W) x + f (W x)
    GIC_CUDA(cudaMemcpyAsync(I, R, elems(t) * sizeof(T), cudaMemcpyDeviceToDevice, ctx.stream));
    to_fourier(I, t);
    family_table(t, 1);
    to_real_times_table(I, t, &wb);  // f g is read inside the window only
    window_op(R, I, t, 1, &wb);  // R = W (f g) + (1 - W) g: the window's rows only
  }

  // Transpose of the covector metric (apply_metric(X, out, true)).  The level
  // blocks are symmetric; the cross block (s <- t) = move_{t->s} F_t (filter
  // f_s f_t sqrt(w_s/w_t) on grid t, then interpolation up or block means down)
  // transposes to F_t move^T_{s->t}: the transposed interpolation (deinterpolation
  // at unit scale) or the transposed block mean (each fine cell takes its coarse
  // cell's value / r^3).
  void apply_metric_cov_transpose(Field &X, Field &out) {
    for (int l = 0; l < nl(); ++l) to_fourier(X, l);
    alloc(out);
    for (int t = 0; t < nl(); ++t) {
      T *R = ptr(out, t);
      GIC_CUDA(cudaMemcpyAsync(R, ptr(X, t), elems(t) * sizeof(T), cudaMemcpyDeviceToDevice, ctx.stream));
      if (t < nl() - 1) {
        to_real(R, t);
        windowed_self_real(t, R);
      } else {
        apply_family(R, t, 2);
        to_real(R, t);
      }
      for (int s = 0; s < nl(); ++s)
        if (s != t) cross_transpose_add(R, t, ptr(X, s), s);
      to_fourier(R, t);
      out.fourier[t] = 1;
    }
  }
  void cross_transpose_add(T *target_real, int t, const T *source_k, int s) {
    auto src = ctx.pool.take(elems(s) * sizeof(T)), buf = ctx.pool.take(elems(t) * sizeof(T));
    T *xs = src->template as<T>(), *b = buf->template as<T>();
    GIC_CUDA(cudaMemcpyAsync(xs, source_k, elems(s) * sizeof(T), cudaMemcpyDeviceToDevice, ctx.stream));
    to_real(xs, s);
    GIC_CUDA(cudaMemsetAsync(b, 0, elems(t) * sizeof(T), ctx.stream));
    if (s > t) {
      deinterpolate(xs, s, b, t, true);
    } else {
      const Level &F = lev(t), &Cl = lev(s);
      int r = (int)std::lround(Cl.dx / F.dx);
      int sx = (int)std::lround((F.x0[0] - Cl.x0[0]) / Cl.dx), sy = (int)std::lround((F.x0[1] - Cl.x0[1]) / Cl.dx),
          sz = (int)std::lround((F.x0[2] - Cl.x0[2]) / Cl.dx);
      k_subsample_transpose<T><<<nblk(F.ncells()), 256, 0, ctx.stream>>>(xs, Cl.n, r, sx, sy, sz, b, F.n);
      launched();
    }
    to_fourier(b, t);
    TableSpec sp{};
    sp.power = 1;
    add_filter_factors(sp, s);
    add_filter_factors(sp, t);
    sp.scalar = std::sqrt(level_weight(s) / level_weight(t));
    table(sp, t);
    to_real_times_table(b, t);
    axpy(target_real, b, 1.0, t);
    ctx.pool.give(std::move(src));
    ctx.pool.give(std::move(buf));
  }

  // <C_cov X | X> (OutputField::getChi2 through the covector metric), with the
  // windowed levels' terms summed in real space
  double chi2(Field &X) {
    for (int l = 0; l < nl(); ++l) to_fourier(X, l);
    std::vector<std::unique_ptr<DevBuf>> keep;
    std::vector<Term> terms;
    for (int t = 0; t < nl(); ++t) {
      const size_t bytes = elems(t) * sizeof(T);
      if (t < nl() - 1) {
        // The level's own covector part is P1^T P1 x with P1 = f W + (1 - W)
        // (windowed_self_real), so its term <P1^T P1 x|x> is |P1 x|^2, and
        // P1 x = x + (f - 1) W x is X + (f - 1) FFT(W x) in Fourier space: formed by
        // the forward transform's last pass.  The cross terms add <cross|x> in real
        // space.  x is then needed inside the window and where the cross terms land
        // only: on the coarsest level (no coarser source) that is the next level's
        // footprint, and the transforms are box-restricted to it.
        const int n = lev(t).n;
        const bool prune = fft_prunes(ctx, n);
        const bool in_box = prune && t == 0;
        const CellBox B = in_box ? footprint(t + 1, t, 1) : CellBox::whole(n);
        auto xr = ctx.pool.take(bytes), G = ctx.pool.take(bytes), Cr = ctx.pool.take(bytes);
        T *x = xr->template as<T>(), *g = G->template as<T>(), *cr = Cr->template as<T>();
        fft_c2r_3d_from<T>(ctx, x, ptr(X, t), n, scale(t), nullptr, in_box ? &B : nullptr);
        window_masks(t, t + 1);
        const CellBox wb = win_box;
        CellBox rows_wide = wb;
        rows_wide.set_axis(1, wb.start[1], (long long)wb.start[1] + wb.len[1], 32, n);
        S.win.ensure(bytes);
        T *I = S.win.template as<T>();
        window_op(I, x, t, 2, prune ? &rows_wide : nullptr);  // I = W x
        TableSpec one{}, fm{};
        one.power = fm.power = 1;
        one.scalar = fm.scalar = 1.0;
        add_filter_factors(fm, t);
        fm.offset = -1.0;
        // a lookup that finds its table builds nothing and evicts nothing: both stay valid
        table(one, t);
        table(fm, t);
        const T *tab_fm = tabT();
        table(one, t);
        const T *tab_one = tabT();
        fft_r2c_3d_add<T>(ctx, I, n, scale(t), tab_fm, &wb, g, ptr(X, t), tab_one);
        terms.push_back({g, g, t, kFourier});
        if (in_box) zero_planes(cr, t, B);
        else GIC_CUDA(cudaMemsetAsync(cr, 0, bytes, ctx.stream));
        for (int s = 0; s < nl(); ++s)
          if (s != t) cross_term_impl(cr, t, ptr(X, s), s);
        terms.push_back({cr, x, t, in_box ? kRealBox : kReal, 0, B});
        keep.push_back(std::move(xr));
        keep.push_back(std::move(G));
        keep.push_back(std::move(Cr));
      } else {
        auto R = ctx.pool.take(bytes);
        T *r = R->template as<T>();
        if (nl() > 1) {
          S.win.ensure(bytes);
          T *Cr = S.win.template as<T>();
          // t is the finest level: the first (coarser) source's interpolation assigns
          for (int s = 0; s < nl(); ++s)
            if (s != t) cross_term_impl(Cr, t, ptr(X, s), s, s == 0);
          // r = f_t^2 X_t + FFT(Cr), formed by the transform's last pass
          family_table(t, 2);
          fft_r2c_3d_add<T>(ctx, Cr, lev(t).n, scale(t), nullptr, nullptr, r, ptr(X, t), tabT());
        } else {
          GIC_CUDA(cudaMemcpyAsync(r, ptr(X, t), bytes, cudaMemcpyDeviceToDevice, ctx.stream));
          apply_family(r, t, 2);
        }
        terms.push_back({r, ptr(X, t), t, kFourier});
        keep.push_back(std::move(R));
      }
    }
    double v = inner_groups({terms})[0];
    for (auto &b : keep) ctx.pool.give(std::move(b));
    return v;
  }

  // --- quadratic (variance) modification ---------------------------------------

  void upload_cells(QuadRequest &q) {
    if (q.dcells.size() == q.cells.size()) return;
    q.dcells.clear();
    for (auto &c : q.cells) {
      auto b = std::make_unique<DevBuf>();
      if (!c.empty()) {
        b->ensure(c.size() * sizeof(unsigned long long));
        GIC_CUDA(cudaMemcpyAsync(b->ptr, c.data(), c.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                                 ctx.stream));
      }
      q.dcells.push_back(std::move(b));
    }
  }

  // real field of level l: keep the flagged cells, zero the rest; with `center`,
  // also apply the variance operator to the kept values
  void window_cells(T *real, int l, QuadRequest &q, bool center) {
    const size_t count = q.cells[l].size();
    const unsigned long long *cells = q.dcells[l]->template as<unsigned long long>();
    T *v = nullptr;
    if (count) {
      S.compact.ensure(count * sizeof(T));
      v = S.compact.template as<T>();
      k_gather_cells<T><<<nblk(count), 256, 0, ctx.stream>>>(real, lev(l).n, cells, count, v);
      launched();
      if (center) {
        k_center_cells<T><<<1, 1024, 0, ctx.stream>>>(v, count);
        launched();
      }
    }
    GIC_CUDA(cudaMemsetAsync(real, 0, elems(l) * sizeof(T), ctx.stream));
    if (count) {
      k_scatter_cells<T><<<nblk(count), 256, 0, ctx.stream>>>(v, lev(l).n, cells, count, real);
      launched();
    }
  }

  void mul_sqrtp_dm(T *p, int l) {
    build_sqrtp_dm(l);
    TableSpec sp{};
    sp.power = 1;
    sp.scalar = 1.0;
    sp.sqrtp = lev(l).sqrtp_dm.template as<double>();
    table(sp, l);
    mul_table(p, l);
  }

  void variance_highpass_table(int l, double scale) {
    TableSpec sp{};
    sp.power = 1;
    sp.scalar = 1.0;
    sp.var_cut = 2. * M_PI / scale;
    table(sp, l);
  }

  // QuadraticModification::pushMultiLevelFieldThroughMatrix (quadraticmodification.hpp:59-92)
  // with FilteredVarianceModification::pushOneLevelFieldThroughMatrix (:152-170):
  // out = sqrt(P) C_cov [W F V F W] sqrt(P) X, a covector in Fourier space
  void push_variance(Field &X, QuadRequest &q, Field &out) {
    Field R;
    alloc(R);
    for (int l = 0; l < nl(); ++l) {
      to_fourier(X, l);
      T *p = ptr(R, l);
      GIC_CUDA(cudaMemcpyAsync(p, ptr(X, l), elems(l) * sizeof(T), cudaMemcpyDeviceToDevice, ctx.stream));
      mul_sqrtp_dm(p, l);
    }
    apply_Q(R, q);
    apply_metric(R, out, true);
    for (int l = 0; l < nl(); ++l) mul_sqrtp_dm(ptr(out, l), l);
  }

  // The transpose of the pushed map: sqrt(P) [W F V F W] C_cov^T sqrt(P) X.  With
  // push_variance it gives the gradient (A + A^T) X of <A X|X>.
  void push_variance_transpose(Field &X, QuadRequest &q, Field &out) {
    Field R;
    alloc(R);
    for (int l = 0; l < nl(); ++l) {
      to_fourier(X, l);
      T *p = ptr(R, l);
      GIC_CUDA(cudaMemcpyAsync(p, ptr(X, l), elems(l) * sizeof(T), cudaMemcpyDeviceToDevice, ctx.stream));
      mul_sqrtp_dm(p, l);
      R.fourier[l] = 1;
    }
    apply_metric_cov_transpose(R, out);
    apply_Q(out, q);
    for (int l = 0; l < nl(); ++l) {
      to_fourier(out, l);
      mul_sqrtp_dm(ptr(out, l), l);
    }
  }

  // per level W F V F W (pushOneLevelFieldThroughMatrix): Fourier in, real out
  void apply_Q(Field &R, QuadRequest &q) {
    upload_cells(q);
    for (int l = 0; l < nl(); ++l) {
      T *p = ptr(R, l);
      to_real(R, l);
      window_cells(p, l, q, false);
      variance_highpass_table(l, q.scale);
      to_fourier(p, l);
      to_real_times_table(p, l);
      window_cells(p, l, q, true);  // windowOperator then the variance operator
      to_fourier(p, l);
      to_real_times_table(p, l);
      window_cells(p, l, q, false);
      R.fourier[l] = 0;
    }
  }

  // --- realisation maps on real-space white noise, and their adjoints -----------
  // No reference counterpart: they serve gradients through the realisation.  The
  // white noise of a level is taken as the real field w (unit gaussians); its
  // unitary transform is the half spectrum genetIC draws.  Level L's field is
  // C2R(m_L R2C(w_L)), plus for a zoom level L = 1 the base level's
  // C2R(m_LP R2C(w_0)) interpolated onto the zoom cells; the adjoint applies
  // conj(m) and, for the coarse part, the transposed interpolation.

  void pad_from(const void *compact, T *padded, int l) {
    k_pad<T><<<nblk(lev(l).ncells()), 256, 0, ctx.stream>>>(static_cast<const T *>(compact), padded, lev(l).n);
    launched();
  }
  void unpad_to(const T *padded, void *compact, int l, T scale = (T)1) {
    k_unpad<T><<<nblk(lev(l).ncells()), 256, 0, ctx.stream>>>(padded, static_cast<T *>(compact), lev(l).n, scale);
    launched();
  }
  void field_mult(T *p, int l, const T *tab, int what, int conj) {
    k_field_mult<T><<<hs_grid(lev(l).n), hs_block(), 0, ctx.stream>>>(reinterpret_cast<C *>(p), lev(l).n, tab,
                                                                       (T)lev(l).kmin(), what, conj);
    launched();
  }
  void check_map(int L, int what) {
    if (L < 0 || L >= nl()) fail(GIC_ERR_INVALID_ARG, "level out of range");
    if (what < 0 || what > 3) fail(GIC_ERR_INVALID_ARG, "field must be delta or a displacement component");
    if (L > 1) fail(GIC_ERR_INVALID_ARG, "gradients through the zoom combination are available for the first zoom level");
  }

  void map_forward(int L, int what, const void *const *noise, void *out) {
    check_map(L, what);
    level_tables(ctx, L);
    auto b = ctx.pool.take(elems(L) * sizeof(T));
    T *p = b->template as<T>();
    pad_from(noise[L], p, L);
    to_fourier(p, L);
    field_mult(p, L, tab_main<T>(lev(L)), what, 0);
    to_real(p, L);
    if (L == 1) {
      lowpass_tables(ctx, 0);
      auto c = ctx.pool.take(elems(0) * sizeof(T));
      T *q = c->template as<T>();
      pad_from(noise[0], q, 0);
      to_fourier(q, 0);
      field_mult(q, 0, tab_lp_src<T>(lev(0)), what, 0);
      to_real(q, 0);
      const T *src[1] = {q};
      T *dst[1] = {p};
      interp_add<T, 1>(ctx, lev(0), src, lev(1), dst);
      ctx.pool.give(std::move(c));
    }
    unpad_to(p, out, L);
    GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    ctx.pool.give(std::move(b));
  }

  void map_adjoint(int L, int what, const void *g, void *const *grad) {
    check_map(L, what);
    level_tables(ctx, L);
    for (int l = 0; l < nl(); ++l)
      if (l != L && !(L == 1 && l == 0) && grad[l])
        GIC_CUDA(cudaMemsetAsync(grad[l], 0, lev(l).ncells() * sizeof(T), ctx.stream));
    auto b = ctx.pool.take(elems(L) * sizeof(T));
    T *p = b->template as<T>();
    pad_from(g, p, L);
    std::unique_ptr<DevBuf> c;
    if (L == 1) {
      // transposed interpolation of the zoom-level gradient onto the base level
      lowpass_tables(ctx, 0);
      c = ctx.pool.take(elems(0) * sizeof(T));
      T *q = c->template as<T>();
      GIC_CUDA(cudaMemsetAsync(q, 0, elems(0) * sizeof(T), ctx.stream));
      deinterpolate(p, 1, q, 0, true);
    }
    to_fourier(p, L);
    field_mult(p, L, tab_main<T>(lev(L)), what, 1);
    to_real(p, L);
    unpad_to(p, grad[L], L);
    if (L == 1) {
      T *q = c->template as<T>();
      to_fourier(q, 0);
      field_mult(q, 0, tab_lp_src<T>(lev(0)), what, 1);
      to_real(q, 0);
      unpad_to(q, grad[0], 0);
    }
    GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    ctx.pool.give(std::move(b));
    if (c) ctx.pool.give(std::move(c));
  }

  // value <A w|w> of the variance functional (p = A w is the pushed covector,
  // quadraticmodification.hpp:51-92) and its gradient: exact, (A + A^T) w, or the
  // direction of the reference's quadratic solver, 2 p (equal when A is symmetric,
  // as on one level)
  double variance_grad(QuadRequest &q, const void *const *noise, void *const *grad, bool exact) {
    Field W, P;
    alloc(W);
    for (int l = 0; l < nl(); ++l) {
      pad_from(noise[l], ptr(W, l), l);
      W.fourier[l] = 0;
      to_fourier(W, l);
    }
    push_variance(W, q, P);
    double v = inner(P, W);
    if (exact) {
      Field PT;
      push_variance_transpose(W, q, PT);
      for (int l = 0; l < nl(); ++l) {
        axpy(ptr(P, l), ptr(PT, l), 1.0, l);
        to_real(P, l);
        unpad_to(ptr(P, l), grad[l], l, (T)1);
      }
    } else {
      for (int l = 0; l < nl(); ++l) {
        to_real(P, l);
        unpad_to(ptr(P, l), grad[l], l, (T)2);
      }
    }
    GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    return v;
  }

  void noise_to_real(int l, void *out) {
    if (!lev(l).have_noise) fail(GIC_ERR_NOT_READY, "white noise has not been drawn");
    auto b = ctx.pool.take(elems(l) * sizeof(T));
    GIC_CUDA(cudaMemcpyAsync(b->ptr, lev(l).noise.ptr, elems(l) * sizeof(T), cudaMemcpyDeviceToDevice, ctx.stream));
    to_real(b->template as<T>(), l);
    unpad_to(b->template as<T>(), out, l);
    GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    ctx.pool.give(std::move(b));
  }

  // --- splicing (splice.hpp:37-118, tools/numerics/cg.hpp:13-59) -------------------
  // genetIC holds a real field compact at the front of the padded transform buffer; its
  // +=, -=, addScaled, negation and innerProduct run over the whole buffer, the mask
  // multiply over the n^3 values only.  The CG's scalars therefore include the
  // buffer's tail, the part of the last inverse transform's padded output that the
  // compaction did not overwrite.  A Stored field carries that tail (2 n^2 values)
  // beside the padded field, so the iterations follow the reference's.
  struct Stored {
    std::unique_ptr<DevBuf> buf, tail;
  };
  size_t tail_len(int l) {
    const size_t n = lev(l).n;
    return n * n * (n + 2) - n * n * n;
  }
  void take(Stored &s, int l) {
    s.buf = ctx.pool.take(elems(l) * sizeof(T));
    s.tail = ctx.pool.take(tail_len(l) * sizeof(T));
  }
  void give(Stored &s) {
    ctx.pool.give(std::move(s.buf));
    ctx.pool.give(std::move(s.tail));
  }
  T *sb(Stored &s) { return s.buf->template as<T>(); }
  T *st(Stored &s) { return s.tail->template as<T>(); }
  void copy_stored(Stored &dst, Stored &src, int l) {
    GIC_CUDA(cudaMemcpyAsync(dst.buf->ptr, src.buf->ptr, elems(l) * sizeof(T), cudaMemcpyDeviceToDevice, ctx.stream));
    GIC_CUDA(cudaMemcpyAsync(dst.tail->ptr, src.tail->ptr, tail_len(l) * sizeof(T), cudaMemcpyDeviceToDevice,
                             ctx.stream));
  }
  void extract_tail(Stored &s, int l) {
    k_extract_tail<T><<<nblk(tail_len(l)), 256, 0, ctx.stream>>>(sb(s), st(s), lev(l).n, (T)scale(l));
    launched();
  }
  void axpy_stored(Stored &a, Stored &b, double c, int l) {
    axpy(sb(a), sb(b), c, l);
    k_axpy<T><<<nblk(tail_len(l)), 256, 0, ctx.stream>>>(st(a), st(b), (T)c, tail_len(l));
    launched();
  }
  void scale_stored(Stored &a, double c, int l) {
    scale_by(sb(a), c, l);
    k_scale<T><<<nblk(tail_len(l)), 256, 0, ctx.stream>>>(st(a), c, tail_len(l));
    launched();
  }
  // <a|b> and <c|d> over the whole buffers, read back together
  std::vector<double> dots(Stored &a, Stored &b, Stored &c, Stored &d, int l) {
    return inner_groups({{{sb(a), sb(b), l, kReal}, {st(a), st(b), l, kFlat, tail_len(l)}},
                         {{sb(c), sb(d), l, kReal}, {st(c), st(d), l, kFlat, tail_len(l)}}});
  }
  // real field -> R2C -> times tab -> C2R (Field::applyTransferFunction between transforms)
  void apply_precond(T *buf, int l, const T *tab) {
    to_fourier(buf, l);
    fft_c2r_3d<T>(ctx, buf, lev(l).n, scale(l), tab);
  }
  void zero_cells(T *buf, int l, const unsigned long long *cells, size_t count) {
    if (!count) return;
    k_zero_cells<T><<<nblk(count), 256, 0, ctx.stream>>>(buf, lev(l).n, cells, count);
    launched();
  }
  void keep_cells(T *buf, int l, const unsigned long long *cells, size_t count) {
    T *v = nullptr;
    if (count) {
      S.compact.ensure(count * sizeof(T));
      v = S.compact.template as<T>();
      k_gather_cells<T><<<nblk(count), 256, 0, ctx.stream>>>(buf, lev(l).n, cells, count, v);
      launched();
    }
    GIC_CUDA(cudaMemsetAsync(buf, 0, elems(l) * sizeof(T), ctx.stream));
    if (count) {
      k_scatter_cells<T><<<nblk(count), 256, 0, ctx.stream>>>(v, lev(l).n, cells, count, buf);
      launched();
    }
  }

  // spliceOneLevel(a = new, b = original): Fourier in (a_k, b_k), Fourier out (into out_k)
  int splice_level(int l, const T *a_k, const T *b_k, T *out_k, const unsigned long long *cells, size_t count) {
    const size_t bytes = elems(l) * sizeof(T);
    DevBuf half, minus1, mhalf;
    preconditioner_table(ctx, lev(l), 0.5, half);
    preconditioner_table(ctx, lev(l), -1.0, minus1);
    preconditioner_table(ctx, lev(l), -0.5, mhalf);
    // in the fields' precision
    DevBuf half_t, minus1_t, mhalf_t;
    const size_t nq = 3 * (size_t)(lev(l).n / 2) * (lev(l).n / 2) + 1;
    const T *h = typed_table<T>(ctx, half_t, half.template as<double>(), nq);
    const T *m1 = typed_table<T>(ctx, minus1_t, minus1.template as<double>(), nq);
    const T *mh = typed_table<T>(ctx, mhalf_t, mhalf.template as<double>(), nq);
    Stored dd, z, r, d, x, qd;
    for (Stored *s : {&dd, &z, &r, &d, &x, &qd}) take(*s, l);
    // delta_diff = C^1/2 (b - a), real
    GIC_CUDA(cudaMemcpyAsync(sb(dd), b_k, bytes, cudaMemcpyDeviceToDevice, ctx.stream));
    axpy(sb(dd), a_k, -1.0, l);
    fft_c2r_3d<T>(ctx, sb(dd), lev(l).n, scale(l), h);
    extract_tail(dd, l);
    // z = C^1/2 Mc C^-1 M delta_diff
    GIC_CUDA(cudaMemcpyAsync(sb(z), sb(dd), bytes, cudaMemcpyDeviceToDevice, ctx.stream));
    keep_cells(sb(z), l, cells, count);
    apply_precond(sb(z), l, m1);
    zero_cells(sb(z), l, cells, count);
    apply_precond(sb(z), l, h);
    extract_tail(z, l);
    // X v = C^1/2 Mc C^-1 Mc C^1/2 v
    auto X = [&](Stored &v, Stored &o) {
      GIC_CUDA(cudaMemcpyAsync(sb(o), sb(v), bytes, cudaMemcpyDeviceToDevice, ctx.stream));
      apply_precond(sb(o), l, h);
      zero_cells(sb(o), l, cells, count);
      apply_precond(sb(o), l, m1);
      zero_cells(sb(o), l, cells, count);
      apply_precond(sb(o), l, h);
      extract_tail(o, l);
    };
    // conjugateGradient(X, z), rtol 1e-6, atol 1e-12
    copy_stored(r, z, l);
    copy_stored(d, r, l);
    scale_stored(d, -1.0, l);
    GIC_CUDA(cudaMemsetAsync(sb(x), 0, bytes, ctx.stream));
    GIC_CUDA(cudaMemsetAsync(st(x), 0, tail_len(l) * sizeof(T), ctx.stream));
    const double scale_b = std::sqrt(dots(z, z, z, z, l)[0]);
    int it = 0;
    if (scale_b != 0.0) {
      const long long n3 = (long long)lev(l).ncells();
      // the reference stops at n^3 + 1 iterations; a mixed-precision solve that stops
      // improving (no new smallest residual in 100 iterations) ends early
      const long long cap = std::min<long long>(n3 + 1, 100000);
      double best = INFINITY;
      int since_best = 0;
      for (it = 0; it < cap; ++it) {
        X(d, qd);
        std::vector<double> a = dots(r, d, d, qd, l);
        const double dqd = a[1], alpha = -a[0] / dqd;
        axpy_stored(x, d, alpha, l);
        X(x, r);
        axpy_stored(r, z, -1.0, l);
        std::vector<double> b = dots(r, r, r, qd, l);
        const double norm = std::sqrt(b[0]);
        if (norm < 1e-6 * scale_b || norm < 1e-12) break;
        if (norm < best) {
          best = norm;
          since_best = 0;
        } else if (!ctx.dbl() && ++since_best >= 100) {
          break;
        }
        const double beta = b[1] / dqd;
        scale_stored(d, beta, l);
        axpy_stored(d, r, -1.0, l);
      }
    }
    // alpha = C^1/2 x; result = Mc alpha + C^1/2 b - M delta_diff, then C^-1/2
    apply_precond(sb(x), l, h);
    zero_cells(sb(x), l, cells, count);
    GIC_CUDA(cudaMemcpyAsync(sb(qd), b_k, bytes, cudaMemcpyDeviceToDevice, ctx.stream));
    fft_c2r_3d<T>(ctx, sb(qd), lev(l).n, scale(l), h);
    axpy(sb(x), sb(qd), 1.0, l);
    keep_cells(sb(dd), l, cells, count);
    axpy(sb(x), sb(dd), -1.0, l);
    fft_r2c_3d<T>(ctx, sb(x), lev(l).n, scale(l), mh);
    GIC_CUDA(cudaMemcpyAsync(out_k, sb(x), bytes, cudaMemcpyDeviceToDevice, ctx.stream));
    GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    for (Stored *s : {&dd, &z, &r, &d, &x, &qd}) give(*s);
    return it;
  }

  // covector of one modification (kind 0 overdensity, 1..3 velocity x,y,z)
  // the x planes of `box` of a level's real field set to zero (one or two ranges)
  void zero_planes(T *p, int l, const CellBox &box) {
    const int n = lev(l).n;
    const size_t plane = (size_t)n * 2 * (n / 2 + 1) * sizeof(T);
    const int x0 = box.start[0], nx = std::min(box.len[0], n);
    const int first = std::min(nx, n - x0);
    GIC_CUDA(cudaMemsetAsync(reinterpret_cast<char *>(p) + (size_t)x0 * plane, 0, (size_t)first * plane, ctx.stream));
    if (nx > first) GIC_CUDA(cudaMemsetAsync(p, 0, (size_t)(nx - first) * plane, ctx.stream));
  }

  // covector of one modification (kind 0 overdensity, 1..3 velocity x,y,z, 4 potential,
  // 5..7 angular momentum); the request keeps its device cells, box and centre
  void covector(Field &out, ModRequest &m) {
    const int kind = m.kind;
    const unsigned long long *flagged = m.cells.data();
    const size_t count = m.cells.size();
    int F = nl() - 1;
    alloc(out);
    if (!m.dcells) {
      m.dcells = std::make_shared<DevBuf>();
      m.dcells->ensure(count * sizeof(unsigned long long));
      GIC_CUDA(cudaMemcpyAsync(m.dcells->ptr, flagged, count * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                               ctx.stream));
    }
    if (!m.have_box) {
      // the flagged cells and the stencils' reach (2 cells)
      m.box = cells_box(flagged, count, lev(F).n, 2);
      m.have_box = true;
    }
    FlagLookup fl{};
    fl.n = lev(F).n;
    for (int a = 0; a < 3; ++a) {
      fl.start[a] = m.box.start[a];
      fl.len[a] = m.box.len[a];
    }
    const size_t box_cells = (size_t)fl.len[0] * fl.len[1] * fl.len[2];
    if (kind != 0 && box_cells <= (size_t)1 << 26) {
      if (!m.dmap) {
        m.dmap = std::make_shared<DevBuf>();
        m.dmap->ensure(box_cells * sizeof(int));
        GIC_CUDA(cudaMemsetAsync(m.dmap->ptr, 0xff, box_cells * sizeof(int), ctx.stream));
        k_flag_map<<<nblk(count), 256, 0, ctx.stream>>>(m.dcells->template as<unsigned long long>(), count, fl,
                                                        m.dmap->template as<int>());
        launched();
      }
      fl.map = m.dmap->template as<int>();
    }
    // a level's real covector is read inside its support only when its transform is
    // box-restricted: then only the support's x planes are zeroed
    if (fft_prunes(ctx, lev(F).n)) zero_planes(ptr(out, F), F, m.box);
    else zero(out, F);
    const unsigned long long *dcells = m.dcells->template as<unsigned long long>();
    double w = 1.0 / (double)count;
    if (kind >= GIC_MOD_LX) {
      // centre of the flagged cells, wrapped (Grid::getCentreWrapped, grid.hpp:466-494)
      const Level &Lf = lev(F);
      const double P = Lf.periodic;
      auto wrapped = [P](double v) {
        if (v > P / 2) v -= P;
        if (v < -P / 2) v += P;
        return v;
      };
      auto centroid = [&](unsigned long long id, int axis) {
        unsigned long long zz = id % Lf.n, rr = id / Lf.n, yy = rr % Lf.n, xx = rr / Lf.n;
        unsigned long long ii = axis == 0 ? xx : (axis == 1 ? yy : zz);
        return (double)ii * Lf.dx + Lf.x0[axis] + Lf.dx / 2;
      };
      if (!m.have_centre) {
        for (int ax = 0; ax < 3; ++ax) {
          double p0 = centroid(flagged[0], ax), run = 0.0;
          for (size_t i = 1; i < count; ++i) run += wrapped(centroid(flagged[i], ax) - p0);
          run /= (double)count;
          double v = run + p0;
          v = std::fmod(v, P);
          if (v < 0) v += P;
          m.centre[ax] = v;
        }
        m.have_centre = true;
      }
      const double *cen = m.centre;
      const double norm = (double)count * Lf.dx;
      k_localise_am<T><<<nblk(8 * count), 256, 0, ctx.stream>>>(ptr(out, F), Lf.n, dcells,
                                                           count, kind - GIC_MOD_LX, Lf.dx, Lf.x0[0], Lf.x0[1], Lf.x0[2],
                                                           cen[0], cen[1], cen[2], P, 1. / 12. / norm, -2. / 3. / norm,
                                                           fl);
    } else {
      const bool vel = kind >= GIC_MOD_VX && kind <= GIC_MOD_VZ;
      double a = -w / 12. / lev(F).dx, b = w * 2. / 3. / lev(F).dx;
      k_localise<T><<<nblk(vel ? 4 * count : count), 256, 0, ctx.stream>>>(ptr(out, F), lev(F).n, dcells,
                                                        count, vel ? 1 : 0, vel ? kind - GIC_MOD_VX : 0, w, a, b, fl);
    }
    launched();
    // the reference transforms the localisation covector to Fourier space and back
    // before deinterpolating; that round trip is the identity and is skipped
    out.fourier[F] = 0;
    // support of each level's real covector: the flagged cells and the stencils' reach
    // (2 cells) on the finest level, the deinterpolation block on coarser ones
    std::vector<CellBox> support(nl());
    support[F] = m.box;
    if (F > 0) {
      for (int l = F - 1; l >= 0; --l) {
        out.fourier[l] = 0;
        const bool prune = fft_prunes(ctx, lev(l).n);
        if (!prune) zero(out, l);
        support[l] = deinterpolate(ptr(out, l + 1), l + 1, ptr(out, l), l, false, &support[l + 1], prune);
      }
    }
    for (int l = 0; l < nl(); ++l) {
      // weight ratio (dx_l/dx_F)^3, the level's family filter, sqrt(P_dm) and, for
      // velocities and angular momenta, -v/k^2: one table, applied as the forward
      // transform stores its last pass
      build_sqrtp_dm(l);
      TableSpec sp{};
      sp.power = 1;
      sp.scalar = level_weight(l) / level_weight(F);
      add_filter_factors(sp, l);
      sp.sqrtp = lev(l).sqrtp_dm.template as<double>();
      const bool velocity_like = (kind >= GIC_MOD_VX && kind <= GIC_MOD_VZ) || kind >= GIC_MOD_LX;
      sp.vel = velocity_like ? velocity_ratio() : 0.0;
      table(sp, l);
      fft_r2c_3d<T>(ctx, ptr(out, l), lev(l).n, scale(l), tabT(), &support[l]);
      out.fourier[l] = 1;
      if (kind == GIC_MOD_POTENTIAL) {
        // 3/2 Om0 / a (H0/h)^2 / c^2 in (h/Mpc)^2 (cosmology/parameters.hpp:213-216)
        const double prefac = 3. / 2. * ctx.cosmo.om / ctx.cosmo.a * 100. * 100. / (299792.) / (299792.);
        k_density_to_potential<T><<<hs_grid(lev(l).n), hs_block(), 0, ctx.stream>>>(reinterpret_cast<C *>(ptr(out, l)),
                                                                                     lev(l).n, lev(l).kmin(), prefac);
        launched();
      }
    }
  }
  double velocity_ratio();
  void build_sqrtp_dm(int l);

  // transpose tricubic: fine real (level f) / r^3 added into coarse real (level c)
  // unit_scale: the plain transpose of the tricubic interpolation (no 1/r^3)
  // returns the block of coarse cells it adds into
  // fine_box: the fine field is zero outside it; the passes then run over its cells
  // only (an axis whose range wraps around the fine grid is taken whole).  Skipped
  // cells would only add zeros, so the sums are the same.
  // zero_block: first set to zero the coarse x planes the block covers (a caller that
  // reads the coarse field in the block's planes only need not zero the rest)
  CellBox deinterpolate(const T *fine, int f, T *coarse, int c, bool unit_scale = false,
                        const CellBox *fine_box = nullptr, bool zero_block = false) {
    const Level &Fl = lev(f), &Cl = lev(c);
    int nf = Fl.n;
    int r = (int)std::lround(Cl.dx / Fl.dx);
    T scale = unit_scale ? (T)1 : (T)(1.0 / ((double)r * r * r));
    // the per-axis stencil geometry of this pair of levels, computed once
    bool fresh = false;
    GeomEntry &ge = geom_entry({2.0, (double)f, (double)c, (double)nf, Fl.dx, Fl.x0[0], Fl.x0[1], Fl.x0[2], Cl.x0[0],
                                Cl.x0[1], Cl.x0[2], Cl.dx, Cl.periodic, (double)Cl.n, (double)sizeof(T)},
                               fresh);
    if (fresh) {
      ge.dev.ensure(3 * (size_t)nf * (sizeof(int) + sizeof(T)));
      int *ub0 = ge.dev.template as<int>();
      k_axes_geom<T><<<nblk(3 * nf, 128), 128, 0, ctx.stream>>>(nf, Fl.dx, Fl.x0[0], Fl.x0[1], Fl.x0[2], Cl.x0[0], Cl.x0[1],
                                                                Cl.x0[2], Cl.dx, Cl.periodic, Cl.n, ub0,
                                                                reinterpret_cast<T *>(ub0 + 3 * nf));
      launched();
      ge.host.resize(3 * nf);
      GIC_CUDA(cudaMemcpyAsync(ge.host.data(), ub0, 3 * nf * sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
      GIC_CUDA(cudaStreamSynchronize(ctx.stream));
      // per axis, the fine cells reaching each coarse index: [first, last]
      std::vector<int> rg;
      for (int a = 0; a < 3; ++a) {
        const int *ua = &ge.host[(size_t)a * nf];
        int lo = ua[0], hi = ua[0];
        for (int x = 1; x < nf; ++x) {
          lo = std::min(lo, ua[x]);
          hi = std::max(hi, ua[x]);
        }
        ge.umin[a] = lo - 1;
        ge.ncu[a] = hi + 3 - ge.umin[a];
        ge.roff[a] = (int)(rg.size() / 2);
        rg.resize(rg.size() + 2 * (size_t)ge.ncu[a]);
        int *t = &rg[2 * (size_t)ge.roff[a]];
        for (int i = 0; i < ge.ncu[a]; ++i) {
          t[2 * i] = nf;
          t[2 * i + 1] = -1;
        }
        for (int x = 0; x < nf; ++x)
          for (int k = 0; k < 4; ++k) {
            const int i = ua[x] - 1 + k - ge.umin[a];
            t[2 * i] = std::min(t[2 * i], x);
            t[2 * i + 1] = std::max(t[2 * i + 1], x);
          }
      }
      ge.aux.ensure(rg.size() * sizeof(int));
      GIC_CUDA(cudaMemcpyAsync(ge.aux.ptr, rg.data(), rg.size() * sizeof(int), cudaMemcpyHostToDevice, ctx.stream));
      GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    }
    const int2 *ranges = ge.aux.template as<int2>();
    int *ub = ge.dev.template as<int>();
    T *fr = reinterpret_cast<T *>(ub + 3 * nf);
    const std::vector<int> &h = ge.host;
    // fine ranges [f0, f0 + fn) per axis, and the coarse block they reach
    int f0[3], fn[3], c0[3], cnt[3];
    for (int a = 0; a < 3; ++a) {
      const bool cut = fine_box && fine_box->len[a] < nf && fine_box->start[a] + fine_box->len[a] <= nf;
      f0[a] = cut ? fine_box->start[a] : 0;
      fn[a] = cut ? fine_box->len[a] : nf;
      c0[a] = h[(size_t)a * nf + f0[a]] - 1;
      cnt[a] = h[(size_t)a * nf + f0[a] + fn[a] - 1] + 3 - c0[a];
    }
    const long long frs = 2 * (nf / 2 + 1);
    const T *in = fine + (long long)f0[0] * nf * frs + (long long)f0[1] * frs + f0[2];
    // pass x: fine box (fn0, fn1, fn2) -> t1 (cnt0, fn1, fn2)
    const size_t b1 = (size_t)cnt[0] * fn[1] * fn[2];
    S.t1.ensure(b1 * sizeof(T));
    k_deinterp_gather<T><<<nblk(b1), 256, 0, ctx.stream>>>(
        in, (long long)nf * frs, frs, S.t1.template as<T>(), (long long)fn[1] * fn[2], fn[2], 0, fn[0], fn[1], fn[2], fn[0],
        ub + f0[0], fr + f0[0], ranges + ge.roff[0], ge.umin[0], ge.ncu[0], f0[0], c0[0], cnt[0], scale);
    // pass y: t1 (cnt0, fn1, fn2) -> t2 (cnt0, cnt1, fn2)
    const size_t b2 = (size_t)cnt[0] * cnt[1] * fn[2];
    S.t2.ensure(b2 * sizeof(T));
    k_deinterp_gather<T><<<nblk(b2), 256, 0, ctx.stream>>>(
        S.t1.template as<T>(), (long long)fn[1] * fn[2], fn[2], S.t2.template as<T>(), (long long)cnt[1] * fn[2], fn[2], 1,
        cnt[0], fn[1], fn[2], fn[1], ub + nf + f0[1], fr + nf + f0[1], ranges + ge.roff[1], ge.umin[1], ge.ncu[1], f0[1],
        c0[1], cnt[1], (T)1);
    // pass z: t2 (cnt0, cnt1, fn2) -> t3 (cnt0, cnt1, cnt2)
    const size_t b3 = (size_t)cnt[0] * cnt[1] * cnt[2];
    S.t3.ensure(b3 * sizeof(T));
    k_deinterp_gather<T><<<nblk(b3), 256, 0, ctx.stream>>>(
        S.t2.template as<T>(), (long long)cnt[1] * fn[2], fn[2], S.t3.template as<T>(), (long long)cnt[1] * cnt[2], cnt[2], 2,
        cnt[0], cnt[1], fn[2], fn[2], ub + 2 * nf + f0[2], fr + 2 * nf + f0[2], ranges + ge.roff[2], ge.umin[2],
        ge.ncu[2], f0[2], c0[2], cnt[2], (T)1);
    CellBox b = CellBox::whole(Cl.n);
    for (int a = 0; a < 3; ++a) b.set_axis(a, c0[a], (long long)c0[a] + cnt[a], 0, Cl.n);
    if (zero_block) zero_planes(coarse, c, b);
    k_add_block<T><<<nblk(b3), 256, 0, ctx.stream>>>(S.t3.template as<T>(), cnt[0], cnt[1], cnt[2], c0[0], c0[1], c0[2],
                                                    coarse, Cl.n);
    launched(4);
    return b;
  }
};

template <typename T>
double ModEngine<T>::velocity_ratio() {
  return velocity_to_offset_ratio(ctx.cosmo);
}

template <typename T>
void ModEngine<T>::build_sqrtp_dm(int l) {
  build_sqrtp_table_species(ctx, lev(l), 1);
}

// --- the modification manager ------------------------------------------------------

// W borrows the levels' noise buffers (no copy) for the lifetime of the loan; the
// buffers return to the levels when it ends, also on an error
template <typename T>
struct NoiseLoan {
  ModEngine<T> &E;
  typename ModEngine<T>::Field &W;
  NoiseLoan(ModEngine<T> &e, typename ModEngine<T>::Field &w) : E(e), W(w) {
    W.pool = nullptr;
    W.b.resize(E.nl());
    W.fourier.assign(E.nl(), 1);
    for (int l = 0; l < E.nl(); ++l) {
      Level &L = E.lev(l);
      if (!L.have_noise || !L.noise.ptr) fail(GIC_ERR_NOT_READY, "white noise has not been drawn");
      W.b[l] = std::make_unique<DevBuf>();
      std::swap(W.b[l]->ptr, L.noise.ptr);
      std::swap(W.b[l]->bytes, L.noise.bytes);
    }
  }
  ~NoiseLoan() {
    for (int l = 0; l < (int)W.b.size(); ++l) {
      if (!W.b[l]) continue;
      Level &L = E.lev(l);
      std::swap(W.b[l]->ptr, L.noise.ptr);
      std::swap(W.b[l]->bytes, L.noise.bytes);
    }
    W.b.clear();
  }
};

template <typename T>
static void noise_field(ModEngine<T> &E, typename ModEngine<T>::Field &W) {
  E.alloc(W);
  for (int l = 0; l < E.nl(); ++l) {
    if (!E.lev(l).have_noise) fail(GIC_ERR_NOT_READY, "white noise has not been drawn");
    E.copy_level(*W.b[l], E.lev(l).noise, l);
    W.fourier[l] = 1;
  }
}

template <typename T>
static double current_value(Context &ctx, ModRequest &m) {
  ModEngine<T> E(ctx);
  typename ModEngine<T>::Field W, a;
  NoiseLoan<T> loan(E, W);
  E.covector(a, m);
  return E.inner(a, W);
}

template <typename T>
static double chi2_of_noise(Context &ctx) {
  ModEngine<T> E(ctx);
  typename ModEngine<T>::Field W;
  NoiseLoan<T> loan(E, W);
  return E.chi2(W);
}

// tools::linspace (util_functions.hpp:77-92): n + 1 points for n > 1
static std::vector<double> linspace_targets(double start, double end, int n) {
  std::vector<double> a;
  if (n == 0 || n == 1 || start == end) {
    a.push_back(end);
  } else {
    double step = (end - start) / n;
    for (int c = 0; c < n + 1; ++c) a.push_back(start + c * step);
  }
  return a;
}

// ModificationManager::performIterations (modificationmanager.hpp:249-275) with
// addToOrthonormalFamily (:318-333).  `lin` are the linear modifications'
// orthonormalised vectors and D their plain products D[m][j] = <v_m|v_j>.  The
// pushed covector of the start value is reused by the first step (the reference
// recomputes it on the unchanged field).
template <typename T>
static void perform_iterations(ModEngine<T> &E, typename ModEngine<T>::Field &X,
                               std::vector<typename ModEngine<T>::Field> &lin, const std::vector<double> &D,
                               QuadRequest &q, int n_steps) {
  using F = typename ModEngine<T>::Field;
  const int n = (int)lin.size();
  F P, CP, CP2;
  E.push_variance(X, q, P);
  const double start = E.inner(P, X);
  std::vector<double> targets = linspace_targets(start, q.target, n_steps);
  if ((int)targets.size() < n_steps + 1) fail(GIC_ERR_INVALID_ARG, "the quadratic algorithm needs at least 2 steps");
  for (int i = 0; i < n_steps; ++i) {
    if (i > 0) E.push_variance(X, q, P);
    E.apply_metric(P, CP, false);
    std::vector<F *> Bs{&X, &CP};
    for (int j = 0; j < n; ++j) Bs.push_back(&lin[j]);
    std::vector<double> ip = E.inner_block({&P}, Bs);
    const double current = ip[0], norm = std::sqrt(ip[1]);
    double scale_vec = 1.0;
    F *vec = &CP;
    if (n > 0) {
      // p <- p - r_j v_j in order, r_j = <p|v_j> with p already reduced by v_0..v_{j-1}
      std::vector<double> r(n);
      for (int j = 0; j < n; ++j) {
        r[j] = ip[2 + j];
        for (int m = 0; m < j; ++m) r[j] -= r[m] * D[(size_t)m * n + j];
      }
      std::vector<double> mr(n);
      for (int j = 0; j < n; ++j) mr[j] = -r[j];
      for (int l = 0; l < E.nl(); ++l) {
        std::vector<const T *> srcs;
        for (int j = 0; j < n; ++j) srcs.push_back(E.ptr(lin[j], l));
        E.axpy_many(E.ptr(P, l), srcs, mr, l);
      }
      E.apply_metric(P, CP2, false);
      scale_vec = 1.0 / std::sqrt(E.inner(P, CP2));
      vec = &CP2;
    } else {
      scale_vec = 1.0 / norm;
    }
    const double mult = 0.5 * (targets[i + 1] - current) / norm;
    for (int l = 0; l < E.nl(); ++l) E.axpy(E.ptr(X, l), E.ptr(*vec, l), mult * scale_vec, l);
  }
}

// applyLinQuadModif (modificationmanager.hpp:221-246) and calculateCorrectNumberSteps (:278-285)
template <typename T>
static void apply_quadratic(ModEngine<T> &E, typename ModEngine<T>::Field &W,
                            std::vector<typename ModEngine<T>::Field> &lin, QuadRequest &q) {
  using F = typename ModEngine<T>::Field;
  const int n = (int)lin.size();
  std::vector<double> D;
  if (n > 0) {
    std::vector<std::pair<F *, F *>> pairs;
    for (int m = 0; m < n; ++m)
      for (int j = 0; j < n; ++j) pairs.push_back({&lin[m], &lin[j]});
    D = E.inner_many(pairs);
  }
  int steps = q.init_steps;
  {
    F test;
    E.copy(test, W);
    perform_iterations<T>(E, test, lin, D, q, q.init_steps);
    F P;
    E.push_variance(test, q, P);
    const double achieved = std::fabs(E.inner(P, test) - q.target);
    const double wanted = q.target * q.precision;
    const int n_steps = q.init_steps * (int)std::ceil(std::sqrt(achieved / wanted));
    if (n_steps > q.init_steps) steps = n_steps;
  }
  perform_iterations<T>(E, W, lin, D, q, steps);
}

template <typename T>
static void apply_mods(Context &ctx, double *chi2_before, double *chi2_after) {
  ModEngine<T> E(ctx);
  using F = typename ModEngine<T>::Field;
  int n = (int)ctx.mods.size();
  if (chi2_before) *chi2_before = chi2_of_noise<T>(ctx);
  {
  // the modifications work on the noise buffers themselves
  F W;
  NoiseLoan<T> loan(E, W);
  std::vector<F> alpha(n), vec(n);
  std::vector<double> t(n);
  for (int i = 0; i < n; ++i) {
    E.covector(alpha[i], ctx.mods[i]);
    E.apply_metric(alpha[i], vec[i], false);
    t[i] = ctx.mods[i].target;
  }
  // <a_i|W> and the Gram matrix G_ij = <a_i|C a_j>, read back together.  G is not
  // assumed symmetric: the cross-level terms of C (interpolation up, block means
  // down) are not exact transposes of each other.
  std::vector<F *> As, Bs{&W};
  for (int i = 0; i < n; ++i) As.push_back(&alpha[i]);
  for (int j = 0; j < n; ++j) Bs.push_back(&vec[j]);
  if (ctx.quads.empty() && n <= kDevGramMax) {
    // the Gram block stays on the device; one thread forms the coefficients, and the
    // correction reads them there: no host round trip
    const double *Md = E.inner_block_dev(As, Bs);
    if (n > 0) {
      GramTargets tg{};
      tg.n = n;
      for (int i = 0; i < n; ++i) tg.t[i] = t[i];
      E.S.gram.ensure(kDevGramMax * sizeof(T));
      k_gram_coefficients<T><<<1, 1, 0, ctx.stream>>>(Md, tg, E.S.gram.template as<T>());
      launched();
      const std::vector<double> none(n, 0.0);
      for (int l = 0; l < E.nl(); ++l) {
        std::vector<const T *> srcs;
        for (int k = 0; k < n; ++k) srcs.push_back(E.ptr(vec[k], l));
        E.axpy_many(E.ptr(W, l), srcs, none, l, E.S.gram.template as<T>());
      }
    }
  } else {
  std::vector<double> M = E.inner_block(As, Bs);  // M[i][0] = <a_i|W>, M[i][1 + j] = G_ij
  std::vector<double> b(n), G((size_t)n * n);
  for (int i = 0; i < n; ++i) {
    b[i] = M[(size_t)i * (n + 1)];
    for (int j = 0; j < n; ++j) G[(size_t)i * n + j] = M[(size_t)i * (n + 1) + 1 + j];
  }
  // Gram-Schmidt in the order of modificationmanager.hpp:288-312, on coefficient
  // vectors: row i of L holds a'_i = sum_k L[i][k] a_k
  std::vector<double> L((size_t)n * n, 0.0);
  auto ip = [&](const double *x, const double *y) {
    double s = 0;
    for (int k = 0; k < n; ++k)
      for (int m = 0; m < n; ++m) s += x[k] * y[m] * G[(size_t)k * n + m];
    return s;
  };
  for (int i = 0; i < n; ++i) {
    double *li = &L[(size_t)i * n];
    li[i] = 1.0;
    for (int j = 0; j < i; ++j) {
      double *lj = &L[(size_t)j * n];
      double r = ip(li, lj);
      for (int k = 0; k < n; ++k) li[k] -= r * lj[k];
      t[i] -= r * t[j];
    }
    double nrm = std::sqrt(ip(li, li));
    for (int k = 0; k < n; ++k) li[k] /= nrm;
    t[i] /= nrm;
  }
  std::vector<double> coef(n, 0.0);
  for (int i = 0; i < n; ++i) {
    double existing = 0;
    for (int k = 0; k < n; ++k) existing += L[(size_t)i * n + k] * b[k];
    double d = t[i] - existing;
    for (int k = 0; k < n; ++k) coef[k] += d * L[(size_t)i * n + k];
  }
  for (int l = 0; l < E.nl() && n > 0; ++l) {
    std::vector<const T *> srcs;
    for (int k = 0; k < n; ++k) srcs.push_back(E.ptr(vec[k], l));
    E.axpy_many(E.ptr(W, l), srcs, coef, l);
  }
  if (!ctx.quads.empty()) {
    // applyLinearModif leaves the orthonormalised covectors converted to vectors,
    // C a'_i = sum_k L[i][k] C a_k; the quadratic steps project against those
    std::vector<F> lin(n);
    for (int i = 0; i < n; ++i) {
      E.alloc(lin[i]);
      for (int l = 0; l < E.nl(); ++l) {
        E.zero(lin[i], l);
        for (int k = 0; k < n; ++k) E.axpy(E.ptr(lin[i], l), E.ptr(vec[k], l), L[(size_t)i * n + k], l);
      }
    }
    alpha.clear();
    vec.clear();
    for (auto &q : ctx.quads) apply_quadratic<T>(E, W, lin, q);
  }
  }
  }
  for (int l = 0; l < E.nl(); ++l) E.lev(l).have_fields = E.lev(l).have_lpt2 = false;
  if (!ctx.defer_checks) GIC_CUDA(cudaStreamSynchronize(ctx.stream));
  if (chi2_after) *chi2_after = chi2_of_noise<T>(ctx);
}

template <typename T>
static double variance_value_t(Context &ctx, QuadRequest &q) {
  ModEngine<T> E(ctx);
  typename ModEngine<T>::Field W, P;
  noise_field(E, W);
  E.push_variance(W, q, P);
  return E.inner(P, W);
}

double variance_value(Context &ctx, QuadRequest &q) {
  return ctx.dbl() ? variance_value_t<double>(ctx, q) : variance_value_t<float>(ctx, q);
}

void field_from_noise(Context &ctx, int level, int what, const void *const *noise, void *out) {
  if (ctx.dbl()) ModEngine<double>(ctx).map_forward(level, what, noise, out);
  else ModEngine<float>(ctx).map_forward(level, what, noise, out);
}

void field_from_noise_adjoint(Context &ctx, int level, int what, const void *grad_out, void *const *grad_noise) {
  if (ctx.dbl()) ModEngine<double>(ctx).map_adjoint(level, what, grad_out, grad_noise);
  else ModEngine<float>(ctx).map_adjoint(level, what, grad_out, grad_noise);
}

double variance_gradient(Context &ctx, QuadRequest &q, const void *const *noise, void *const *grad, bool exact) {
  return ctx.dbl() ? ModEngine<double>(ctx).variance_grad(q, noise, grad, exact)
                   : ModEngine<float>(ctx).variance_grad(q, noise, grad, exact);
}

template <typename T>
static std::vector<int> splice_t(Context &ctx, unsigned long long new_seed,
                                 const std::vector<std::vector<unsigned long long>> &cells) {
  ModEngine<T> E(ctx);
  const int nl = E.nl();
  // the original noise, then a new real-space draw into the levels (ic.hpp:1658-1688)
  std::vector<std::unique_ptr<DevBuf>> original(nl);
  for (int l = 0; l < nl; ++l) {
    original[l] = ctx.pool.take(E.elems(l) * sizeof(T));
    GIC_CUDA(cudaMemcpyAsync(original[l]->ptr, E.lev(l).noise.ptr, E.elems(l) * sizeof(T), cudaMemcpyDeviceToDevice,
                             ctx.stream));
  }
  draw_noise_all(ctx, new_seed, GIC_SEED_REAL_SPACE);
  std::vector<int> its(nl);
  std::vector<std::unique_ptr<DevBuf>> dcells(nl);
  for (int l = 0; l < nl; ++l) {
    const size_t count = cells[l].size();
    dcells[l] = std::make_unique<DevBuf>();
    if (count) {
      dcells[l]->ensure(count * sizeof(unsigned long long));
      GIC_CUDA(cudaMemcpyAsync(dcells[l]->ptr, cells[l].data(), count * sizeof(unsigned long long),
                               cudaMemcpyHostToDevice, ctx.stream));
    }
    T *noise = E.lev(l).noise.template as<T>();
    its[l] = E.splice_level(l, noise, original[l]->template as<T>(), noise,
                            dcells[l]->template as<unsigned long long>(), count);
    E.lev(l).have_fields = E.lev(l).have_lpt2 = false;
  }
  for (auto &b : original) ctx.pool.give(std::move(b));
  return its;
}

std::vector<int> splice(Context &ctx, unsigned long long new_seed,
                        const std::vector<std::vector<unsigned long long>> &cells) {
  return ctx.dbl() ? splice_t<double>(ctx, new_seed, cells) : splice_t<float>(ctx, new_seed, cells);
}

void noise_real(Context &ctx, int level, void *out) {
  if (ctx.dbl()) ModEngine<double>(ctx).noise_to_real(level, out);
  else ModEngine<float>(ctx).noise_to_real(level, out);
}

double modification_value(Context &ctx, ModRequest &m) {
  return ctx.dbl() ? current_value<double>(ctx, m) : current_value<float>(ctx, m);
}

double noise_chi2(Context &ctx) { return ctx.dbl() ? chi2_of_noise<double>(ctx) : chi2_of_noise<float>(ctx); }

void apply_modifications(Context &ctx, double *chi2_before, double *chi2_after) {
  if (ctx.dbl())
    apply_mods<double>(ctx, chi2_before, chi2_after);
  else
    apply_mods<float>(ctx, chi2_before, chi2_after);
}

}  // namespace gic
