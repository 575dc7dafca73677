// Normalised 3-D real FFTs on the half-spectrum layout genetIC uses
// (genetIC/src/tools/numerics/fourier.hpp:479-518): an N^3 real field stored in
// place with rows padded to 2(N/2+1) reals, Fourier coefficients
// C[kx][ky][kz], kz in [0, N/2], kz fastest.
//
// Inverse (c2r): Hermitian mirroring of the kz = 0 and kz = N/2 planes
// (fourier.hpp:331-357), complex inverse transforms along x then y (strided
// passes), then a real inverse transform along each z row.  Forward (r2c): the
// reverse order.  Each pass is one HBM read + one HBM write of the array:
//  - strided pass: a CTA owns a tile of TC adjacent columns (64-byte segments)
//    times the whole transform axis, loads it into shared memory, runs
//    Stockham radix-8/4/3/2 stages (ping-pong in shared memory), and the last
//    stage writes straight back to HBM;
//  - row pass: a length-N real transform is a length-N/2 complex transform plus
//    an O(N) pre/post twiddle step; a CTA owns RPC rows.
// Twiddles are computed in long double on the host once per size and stored
// in the working precision.
#include "gic_internal.h"
#include <cuda.h>
#include <type_traits>
#include <cmath>
#include <algorithm>
#include <atomic>
#include <mutex>

namespace gic {
namespace {

template <typename T> struct Cx;
template <> struct Cx<float> { using type = float2; };
template <> struct Cx<double> { using type = double2; };

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
// complex product with its fused multiply-adds spelled out, so that every pass
// (fixed-length or runtime-length, any tile width) rounds it the same way
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  float2 r;
  r.x = fmaf(a.x, b.x, -(a.y * b.y));
  r.y = fmaf(a.x, b.y, a.y * b.x);
  return r;
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  double2 r;
  r.x = fma(a.x, b.x, -(a.y * b.y));
  r.y = fma(a.x, b.y, a.y * b.x);
  return r;
}
// multiply by s*i (s = +-1)
template <typename C> __device__ __forceinline__ C cmuli(C a, int s) {
  C r; if (s > 0) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; } return r;
}
template <typename C, typename T> __device__ __forceinline__ C cscale(C a, T s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }
template <typename C> __device__ __forceinline__ C cconj(C a) { C r; r.x = a.x; r.y = -a.y; return r; }

// w_N^m for sign -1 (forward), conjugate for sign +1; table holds exp(-2 pi i m / N)
template <typename C> __device__ __forceinline__ C twid(const C *tw, int m, int sign) {
  C w = tw[m];
  if (sign > 0) w.y = -w.y;
  return w;
}

// per-|k|^2 table value at half-spectrum cell (kx, col), col = ky (N/2 + 1) + kz, of
// an N^3 grid: the multiplier fused into the x pass (first of c2r, last of r2c).
// Tables are in the transform's precision: a float FFT reads float values, as a
// double-to-float conversion per element would occupy the FP64 pipe.
template <typename TT>
__device__ __forceinline__ TT qtab(const TT *tab, int N, int kx, long long col) {
  const int S = N / 2 + 1, H = N / 2;
  const int ky = (int)(col / S), kz = (int)(col - (long long)ky * S);
  const long long a = kx > H ? kx - N : kx, b = ky > H ? ky - N : ky;
  return tab[a * a + b * b + (long long)kz * kz];
}

// The multiplier of a fixed-length x pass: the per-|k|^2 table q, and optionally the
// same values laid out per coefficient, col[f][c] = q[|k|^2] for kx = f or N - f
// (f <= N/2) and half-spectrum column c = ky (N/2 + 1) + kz.  Along a tile's columns
// the per-coefficient values are contiguous, where the per-|k|^2 ones are a gather
// (the index steps by 2 kz + 1, a 32-byte sector per value).
template <typename TT>
struct XTab {
  const TT *q = nullptr;
  const TT *col = nullptr;
  __host__ __device__ explicit operator bool() const { return q != nullptr; }
  __device__ __forceinline__ TT at(int N, int kx, long long c) const {
    if (col) {
      const int f = kx > N / 2 ? N - kx : kx;
      return col[(size_t)f * (size_t)N * (size_t)(N / 2 + 1) + (size_t)c];
    }
    return qtab(q, N, kx, c);
  }
};

template <typename T, typename C, int R> struct Dft;
template <typename T, typename C> struct Dft<T, C, 2> {
  static __device__ __forceinline__ void run(C (&v)[2], int) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};
template <typename T, typename C> struct Dft<T, C, 4> {
  static __device__ __forceinline__ void run(C (&v)[4], int s) {
    C t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    C t2 = cadd(v[1], v[3]), t3 = cmuli(csub(v[1], v[3]), s);
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  }
};
template <typename T, typename C> struct Dft<T, C, 3> {
  static __device__ __forceinline__ void run(C (&v)[3], int s) {
    const T h = (T)0.8660254037844386467637231707529362;  // sqrt(3)/2
    C t = cadd(v[1], v[2]);
    C u = csub(v[1], v[2]);
    C m = csub(v[0], cscale(t, (T)0.5));
    C ju = cmuli(cscale(u, h), s);
    v[0] = cadd(v[0], t);
    v[1] = cadd(m, ju);
    v[2] = csub(m, ju);
  }
};
template <typename T, typename C> struct Dft<T, C, 8> {
  static __device__ __forceinline__ void run(C (&v)[8], int s) {
    C e[4] = {v[0], v[2], v[4], v[6]};
    C o[4] = {v[1], v[3], v[5], v[7]};
    Dft<T, C, 4>::run(e, s);
    Dft<T, C, 4>::run(o, s);
    const T r2 = (T)0.7071067811865475244008443621048490;
    // w8^k, w8 = exp(s i pi/4)
    C w1; w1.x = r2; w1.y = (T)s * r2;
    C w3; w3.x = -r2; w3.y = (T)s * r2;
    C o1 = cmul(o[1], w1);
    C o2 = cmuli(o[2], s);
    C o3 = cmul(o[3], w3);
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
  }
};

// Asynchronous global -> shared copies (cp.async): the whole tile is in flight
// before the first butterfly.  8-byte copies for float complex (rows of a padded
// half spectrum are only 8-byte aligned), 16-byte for double complex.
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

struct Radix {
  int n;
  int r[8];
};

Radix make_plan(int L) {
  Radix p{};
  int m = L;
  while (m % 8 == 0 && m > 8) { p.r[p.n++] = 8; m /= 8; }
  while (m > 1) {
    int r = (m % 8 == 0) ? 8 : (m % 4 == 0) ? 4 : (m % 2 == 0) ? 2 : (m % 3 == 0) ? 3 : 0;
    if (!r || p.n >= 8) fail(GIC_ERR_INVALID_ARG, "grid size must be of the form 2^a 3^b");
    p.r[p.n++] = r;
    m /= r;
  }
  return p;
}

// ---- strided pass: complex array (A, L, B), transform along L ----------------

// j % Ns, j / Ns and L / (Ns R) with shifts when Ns is a power of two (ns_log >= 0)
__device__ __forceinline__ void ns_split(int j, int Ns, int ns_log, int &jm, int &jq) {
  if (ns_log >= 0) {
    jm = j & (Ns - 1);
    jq = j >> ns_log;
  } else {
    jm = j % Ns;
    jq = j / Ns;
  }
}

template <typename T, int R, int TC>
__device__ __forceinline__ void strided_stage(const typename Cx<T>::type *src, typename Cx<T>::type *dst,
                                              typename Cx<T>::type *gout, long long B, int tcv, int L, int Ns,
                                              int ns_log, int sign, const typename Cx<T>::type *tw, T scale,
                                              const T *tab, long long b0) {
  using C = typename Cx<T>::type;
  const int LR = L / R;
  const int nb = LR * TC;
  const int span = L / (Ns * R);
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    int c = b % TC, j = b / TC;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[(j + r * LR) * TC + c];
    int jm, jq;
    ns_split(j, Ns, ns_log, jm, jq);
    int tstep = jm * span;
#pragma unroll
    for (int r = 1; r < R; ++r) v[r] = cmul(v[r], twid(tw, r * tstep, sign));
    Dft<T, C, R>::run(v, sign);
    int d = jq * Ns * R + jm;
    if (gout) {
      if (c < tcv) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          C o = cscale(v[r], scale);
          if (tab) o = cscale(o, qtab(tab, L, d + r * Ns, b0 + c));
          gout[(size_t)(d + r * Ns) * (size_t)B + c] = o;
        }
      }
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) dst[(d + r * Ns) * TC + c] = v[r];
    }
  }
}

// tab: optional per-|k|^2 multiplier of the x pass, on the inputs (sign > 0) or the
// scaled outputs (sign < 0)
template <typename T, int TC>
__global__ void __launch_bounds__(256) k_fft_strided(typename Cx<T>::type *data, int L, long long B,
                                                     Radix plan, int sign, const typename Cx<T>::type *tw,
                                                     T scale, const T *tab) {
  using C = typename Cx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  C *buf0 = reinterpret_cast<C *>(smraw);
  C *buf1 = buf0 + L * TC;
  long long b0 = (long long)blockIdx.x * TC;
  size_t a = blockIdx.y;
  C *base = data + a * (size_t)L * (size_t)B + b0;
  int tcv = (int)min((long long)TC, B - b0);
  for (int e = threadIdx.x; e < L * TC; e += blockDim.x) {
    int i = e / TC, c = e % TC;
    if (c < tcv) {
      cp_async<sizeof(C)>(buf0 + e, base + (size_t)i * (size_t)B + c);
    } else {
      C z;
      z.x = 0;
      z.y = 0;
      buf0[e] = z;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  if (sign > 0 && tab) {
    for (int e = threadIdx.x; e < L * TC; e += blockDim.x) {
      int i = e / TC, c = e % TC;
      if (c < tcv) buf0[e] = cscale(buf0[e], qtab(tab, L, i, b0 + c));
    }
    __syncthreads();
  }
  const T *otab = sign < 0 ? tab : nullptr;
  C *src = buf0, *dst = buf1;
  int Ns = 1, ns_log = 0;
  for (int s = 0; s < plan.n; ++s) {
    int R = plan.r[s];
    C *g = (s == plan.n - 1) ? base : nullptr;
    if (R == 8) strided_stage<T, 8, TC>(src, dst, g, B, tcv, L, Ns, ns_log, sign, tw, scale, otab, b0);
    else if (R == 4) strided_stage<T, 4, TC>(src, dst, g, B, tcv, L, Ns, ns_log, sign, tw, scale, otab, b0);
    else if (R == 2) strided_stage<T, 2, TC>(src, dst, g, B, tcv, L, Ns, ns_log, sign, tw, scale, otab, b0);
    else strided_stage<T, 3, TC>(src, dst, g, B, tcv, L, Ns, ns_log, sign, tw, scale, otab, b0);
    __syncthreads();
    C *t = src; src = dst; dst = t;
    Ns *= R;
    ns_log = (ns_log >= 0 && R != 3) ? ns_log + (R == 8 ? 3 : R == 4 ? 2 : 1) : -1;
  }
}

// ---- row pass: real transforms along contiguous z rows ------------------------
// smem layout: row-major [RPC][H+1]; tw is the length-N table (w_H^m = w_N^(2m)).

template <typename T, int R>
__device__ __forceinline__ void row_stage(const typename Cx<T>::type *src, typename Cx<T>::type *dst,
                                          typename Cx<T>::type *gout, int rows_valid, int H, int Ns, int ns_log,
                                          int h_log, int RPC, int sign, const typename Cx<T>::type *tw, T scale) {
  using C = typename Cx<T>::type;
  const int HR = H / R;
  const int nb = HR * RPC;
  const int S = H + 1;
  const int hr_log = h_log >= 0 ? h_log - (R == 8 ? 3 : R == 4 ? 2 : 1) : -1;
  const int span = H / (Ns * R);
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    int row, j;
    if (hr_log >= 0) {
      row = b >> hr_log;
      j = b & (HR - 1);
    } else {
      row = b / HR;
      j = b % HR;
    }
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[row * S + j + r * HR];
    int jm, jq;
    ns_split(j, Ns, ns_log, jm, jq);
    int tstep = jm * span;
#pragma unroll
    for (int r = 1; r < R; ++r) v[r] = cmul(v[r], twid(tw, 2 * r * tstep, sign));
    Dft<T, C, R>::run(v, sign);
    int d = jq * Ns * R + jm;
    if (gout) {
      if (row < rows_valid) {
#pragma unroll
        for (int r = 0; r < R; ++r) gout[(size_t)row * S + d + r * Ns] = cscale(v[r], scale);
      }
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) dst[row * S + d + r * Ns] = v[r];
    }
  }
}

template <typename T>
__device__ __forceinline__ void row_stage_any(int R, const typename Cx<T>::type *src, typename Cx<T>::type *dst,
                                              typename Cx<T>::type *gout, int rows_valid, int H, int Ns, int ns_log,
                                              int h_log, int RPC, int sign, const typename Cx<T>::type *tw, T scale) {
  if (R == 8) row_stage<T, 8>(src, dst, gout, rows_valid, H, Ns, ns_log, h_log, RPC, sign, tw, scale);
  else if (R == 4) row_stage<T, 4>(src, dst, gout, rows_valid, H, Ns, ns_log, h_log, RPC, sign, tw, scale);
  else if (R == 2) row_stage<T, 2>(src, dst, gout, rows_valid, H, Ns, ns_log, h_log, RPC, sign, tw, scale);
  else row_stage<T, 3>(src, dst, gout, rows_valid, H, Ns, ns_log, -1, RPC, sign, tw, scale);
}

__device__ __forceinline__ int ilog2_or_neg(int v) { return (v & (v - 1)) == 0 ? 31 - __clz(v) : -1; }

// c2r rows: in = N/2+1 Hermitian coefficients per row, out = N reals (in place)
template <typename T>
__global__ void __launch_bounds__(256) k_fft_rows_c2r(typename Cx<T>::type *data, long long nrows, int N, int RPC,
                                                      Radix plan, const typename Cx<T>::type *tw, T scale) {
  using C = typename Cx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int H = N / 2, S = H + 1;
  C *buf0 = reinterpret_cast<C *>(smraw);
  C *buf1 = buf0 + RPC * S;
  long long r0 = (long long)blockIdx.x * RPC;
  int rows_valid = (int)min((long long)RPC, nrows - r0);
  C *base = data + (size_t)r0 * S;
  for (int e = threadIdx.x; e < RPC * S; e += blockDim.x) {
    int row = e / S;
    if (row < rows_valid) {
      cp_async<sizeof(C)>(buf1 + e, base + e);
    } else {
      C z;
      z.x = 0;
      z.y = 0;
      buf1[e] = z;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  // Z[k] = E + i O, E = X[k] + conj(X[H-k]), O = (X[k] - conj(X[H-k])) e^{+2 pi i k/N}
  for (int e = threadIdx.x; e < RPC * H; e += blockDim.x) {
    int row = e / H, k = e % H;
    C a = buf1[row * S + k];
    C bq = buf1[row * S + H - k];
    if (k == 0) { a.y = 0; bq.y = 0; }
    C bc = cconj(bq);
    C E = cadd(a, bc);
    C O = cmul(csub(a, bc), twid(tw, k, +1));
    buf0[row * S + k] = cadd(E, cmuli(O, +1));
  }
  __syncthreads();
  C *src = buf0, *dst = buf1;
  int Ns = 1, ns_log = 0;
  const int h_log = ilog2_or_neg(H);
  for (int s = 0; s < plan.n; ++s) {
    int R = plan.r[s];
    C *g = (s == plan.n - 1) ? base : nullptr;
    row_stage_any<T>(R, src, dst, g, rows_valid, H, Ns, ns_log, h_log, RPC, +1, tw, scale);
    __syncthreads();
    C *t = src; src = dst; dst = t;
    Ns *= R;
    ns_log = (ns_log >= 0 && R != 3) ? ns_log + (R == 8 ? 3 : R == 4 ? 2 : 1) : -1;
  }
}

// r2c rows: in = N reals per row (as N/2 complex), out = N/2+1 coefficients
template <typename T>
__global__ void __launch_bounds__(256) k_fft_rows_r2c(typename Cx<T>::type *data, long long nrows, int N, int RPC,
                                                      Radix plan, const typename Cx<T>::type *tw, T scale) {
  using C = typename Cx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int H = N / 2, S = H + 1;
  C *buf0 = reinterpret_cast<C *>(smraw);
  C *buf1 = buf0 + RPC * S;
  long long r0 = (long long)blockIdx.x * RPC;
  int rows_valid = (int)min((long long)RPC, nrows - r0);
  C *base = data + (size_t)r0 * S;
  for (int e = threadIdx.x; e < RPC * H; e += blockDim.x) {
    int row = e / H, m = e % H;
    if (row < rows_valid) {
      cp_async<sizeof(C)>(buf0 + row * S + m, base + (size_t)row * S + m);
    } else {
      C z;
      z.x = 0;
      z.y = 0;
      buf0[row * S + m] = z;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  C *src = buf0, *dst = buf1;
  int Ns = 1, ns_log = 0;
  const int h_log = ilog2_or_neg(H);
  for (int s = 0; s < plan.n; ++s) {
    int R = plan.r[s];
    row_stage_any<T>(R, src, dst, nullptr, rows_valid, H, Ns, ns_log, h_log, RPC, -1, tw, (T)1);
    __syncthreads();
    C *t = src; src = dst; dst = t;
    Ns *= R;
    ns_log = (ns_log >= 0 && R != 3) ? ns_log + (R == 8 ? 3 : R == 4 ? 2 : 1) : -1;
  }
  // src holds Z; X[k] = (Z[k] + conj Z[H-k])/2 - i/2 e^{-2 pi i k/N} (Z[k] - conj Z[H-k])
  for (int e = threadIdx.x; e < RPC * S; e += blockDim.x) {
    int row = e / S, k = e % S;
    if (row >= rows_valid) continue;
    C zk = src[row * S + (k % H)];
    C zc = cconj(src[row * S + ((H - k) % H)]);
    C ev = cscale(cadd(zk, zc), (T)0.5);
    C od = cscale(csub(zk, zc), (T)0.5);
    C t = cmul(od, twid(tw, k, -1));
    C X = cadd(ev, cmuli(t, -1));
    base[(size_t)row * S + k] = cscale(X, scale);
  }
}

// Hermitian mirroring of the kz = 0 and kz = N/2 planes: negative-kx half (and
// negative ky on the kx = 0, N/2 rows) take the conjugate of their partner.
template <typename T>
__global__ void k_mirror(typename Cx<T>::type *data, int N) {
  using C = typename Cx<T>::type;
  const int H = N / 2, S = H + 1;
  long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per_plane = (long long)N * N;
  if (id >= 2 * per_plane) return;
  int plane = (int)(id / per_plane);
  int kz = plane ? H : 0;
  long long rem = id % per_plane;
  int kx = (int)(rem / N), ky = (int)(rem % N);
  int sx, sy;
  if (kx > H) {
    sx = N - kx;
    sy = (N - ky) % N;
  } else if ((kx == 0 || kx == H) && ky > H) {
    sx = kx;
    sy = N - ky;
  } else {
    return;
  }
  data[((size_t)kx * N + ky) * S + kz] = cconj(data[((size_t)sx * N + sy) * S + kz]);
}

// The same mirroring out of place: the kz = 0 and kz = N/2 planes of src, mirrored,
// into dst (the first pass of an out-of-place inverse reads those two planes from dst
// and every other column from src)
template <typename T>
__global__ void k_mirror_from(typename Cx<T>::type *dst, const typename Cx<T>::type *src, int N) {
  const int H = N / 2, S = H + 1;
  long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long per_plane = (long long)N * N;
  if (id >= 2 * per_plane) return;
  int plane = (int)(id / per_plane);
  int kz = plane ? H : 0;
  long long rem = id % per_plane;
  int kx = (int)(rem / N), ky = (int)(rem % N);
  const size_t at = ((size_t)kx * N + ky) * S + kz;
  if (kx > H) dst[at] = cconj(src[((size_t)(N - kx) * N + (N - ky) % N) * S + kz]);
  else if ((kx == 0 || kx == H) && ky > H) dst[at] = cconj(src[((size_t)kx * N + (N - ky)) * S + kz]);
  else dst[at] = src[at];
}

// ---- fixed-length passes (power-of-two lengths): one padded tile, in place ----
// A CTA owns TC transforms of compile-time length L held as a tile [L][TC + 1] in
// shared memory (column c of the tile is one transform; the +1 pad makes row
// strides odd in 8-byte words).  Each Stockham stage reads every butterfly's
// inputs into registers, synchronises, and writes its outputs back in place, so
// one buffer suffices.  Butterflies are numbered with the column fastest:
// neighbouring threads touch neighbouring words of a tile row, free of bank
// conflicts.  The radix schedule (8, then 4 or 2 for the remainder) and every
// index are compile-time constants.

template <typename T, int L, int TC, int TCP, int NT, int R, int NS, int SIGN, int TWM>
__device__ __forceinline__ void tile_stage(typename Cx<T>::type *tile, const typename Cx<T>::type *tw) {
  using C = typename Cx<T>::type;
  constexpr int LR = L / R, NB = LR * TC, PER = (NB + NT - 1) / NT;
  C v[PER][R];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int b = threadIdx.x + p * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % TC, j = b / TC;
#pragma unroll
      for (int r = 0; r < R; ++r) v[p][r] = tile[(j + r * LR) * TCP + c];
    }
  }
  __syncthreads();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int b = threadIdx.x + p * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % TC, j = b / TC;
      const int jm = j % NS, jq = j / NS;
      if (NS > 1) {
#pragma unroll
        for (int r = 1; r < R; ++r) v[p][r] = cmul(v[p][r], twid(tw, TWM * r * jm * (L / (NS * R)), SIGN));
      }
      Dft<T, C, R>::run(v[p], SIGN);
      const int d = jq * NS * R + jm;
#pragma unroll
      for (int r = 0; r < R; ++r) tile[(d + r * NS) * TCP + c] = v[p][r];
    }
  }
  __syncthreads();
}

template <typename T, int L, int TC, int TCP, int NT, int NS, int SIGN, int TWM, bool DONE = (NS >= L)>
struct TileStages {
  static __device__ __forceinline__ void run(typename Cx<T>::type *tile, const typename Cx<T>::type *tw) {
    constexpr int R = (L / NS) >= 8 ? 8 : (L / NS);
    tile_stage<T, L, TC, TCP, NT, R, NS, SIGN, TWM>(tile, tw);
    TileStages<T, L, TC, TCP, NT, NS * R, SIGN, TWM>::run(tile, tw);
  }
};
template <typename T, int L, int TC, int TCP, int NT, int NS, int SIGN, int TWM>
struct TileStages<T, L, TC, TCP, NT, NS, SIGN, TWM, true> {
  static __device__ __forceinline__ void run(typename Cx<T>::type *, const typename Cx<T>::type *) {}
};

// strided pass over (A, L, B) complex, transform along L; grid (ceil(B / TC), na):
// planes (a0 + blockIdx.y) mod A, na <= A of them
// tab: optional per-|k|^2 multiplier (x pass only, B = L (L/2 + 1)): applied to
// the inputs when SIGN > 0 (c2r) and to the scaled outputs when SIGN < 0 (r2c)
template <typename T, int L, int TC, int NT, int SIGN>
__global__ void __launch_bounds__(NT) k_fft_cols(typename Cx<T>::type *data, long long B,
                                                 const typename Cx<T>::type *tw, T scale, XTab<T> tab, int a0,
                                                 int A, int m0, int mn, const typename Cx<T>::type *src,
                                                 typename Cx<T>::type *dst, const typename Cx<T>::type *xsrc,
                                                 XTab<T> xtab) {
  using C = typename Cx<T>::type;
  constexpr int TCP = TC + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C *tile = reinterpret_cast<C *>(smraw);
  const long long b0 = (long long)blockIdx.x * TC;
  C *base = data + (size_t)((a0 + (int)blockIdx.y) % A) * (size_t)L * (size_t)B + b0;
  const int tcv = (int)min((long long)TC, B - b0);
  // the window limits the loads of a forward pass and the stores of an inverse one
  const int lm0 = SIGN < 0 ? m0 : 0, lmn = SIGN < 0 ? mn : L, sm0 = SIGN > 0 ? m0 : 0, smn = SIGN > 0 ? mn : L;
  for (int e = threadIdx.x; e < L * TC; e += NT) {
    const int i = e / TC, c = e % TC;
    if (c < tcv && (i - lm0 + L) % L < lmn) {
      // out-of-place x pass: columns other than kz = 0 and kz = L/2 come from src
      const int kz = (int)((b0 + c) % (L / 2 + 1));
      const C *from = (src && kz != 0 && kz != L / 2) ? src + (base - data) : base;
      cp_async<sizeof(C)>(tile + i * TCP + c, from + (size_t)i * (size_t)B + c);
    } else {
      C z;
      z.x = 0;
      z.y = 0;
      tile[i * TCP + c] = z;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  if (SIGN > 0 && tab) {
    for (int e = threadIdx.x; e < L * tcv; e += NT) {
      const int i = e / tcv, c = e % tcv;
      tile[i * TCP + c] = cscale(tile[i * TCP + c], tab.at(L, i, b0 + c));
    }
    __syncthreads();
  }
  TileStages<T, L, TC, TCP, NT, 1, SIGN, 1>::run(tile, tw);
  for (int e = threadIdx.x; e < L * TC; e += NT) {
    const int i = e / TC, c = e % TC;
    if (c < tcv && (i - sm0 + L) % L < smn) {
      C v = cscale(tile[i * TCP + c], scale);
      if (SIGN < 0 && tab) v = cscale(v, tab.at(L, i, b0 + c));
      const size_t at = (size_t)i * (size_t)B + c;
      if (dst) {
        const size_t off = (size_t)(base - data);
        dst[off + at] = cadd(cscale(xsrc[off + at], xtab.at(L, i, b0 + c)), v);
      } else {
        base[at] = v;
      }
    }
  }
}

// First row of the row tile a CTA of a fixed-length row pass owns: grid (tiles, planes),
// plane (x0 + blockIdx.y) mod N, tile (ty0 + blockIdx.x) mod (N / RPC) of RPC rows.
// The whole transform is x0 = ty0 = 0 on an (N / RPC, N) grid; a box of rows is a
// cyclic range of planes times a cyclic range of tiles.
template <int N, int RPC>
__device__ __forceinline__ long long row_tile_start(int x0, int ty0) {
  const int plane = (x0 + (int)blockIdx.y) % N, tile = (ty0 + (int)blockIdx.x) % (N / RPC);
  return (long long)plane * N + (long long)tile * RPC;
}

// ---- fused passes: the first stage reads HBM into registers, the last writes HBM ----
// Shared memory then carries only the exchanges between stages (4 accesses per
// element at L = 512 instead of 8).  The tile is unpadded: every access is
// column-fastest.  Inputs and outputs are described by small functors.

__host__ __device__ constexpr int next_radix(int L, int NS) { return (L / NS) >= 8 ? 8 : L / NS; }
__host__ __device__ constexpr int last_stage_ns(int L) {
  int ns = 1;
  while (ns * next_radix(L, ns) < L) ns *= next_radix(L, ns);
  return ns;
}

// stages with NS in [NS, STOP), shared memory to shared memory
template <typename T, int L, int TC, int TCP, int NT, int NS, int STOP, int SIGN, int TWM, bool DONE = (NS >= STOP)>
struct TileStagesUntil {
  static __device__ __forceinline__ void run(typename Cx<T>::type *tile, const typename Cx<T>::type *tw) {
    constexpr int R = next_radix(L, NS);
    tile_stage<T, L, TC, TCP, NT, R, NS, SIGN, TWM>(tile, tw);
    TileStagesUntil<T, L, TC, TCP, NT, NS * R, STOP, SIGN, TWM>::run(tile, tw);
  }
};
template <typename T, int L, int TC, int TCP, int NT, int NS, int STOP, int SIGN, int TWM>
struct TileStagesUntil<T, L, TC, TCP, NT, NS, STOP, SIGN, TWM, true> {
  static __device__ __forceinline__ void run(typename Cx<T>::type *, const typename Cx<T>::type *) {}
};

// no multiplier between a first stage's loads and its butterflies
struct NoMid {
  static constexpr bool kActive = false;
  __device__ __forceinline__ void wait() const {}
  template <typename C>
  __device__ __forceinline__ C operator()(int, int, C v) const {
    return v;
  }
};

// first stage (NS = 1, no twiddles): inputs from `in(c, position)`, outputs to the tile.
// With an active `mid`, every thread's loads are issued first, then mid.wait() (a block
// barrier: all threads reach it), then each input becomes mid(c, position, value).
template <typename T, int L, int TC, int NT, int SIGN, class In, class Mid = NoMid>
__device__ __forceinline__ void first_stage_from(typename Cx<T>::type *tile, const In &in, const Mid &mid = Mid{}) {
  using C = typename Cx<T>::type;
  constexpr int R = next_radix(L, 1), LR = L / R, NB = LR * TC, PER = (NB + NT - 1) / NT;
  C v[PER][R];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int b = threadIdx.x + p * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % TC, j = b / TC;
#pragma unroll
      for (int r = 0; r < R; ++r) v[p][r] = in(c, j + r * LR);
    }
  }
  if constexpr (Mid::kActive) {
    mid.wait();
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int b = threadIdx.x + p * NT;
      if (NB % NT == 0 || b < NB) {
        const int c = b % TC, j = b / TC;
#pragma unroll
        for (int r = 0; r < R; ++r) v[p][r] = mid(c, j + r * LR, v[p][r]);
      }
    }
  }
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int b = threadIdx.x + p * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % TC, j = b / TC;
      Dft<T, C, R>::run(v[p], SIGN);
#pragma unroll
      for (int r = 0; r < R; ++r) tile[(j * R + r) * TC + c] = v[p][r];
    }
  }
  __syncthreads();
}

// An output functor with `kPrefetch` reads a value per output (`prefetch(c, position)`)
// that `put(c, position, value, prefetched)` combines with the result: the last stage
// issues those loads before its butterflies, so no store waits on a load behind it.
template <class O, class = void>
struct HasPrefetch {
  static constexpr bool value = false;
};
template <class O>
struct HasPrefetch<O, std::void_t<decltype(O::kPrefetch)>> {
  static constexpr bool value = O::kPrefetch;
};

// last stage: inputs from the tile, outputs to `out(c, position, value)`
template <typename T, int L, int TC, int NT, int SIGN, int TWM, class Out>
__device__ __forceinline__ void last_stage_to(const typename Cx<T>::type *tile, const typename Cx<T>::type *tw,
                                              const Out &out) {
  using C = typename Cx<T>::type;
  constexpr int NS = last_stage_ns(L), R = L / NS, LR = L / R, NB = LR * TC, PER = (NB + NT - 1) / NT;
  C v[PER][R];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int b = threadIdx.x + p * NT;
    if (NB % NT == 0 || b < NB) {
      const int c = b % TC, j = b / TC;
      if constexpr (HasPrefetch<Out>::value) {
        C x[R];
#pragma unroll
        for (int r = 0; r < R; ++r) x[r] = out.prefetch(c, j + r * NS);
#pragma unroll
        for (int r = 0; r < R; ++r) v[p][r] = tile[(j + r * LR) * TC + c];
#pragma unroll
        for (int r = 1; r < R; ++r) v[p][r] = cmul(v[p][r], twid(tw, TWM * r * j * (L / (NS * R)), SIGN));
        Dft<T, C, R>::run(v[p], SIGN);
#pragma unroll
        for (int r = 0; r < R; ++r) out.put(c, j + r * NS, v[p][r], x[r]);
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) v[p][r] = tile[(j + r * LR) * TC + c];
#pragma unroll
        for (int r = 1; r < R; ++r) v[p][r] = cmul(v[p][r], twid(tw, TWM * r * j * (L / (NS * R)), SIGN));
        Dft<T, C, R>::run(v[p], SIGN);
#pragma unroll
        for (int r = 0; r < R; ++r) out(c, j + r * NS, v[p][r]);
      }
    }
  }
}

template <typename C>
__device__ __forceinline__ C czero() {
  C z;
  z.x = 0;
  z.y = 0;
  return z;
}

// CG: load through L2 only (ld.global.cg), for data that other CTAs of the same
// launch wrote
// m0, mn: the positions (m0 + i) mod L, i < mn, along the transform that are read
// (others are zero: forward passes) or written (others are not wanted: inverse
// passes); mn = L for all
template <typename C, bool CG = false>
struct ColsIn {
  const C *base;
  long long B;
  int tcv;
  XTab<decltype(C::x)> tab;  // optional multiplier (x pass of an L^3 grid), field precision
  int L;
  long long b0;
  int m0 = 0, mn = 1 << 30;
  // out-of-place x pass: columns other than kz = 0 and kz = L/2 come from alt (same layout)
  const C *alt = nullptr;
  __device__ __forceinline__ C operator()(int c, int m) const {
    if (c >= tcv || (m - m0 + L) % L >= mn) return czero<C>();
    const C *from = base;
    if (alt) {
      const int kz = (int)((b0 + c) % (L / 2 + 1));
      if (kz != 0 && kz != L / 2) from = alt;
    }
    const C *p = from + (size_t)m * (size_t)B + c;
    C v = CG ? __ldcg(p) : *p;
    return tab ? cscale(v, tab.at(L, m, b0 + c)) : v;
  }
};
// PF: the epilogue's source values are prefetched by the last stage (kPrefetch)
template <typename C, typename T, bool PF = false>
struct ColsOut {
  C *base;
  long long B;
  int tcv;
  T scale;
  XTab<T> tab;
  int L;
  long long b0;
  int m0 = 0, mn = 1 << 30;
  // forward x pass with an epilogue: the output goes to obase (same layout) as
  // xtab[q] * xsrc + result
  C *obase = nullptr;
  const C *xsrc = nullptr;
  XTab<T> xtab = {};
  // the multipliers staged in shared memory ([L/2 + 1][tcs] by folded kx), where they are
  const T *stab = nullptr, *sxtab = nullptr;
  int tcs = 0;
  static constexpr bool kPrefetch = PF;
  // the epilogue's source value at (c, m) (zero without an epilogue)
  __device__ __forceinline__ C prefetch(int c, int m) const {
    if (!obase || c >= tcv || (m - m0 + L) % L >= mn) return czero<C>();
    return xsrc[(size_t)m * (size_t)B + c];
  }
  __device__ __forceinline__ void put(int c, int m, C v, C x) const {
    if (c >= tcv || (m - m0 + L) % L >= mn) return;
    v = cscale(v, scale);
    const int f = m > L / 2 ? L - m : m;
    if (stab) v = cscale(v, stab[f * tcs + c]);
    else if (tab) v = cscale(v, tab.at(L, m, b0 + c));
    const size_t at = (size_t)m * (size_t)B + c;
    if (obase) {
      obase[at] = cadd(cscale(x, sxtab ? sxtab[f * tcs + c] : xtab.at(L, m, b0 + c)), v);
      return;
    }
    base[at] = v;
  }
  __device__ __forceinline__ void operator()(int c, int m, C v) const { put(c, m, v, prefetch(c, m)); }
};

// The x pass's multipliers for a tile of TC columns from b0, in per-coefficient layout
// (XTab::col), copied to shared memory dst[f][TC], f <= L/2, by 16-byte cp.async.  The
// caller waits (cp_async_wait_all, then a block barrier) before reading them.
template <typename T, int L, int TC, int NT>
__device__ __forceinline__ void stage_col_rows(T *dst, const T *col, long long b0) {
  constexpr int VEC = 16 / (int)sizeof(T), ROWV = TC / VEC, HP = L / 2 + 1;
  static_assert(TC % VEC == 0, "a tile row of multipliers is whole 16-byte chunks");
  for (int e = threadIdx.x; e < HP * ROWV; e += NT) {
    const int f = e / ROWV, k = e - f * ROWV;
    cp_async<16>(dst + f * TC + k * VEC, col + (size_t)f * (size_t)L * HP + (size_t)b0 + (size_t)(k * VEC));
  }
}

// first-stage multiplier of an inverse x pass from the staged values (none: stab null,
// the same for the whole block)
template <typename T, int TC>
struct StagedMid {
  static constexpr bool kActive = true;
  const T *stab;
  int L;
  __device__ __forceinline__ void wait() const {
    if (stab) {
      cp_async_wait_all();
      __syncthreads();
    }
  }
  template <typename C>
  __device__ __forceinline__ C operator()(int c, int m, C v) const {
    return stab ? cscale(v, stab[(m > L / 2 ? L - m : m) * TC + c]) : v;
  }
};
// c2r packing on the fly: Z[m] = (X[m] + conj X[H-m]) + i (X[m] - conj X[H-m]) e^{+2 pi i m / N}
template <typename C>
struct RowsC2RIn {
  const C *base;
  const C *tw;
  int S, H, rows_valid;
  __device__ __forceinline__ C operator()(int c, int m) const {
    if (c >= rows_valid) return czero<C>();
    C a = base[(size_t)c * S + m], bq = base[(size_t)c * S + (H - m)];
    if (m == 0) {
      a.y = 0;
      bq.y = 0;
    }
    C bc = cconj(bq);
    return cadd(cadd(a, bc), cmuli(cmul(csub(a, bc), twid(tw, m, +1)), +1));
  }
};
template <typename C, typename T>
struct RowsOut {
  C *base;
  int S, rows_valid;
  T scale;
  __device__ __forceinline__ void operator()(int c, int m, C v) const {
    if (c < rows_valid) base[(size_t)c * S + m] = cscale(v, scale);
  }
};
template <typename C>
struct RowsIn {
  const C *base;
  int S, rows_valid;
  __device__ __forceinline__ C operator()(int c, int m) const {
    return c < rows_valid ? base[(size_t)c * S + m] : czero<C>();
  }
};

// MINB: CTAs per SM the registers are capped for (1024 / NT: 64 registers).  EXT: the
// out-of-place source, position windows and epilogue are compiled in (a plain pass
// without them keeps fewer registers)
template <typename T, int L, int TC, int NT, int SIGN, int MINB = 1024 / NT, bool EXT = true>
__global__ void __launch_bounds__(NT, MINB) k_fft_cols_fused(typename Cx<T>::type *data, long long B,
                                                       const typename Cx<T>::type *tw, T scale, XTab<T> tab,
                                                       int a0, int A, int m0, int mn,
                                                       const typename Cx<T>::type *src, typename Cx<T>::type *dst,
                                                       const typename Cx<T>::type *xsrc, XTab<T> xtab, bool stage) {
  using C = typename Cx<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  C *tile = reinterpret_cast<C *>(smraw);
  const long long b0 = (long long)blockIdx.x * TC;
  C *base = data + (size_t)((a0 + (int)blockIdx.y) % A) * (size_t)L * (size_t)B + b0;
  const int tcv = (int)min((long long)TC, B - b0);
  // the window limits the loads of a forward pass and the stores of an inverse one
  const int lm0 = EXT && SIGN < 0 ? m0 : 0, lmn = EXT && SIGN < 0 ? mn : (1 << 30);
  const int sm0 = EXT && SIGN > 0 ? m0 : 0, smn = EXT && SIGN > 0 ? mn : (1 << 30);
  const C *alt = EXT && src ? src + (base - data) : nullptr;
  // stage: the multipliers of this tile (per-coefficient layout) go to shared memory after
  // the tile, by cp.async issued before the tile's loads, so no load waits on a table value
  T *stab = nullptr, *sxtab = nullptr;
  if (stage && tcv == TC) {
    T *area = reinterpret_cast<T *>(tile + L * TC);
    if (tab.col) {
      stab = area;
      stage_col_rows<T, L, TC, NT>(stab, tab.col, b0);
      area += (L / 2 + 1) * TC;
    }
    if (EXT && SIGN < 0 && dst && xtab.col) {
      sxtab = area;
      stage_col_rows<T, L, TC, NT>(sxtab, xtab.col, b0);
    }
  }
  const XTab<T> in_tab = SIGN > 0 && !stab ? tab : XTab<T>{};
  if constexpr (SIGN > 0)
    first_stage_from<T, L, TC, NT, SIGN>(tile, ColsIn<C>{base, B, tcv, in_tab, L, b0, lm0, lmn, alt},
                                         StagedMid<T, TC>{stab, L});
  else
    first_stage_from<T, L, TC, NT, SIGN>(tile, ColsIn<C>{base, B, tcv, in_tab, L, b0, lm0, lmn, alt});
  constexpr int R0 = next_radix(L, 1), NSL = last_stage_ns(L);
  TileStagesUntil<T, L, TC, TC, NT, R0, NSL, SIGN, 1>::run(tile, tw);
  if (SIGN < 0 && (stab || sxtab)) {  // the same for the whole block
    cp_async_wait_all();
    __syncthreads();
  }
  const size_t off = (size_t)(base - data);
  if (EXT && SIGN < 0 && dst)
    last_stage_to<T, L, TC, NT, SIGN, 1>(tile, tw,
                                         ColsOut<C, T, true>{base, B, tcv, scale, tab, L, b0, sm0, smn, dst + off,
                                                             xsrc + off, xtab, stab, sxtab, TC});
  else
    last_stage_to<T, L, TC, NT, SIGN, 1>(tile, tw,
                                         ColsOut<C, T>{base, B, tcv, scale, SIGN < 0 ? tab : XTab<T>{}, L, b0, sm0, smn,
                                                       nullptr, nullptr, {}, SIGN < 0 ? stab : nullptr, nullptr, TC});
}

template <typename T, int H, int RPC, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_fft_rows_c2r_fused(typename Cx<T>::type *data, int x0, int ty0,
                                                           const typename Cx<T>::type *tw, T scale) {
  using C = typename Cx<T>::type;
  constexpr int S = H + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C *tile = reinterpret_cast<C *>(smraw);
  const long long r0 = row_tile_start<2 * H, RPC>(x0, ty0);
  const int rows_valid = RPC;
  C *base = data + (size_t)r0 * S;
  first_stage_from<T, H, RPC, NT, +1>(tile, RowsC2RIn<C>{base, tw, S, H, rows_valid});
  constexpr int R0 = next_radix(H, 1), NSL = last_stage_ns(H);
  TileStagesUntil<T, H, RPC, RPC, NT, R0, NSL, +1, 2>::run(tile, tw);
  last_stage_to<T, H, RPC, NT, +1, 2>(tile, tw, RowsOut<C, T>{base, S, rows_valid, scale});
}

template <typename T, int H, int RPC, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) k_fft_rows_r2c_fused(typename Cx<T>::type *data, int x0, int ty0,
                                                           const typename Cx<T>::type *tw, T scale) {
  using C = typename Cx<T>::type;
  constexpr int S = H + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C *tile = reinterpret_cast<C *>(smraw);  // [H + 1][RPC]
  const long long r0 = row_tile_start<2 * H, RPC>(x0, ty0);
  const int rows_valid = RPC;
  C *base = data + (size_t)r0 * S;
  first_stage_from<T, H, RPC, NT, -1>(tile, RowsIn<C>{base, S, rows_valid});
  constexpr int R0 = next_radix(H, 1);
  TileStagesUntil<T, H, RPC, RPC, NT, R0, H, -1, 2>::run(tile, tw);
  // X[k] and X[H-k] from Z[k] and Z[H-k] (Z[H] = Z[0]), in place
  for (int e = threadIdx.x; e < RPC * (H / 2 + 1); e += NT) {
    const int row = e % RPC, k = e / RPC;
    C zk = tile[k * RPC + row];
    C zh = tile[(k == 0 ? 0 : H - k) * RPC + row];
    C zhc = cconj(zh), zkc = cconj(zk);
    C xk = cadd(cscale(cadd(zk, zhc), (T)0.5), cmuli(cmul(cscale(csub(zk, zhc), (T)0.5), twid(tw, k, -1)), -1));
    C xh = cadd(cscale(cadd(zh, zkc), (T)0.5), cmuli(cmul(cscale(csub(zh, zkc), (T)0.5), twid(tw, H - k, -1)), -1));
    if (2 * k != H) tile[(H - k) * RPC + row] = xh;
    tile[k * RPC + row] = xk;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < RPC * S; e += NT) {
    const int row = e % RPC, m = e / RPC;
    if (row < rows_valid) base[(size_t)row * S + m] = cscale(tile[m * RPC + row], scale);
  }
}

// CG: the rows are loaded through L2 only (data other CTAs of the same launch
// wrote), else with asynchronous copies
template <typename T, int H, int RPC, int NT, bool CG>
__device__ __forceinline__ void rows_c2r_tile(typename Cx<T>::type *tile, typename Cx<T>::type *base, int rows_valid,
                                              const typename Cx<T>::type *tw, T scale) {
  using C = typename Cx<T>::type;
  constexpr int S = H + 1, TCP = RPC + 1;
  for (int e = threadIdx.x; e < RPC * S; e += NT) {
    const int row = e / S, m = e % S;
    if (row < rows_valid) {
      if (CG) tile[m * TCP + row] = __ldcg(base + e);
      else cp_async<sizeof(C)>(tile + m * TCP + row, base + e);
    } else {
      tile[m * TCP + row] = czero<C>();
    }
  }
  if (!CG) cp_async_wait_all();
  __syncthreads();
  // Z[k] = E + i O, E = X[k] + conj X[H-k], O = (X[k] - conj X[H-k]) e^{+2 pi i k / N};
  // Z[k] and Z[H-k] both come from X[k] and X[H-k], so pairs are done in place
  for (int e = threadIdx.x; e < RPC * (H / 2 + 1); e += NT) {
    const int row = e % RPC, k = e / RPC;
    C a = tile[k * TCP + row], bq = tile[(H - k) * TCP + row];
    if (k == 0) {
      a.y = 0;
      bq.y = 0;
    }
    C bc = cconj(bq);
    C zk = cadd(cadd(a, bc), cmuli(cmul(csub(a, bc), twid(tw, k, +1)), +1));
    if (k != 0 && 2 * k != H) {
      C ac = cconj(a);
      C zh = cadd(cadd(bq, ac), cmuli(cmul(csub(bq, ac), twid(tw, H - k, +1)), +1));
      tile[(H - k) * TCP + row] = zh;
    }
    tile[k * TCP + row] = zk;
  }
  __syncthreads();
  TileStages<T, H, RPC, TCP, NT, 1, +1, 2>::run(tile, tw);
  for (int e = threadIdx.x; e < RPC * H; e += NT) {
    const int row = e / H, m = e % H;
    if (row < rows_valid) base[(size_t)row * S + m] = cscale(tile[m * TCP + row], scale);
  }
}

// c2r rows of N = 2H reals: rows of H + 1 Hermitian coefficients are copied
// (coalesced) into a tile [H + 1][RPC + 1] with one row per tile column, packed
// into H complex values, transformed, and copied back as N reals per row.
template <typename T, int H, int RPC, int NT>
__global__ void __launch_bounds__(NT) k_fft_rows_c2r_fixed(typename Cx<T>::type *data, int x0, int ty0,
                                                           const typename Cx<T>::type *tw, T scale) {
  using C = typename Cx<T>::type;
  constexpr int S = H + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C *tile = reinterpret_cast<C *>(smraw);
  const long long r0 = row_tile_start<2 * H, RPC>(x0, ty0);
  const int rows_valid = RPC;
  rows_c2r_tile<T, H, RPC, NT, false>(tile, data + (size_t)r0 * S, rows_valid, tw, scale);
}

// r2c rows: N reals per row (read as H complex) -> H + 1 coefficients
template <typename T, int H, int RPC, int NT, bool CG>
__device__ __forceinline__ void rows_r2c_tile(typename Cx<T>::type *tile, typename Cx<T>::type *base, int rows_valid,
                                              const typename Cx<T>::type *tw, T scale) {
  using C = typename Cx<T>::type;
  constexpr int S = H + 1, TCP = RPC + 1;
  for (int e = threadIdx.x; e < RPC * H; e += NT) {
    const int row = e / H, m = e % H;
    if (row < rows_valid) {
      if (CG) tile[m * TCP + row] = __ldcg(base + (size_t)row * S + m);
      else cp_async<sizeof(C)>(tile + m * TCP + row, base + (size_t)row * S + m);
    } else {
      tile[m * TCP + row] = czero<C>();
    }
  }
  if (!CG) cp_async_wait_all();
  __syncthreads();
  TileStages<T, H, RPC, TCP, NT, 1, -1, 2>::run(tile, tw);
  // X[k] = (Z[k] + conj Z[H-k]) / 2 - i/2 e^{-2 pi i k / N} (Z[k] - conj Z[H-k]), k in [0, H]
  // (Z[H] = Z[0]); X[k] and X[H-k] both come from Z[k] and Z[H-k]
  for (int e = threadIdx.x; e < RPC * (H / 2 + 1); e += NT) {
    const int row = e % RPC, k = e / RPC;
    C zk = tile[(k == 0 ? 0 : k) * TCP + row];
    C zh = tile[(k == 0 ? 0 : H - k) * TCP + row];
    C zhc = cconj(zh), zkc = cconj(zk);
    C xk = cadd(cscale(cadd(zk, zhc), (T)0.5), cmuli(cmul(cscale(csub(zk, zhc), (T)0.5), twid(tw, k, -1)), -1));
    C xh = cadd(cscale(cadd(zh, zkc), (T)0.5), cmuli(cmul(cscale(csub(zh, zkc), (T)0.5), twid(tw, H - k, -1)), -1));
    if (2 * k != H) tile[(H - k) * TCP + row] = xh;
    tile[k * TCP + row] = xk;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < RPC * S; e += NT) {
    const int row = e / S, m = e % S;
    if (row < rows_valid) base[e] = cscale(tile[m * TCP + row], scale);
  }
}

template <typename T, int H, int RPC, int NT>
__global__ void __launch_bounds__(NT) k_fft_rows_r2c_fixed(typename Cx<T>::type *data, int x0, int ty0,
                                                           const typename Cx<T>::type *tw, T scale) {
  using C = typename Cx<T>::type;
  constexpr int S = H + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  C *tile = reinterpret_cast<C *>(smraw);
  const long long r0 = row_tile_start<2 * H, RPC>(x0, ty0);
  const int rows_valid = RPC;
  rows_r2c_tile<T, H, RPC, NT, false>(tile, data + (size_t)r0 * S, rows_valid, tw, scale);
}

// ---- plane pass: y transforms and z rows of every x plane in one persistent kernel ----
// After the x pass (before it, for r2c) each x plane of N (N/2 + 1) coefficients is
// finished by the y transforms of its column tiles and the real transforms of its
// rows.  As two passes they send the whole array through HBM twice.  Here resident
// CTAs take tasks from a ticket counter in an order that runs the second kind of
// task of a group of planes `lag` groups after the first kind, so a plane is still
// in L2 when it is read again and HBM carries one read and one write of the array for
// both transforms.  A second-kind task waits (one thread, bounded) for its plane's
// count of finished first-kind tasks; those hold smaller tickets, so they were taken
// by CTAs that are running, and the wait ends.  Tiles written by other CTAs of the
// launch are read through L2 only (ld.global.cg), never from a stale L1 line.
//   c2r (INV): first kind = y transform of TC columns (sign +1), second = RPC rows c2r
//   r2c:       first kind = RPC rows r2c, second = y transform of TC columns (sign -1)
// sync: N plane counters and the ticket, zeroed before the launch; wait_flag is set
// when a wait gives up (the host reports it).  A wait polls at most spin_limit times
// (100 ns apart) for `need` finished first-kind tasks of its plane: the plane's count
// of them, unless a test raises it to make every wait give up.

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_gpu(unsigned *p, unsigned v) {
  asm volatile("fence.acq_rel.gpu;\n\tred.relaxed.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <int N, int TC, int RPC>
struct PlaneTasks {
  static constexpr int S = N / 2 + 1, NY = (S + TC - 1) / TC, NZ = N / RPC;
};

template <typename T, int N, int TC, int RPC, int NT, bool INV>
__global__ void __launch_bounds__(NT, 1024 / NT) k_fft_planes(typename Cx<T>::type *data,
                                                               const typename Cx<T>::type *tw, T scale, int group,
                                                               int lag, unsigned *sync, int *wait_flag,
                                                               unsigned spin_limit, unsigned need) {
  using C = typename Cx<T>::type;
  using PT = PlaneTasks<N, TC, RPC>;
  constexpr int H = N / 2, S = PT::S;
  constexpr int P1 = INV ? PT::NY : PT::NZ, P2 = INV ? PT::NZ : PT::NY;
  extern __shared__ __align__(16) unsigned char smraw[];
  C *tile = reinterpret_cast<C *>(smraw);
  __shared__ int s_ticket;
  unsigned *plane_done = sync, *ticket = sync + N;
  const int ngroups = N / group;
  const int A = P1 * group, B = P2 * group;
  const int total = (A + B) * ngroups;
  for (;;) {
    if (threadIdx.x == 0) s_ticket = (int)atomicAdd(ticket, 1u);
    __syncthreads();
    const int t = s_ticket;
    if (t >= total) return;
    // ticket -> (kind, group, index): lag steps of first kinds, then first and second
    // kinds alternating by group, then the last lag groups' second kinds
    bool first;
    int g, idx;
    if (t < lag * A) {
      first = true;
      g = t / A;
      idx = t % A;
    } else if (t - lag * A < (ngroups - lag) * (A + B)) {
      const int u = t - lag * A, step = lag + u / (A + B), r = u % (A + B);
      first = r < A;
      g = first ? step : step - lag;
      idx = first ? r : r - A;
    } else {
      const int u = t - lag * A - (ngroups - lag) * (A + B);
      first = false;
      g = ngroups + u / B - lag;
      idx = u % B;
    }
    const int plane = g * group + idx % group, sub = idx / group;
    if (!first) {
      if (threadIdx.x == 0) {
        unsigned spins = 0;
        while (ld_acquire_gpu(plane_done + plane) < need) {
          if (++spins > spin_limit) {
            atomicExch(wait_flag, 1);
            break;
          }
          __nanosleep(100);
        }
      }
      __syncthreads();
    }
    const bool rows_task = first != INV;
    C *pbase = data + (size_t)plane * (size_t)N * S;
    if (rows_task) {
      if (INV) rows_c2r_tile<T, H, RPC, NT, true>(tile, pbase + (size_t)sub * RPC * S, RPC, tw, scale);
      else rows_r2c_tile<T, H, RPC, NT, true>(tile, pbase + (size_t)sub * RPC * S, RPC, tw, (T)1);
    } else {
      constexpr int SIGN = INV ? +1 : -1;
      const long long b0 = (long long)sub * TC;
      const int tcv = (int)min((long long)TC, (long long)S - b0);
      C *base = pbase + b0;
      first_stage_from<T, N, TC, NT, SIGN>(tile, ColsIn<C, true>{base, S, tcv, {}, N, b0});
      constexpr int R0 = next_radix(N, 1), NSL = last_stage_ns(N);
      TileStagesUntil<T, N, TC, TC, NT, R0, NSL, SIGN, 1>::run(tile, tw);
      last_stage_to<T, N, TC, NT, SIGN, 1>(tile, tw, ColsOut<C, T>{base, S, tcv, (T)1, {}, N, b0});
    }
    __syncthreads();
    if (first && threadIdx.x == 0) red_release_gpu(plane_done + plane, 1u);
  }
}


// ---- TMA-staged strided pass (persistent) ------------------------------------------
// Each CTA walks its share of the column tiles with a ring of two shared-memory slots
// filled by bulk tensor copies (cp.async.bulk.tensor, completion counted on an mbarrier
// per slot).  The threads read a tile's first-stage inputs from its slot and, once all
// of them have, one thread issues the copy of the tile two ahead into that slot; the
// tile's remaining Stockham stages run in an exchange tile meanwhile, and the last
// stage stores straight to HBM.  So a copy is always in flight behind the arithmetic.
// Twiddles are copied to shared memory once per CTA.  The arithmetic (radix schedule,
// twiddle indices, explicit fused multiply-adds) is the fused pass's: the same bits.
// Plain passes and inverse passes with a store window (EXT) only: with one 16-warp CTA
// per SM the per-|k|^2 table gathers of the x passes' multipliers and epilogues are
// latency-bound here (measured 2-4x slower), so those passes stay with the fused pass.
//
// Tile layouts in a slot, matching the tensor map the host builds:
//   rows  (PAIRS = false): rows of B complex whose byte stride is a multiple of 16 (the
//         x pass, and the y pass in FP64): boxes (TC, <= 256 rows) of one plane, slot [L][TC];
//   pairs (PAIRS = true): FP32 rows of odd length B (the y pass; a row is not 16-byte
//         aligned): two rows seen as one of 2B, a box of TC + 2 values for the even rows
//         at column b0 and one for the odd rows at B - 1 + b0 (16-byte aligned starts),
//         slot [2][L/2][TC + 2], odd rows' values one place in.
// A wait for a copy is bounded (about a second of clock cycles); one that gives up sets
// *err (the FFT wait flag the host reads) and the CTA stops after the copies it issued
// have landed (again bounded).

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// waits for the phase of the given parity to complete; false after `cycles` clocks
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *b, unsigned parity, long long cycles) {
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity))
    if (clock64() - t0 > cycles) return false;
  return true;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
template <typename T>
struct TmaColsArgs {
  typename Cx<T>::type *data;  // the array (A planes of L x B complex)
  long long B;
  int A, a0, ntb, ntiles;      // planes (a0 + i) mod A; ntb column tiles per plane
  const typename Cx<T>::type *tw;
  T scale;
  int sm0, smn;                // inverse: positions (sm0 + i) mod L, i < smn, stored
  int *err;
  long long wait_cycles;
};

template <int L, int TC, bool PAIRS>
struct TmaColsShape {
  static constexpr int SLOT = PAIRS ? L * (TC + 2) : L * TC;  // complex values per slot
  static constexpr int ROWS = PAIRS ? L / 2 : L;              // rows of the tensor per tile
  static constexpr int BOXR = ROWS < 256 ? ROWS : 256;       // rows per bulk copy
  static constexpr int W = PAIRS ? TC + 2 : TC;              // values per row of a box
};

// SHUF (L = 512, 16 columns, 16 warps): the middle and last radix-8 stages run in registers,
// exchanging through warp shuffles instead of the exchange tile.  Each group of 8 lanes holds
// one column's butterflies 8q + s (q = lane in the group) of the middle stage; the last stage
// needs output t of butterflies 8r + s in lane t, an 8 x 8 transpose done by three rounds of
// pairwise swaps (__shfl_xor_sync 4, 2, 1).  The first stage writes the exchange tile with
// its columns permuted by row / 8 (c ^ (row / 8 mod 16)), so that the middle stage's reads of
// 8 rows 8 apart fall in different banks.  The arithmetic is the other variants' (same
// radix schedule, twiddle indices and fused multiply-adds): the same bits.
template <typename T, int L, int TC, int NCW, int SIGN, bool EXT, bool PAIRS, bool SHUF = false>
__global__ void __launch_bounds__(NCW * 32, L >= 512 ? 1 : 2) k_fft_cols_tma(const __grid_constant__ CUtensorMap map,
                                                                            const TmaColsArgs<T> a) {
  using C = typename Cx<T>::type;
  using SH = TmaColsShape<L, TC, PAIRS>;
  constexpr int NC = NCW * 32, SLOT = SH::SLOT, NBOX = SH::ROWS / SH::BOXR;
  extern __shared__ __align__(16) unsigned char smraw[];
  const unsigned pad = (1024u - (smem_u32(smraw) & 1023u)) & 1023u;  // bulk-copy destinations: 1024-byte aligned
  C *slots = reinterpret_cast<C *>(smraw + pad);
  C *xt = slots + 2 * SLOT;
  C *stw = xt + L * TC;
  uint64_t *full = reinterpret_cast<uint64_t *>(stw + L);
  __shared__ int s_stop;
  const int ct = threadIdx.x;
  const int nt = (int)gridDim.x, mine = a.ntiles > (int)blockIdx.x ? (a.ntiles - (int)blockIdx.x + nt - 1) / nt : 0;
  // the copy of this CTA's k-th tile into slot k & 1 (one thread)
  auto issue = [&](int k) {
    const int s = k & 1;
    const int t = (int)blockIdx.x + k * nt;
    const int plane = (a.a0 + t / a.ntb) % a.A, b0 = (t % a.ntb) * TC;
    mbar_expect_tx(&full[s], SLOT * (unsigned)sizeof(C));
    C *dst = slots + s * SLOT;
    // tensor coordinates count scalars (two per complex value) along the rows
#pragma unroll
    for (int r = 0; r < NBOX; ++r) {
      tma_load_3d(dst + r * SH::BOXR * SH::W, &map, 2 * b0, r * SH::BOXR, plane, &full[s]);
      if (PAIRS)
        tma_load_3d(dst + (SH::ROWS + r * SH::BOXR) * SH::W, &map, (int)(2 * (a.B - 1 + b0)), r * SH::BOXR, plane,
                    &full[s]);
    }
  };
  if (ct == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    s_stop = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (mine > 0) issue(0);
    if (mine > 1) issue(1);
  }
  for (int i = ct; i < L; i += NC) stw[i] = a.tw[i];
  __syncthreads();
  constexpr int R = next_radix(L, 1), LR = L / R, NB = LR * TC, PER = (NB + NC - 1) / NC;
  constexpr int NSL = last_stage_ns(L), RL = L / NSL, LRL = L / RL, NBL = LRL * TC, PERL = (NBL + NC - 1) / NC;
  for (int k = 0; k < mine; ++k) {
    const int s = k & 1;
    const unsigned ph = (unsigned)(k >> 1) & 1u;
    if (ct == 0 && !mbar_wait_bounded(&full[s], ph, a.wait_cycles)) {
      s_stop = 1;
      atomicExch(a.err, 3);
      // the copies issued and not yet waited for: this tile's and, if issued, the next one's
      if (k + 1 < mine) mbar_wait_bounded(&full[s ^ 1], ((unsigned)((k + 1) >> 1)) & 1u, a.wait_cycles);
      mbar_wait_bounded(&full[s], ph, a.wait_cycles);
    }
    // also orders this tile's exchange-tile writes after the last tile's final reads
    __syncthreads();
    if (s_stop) return;
    const int t = (int)blockIdx.x + k * nt;
    const int plane = (a.a0 + t / a.ntb) % a.A;
    const long long b0 = (long long)(t % a.ntb) * TC;
    const int tcv = (int)min((long long)TC, a.B - b0);
    const size_t off = (size_t)plane * (size_t)L * (size_t)a.B + (size_t)b0;
    const C *in = slots + s * SLOT;
    C v[PER][R];
    // positions j + r LR of column c; LR is even, so in the pairs layout a thread's rows
    // share one parity and step LR / 2 rows of the box
    static_assert(!PAIRS || LR % 2 == 0, "row pairs need an even stride");
    constexpr int RSTEP = PAIRS ? (LR / 2) * SH::W : LR * TC;
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int b = ct + p * NC;
      if (NB % NC == 0 || b < NB) {
        const int c = b % TC, j = b / TC;
        const C *src = in + (PAIRS ? (j & 1) * (SH::ROWS * SH::W + 1) + (j >> 1) * SH::W + c : j * TC + c);
        const bool valid = c < tcv;
#pragma unroll
        for (int r = 0; r < R; ++r) v[p][r] = valid ? src[r * RSTEP] : czero<C>();
      }
    }
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int b = ct + p * NC;
      if (NB % NC == 0 || b < NB) {
        const int c = b % TC, j = b / TC;
        Dft<T, C, R>::run(v[p], SIGN);
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int row = j * R + r;
          xt[row * TC + (SHUF ? (c ^ ((row >> 3) & (TC - 1))) : c)] = v[p][r];
        }
      }
    }
    __syncthreads();
    // every thread has read slot s: refill it with the tile two ahead
    if (ct == 0 && k + 2 < mine) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(k + 2);
    }
    C *base = a.data + off;
    if constexpr (SHUF) {
      static_assert(L == 512 && TC == 16 && NC == 512 && R == 8 && NSL == 64 && RL == 8,
                    "the shuffle stages are laid out for 512-point columns, 16 per tile, 512 threads");
      const int lane = ct & 31, w = ct >> 5, g = lane >> 3, q = lane & 7;
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const int u = p * 64 + w * 4 + g, c = u & 15, sm = u >> 4;
        // middle stage (NS = 8): butterfly 8q + sm, positions 8q + sm + 64r
        C v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r) {
          const int row = 8 * q + sm + 64 * r;
          v[r] = xt[row * 16 + (c ^ ((row >> 3) & 15))];
        }
#pragma unroll
        for (int r = 1; r < 8; ++r) v[r] = cmul(v[r], twid(stw, r * sm * 8, SIGN));
        Dft<T, C, 8>::run(v, SIGN);
        // output r' of butterfly 8q + sm is position 64q + sm + 8r'; the last stage's butterfly
        // sm + 8t reads positions sm + 8t + 64r: output t of butterfly 8r + sm
#pragma unroll
        for (int kb = 4; kb >= 1; kb >>= 1) {
          const bool up = (q & kb) != 0;
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            if (e & kb) continue;
            const C send = up ? v[e] : v[e | kb];
            C recv;
            recv.x = __shfl_xor_sync(0xffffffffu, send.x, kb);
            recv.y = __shfl_xor_sync(0xffffffffu, send.y, kb);
            if (up) v[e] = recv;
            else v[e | kb] = recv;
          }
        }
        // last stage (NS = 64): butterfly j = sm + 8q, positions j + 64r
        const int j = sm + 8 * q;
#pragma unroll
        for (int r = 1; r < 8; ++r) v[r] = cmul(v[r], twid(stw, r * j, SIGN));
        Dft<T, C, 8>::run(v, SIGN);
        if (c < tcv) {
          C *out = base + (size_t)j * (size_t)a.B + c;
          const size_t ostep = (size_t)64 * (size_t)a.B;
#pragma unroll
          for (int r = 0; r < 8; ++r) {
            if (EXT && (j + r * 64 - a.sm0 + L) % L >= a.smn) continue;
            out[r * ostep] = cscale(v[r], a.scale);
          }
        }
      }
      continue;
    }
    TileStagesUntil<T, L, TC, TC, NC, R, NSL, SIGN, 1>::run(xt, stw);
#pragma unroll
    for (int p = 0; p < PERL; ++p) {
      const int b = ct + p * NC;
      if (NBL % NC == 0 || b < NBL) {
        const int c = b % TC, j = b / TC;
        C w[RL];
#pragma unroll
        for (int r = 0; r < RL; ++r) w[r] = xt[(j + r * LRL) * TC + c];
#pragma unroll
        for (int r = 1; r < RL; ++r) w[r] = cmul(w[r], twid(stw, r * j * (L / (NSL * RL)), SIGN));
        Dft<T, C, RL>::run(w, SIGN);
        if (c < tcv) {
          C *out = base + (size_t)j * (size_t)a.B + c;
          const size_t ostep = (size_t)NSL * (size_t)a.B;
#pragma unroll
          for (int r = 0; r < RL; ++r) {
            if (EXT && (j + r * NSL - a.sm0 + L) % L >= a.smn) continue;
            out[r * ostep] = cscale(w[r], a.scale);
          }
        }
      }
    }
  }
}

template <typename T>
void set_smem(const void *fn, size_t bytes) {
  GIC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

// launchers of the fixed-length passes; candidate tile widths per precision:
//   strided: (TC, threads) = FP32 (8, 256) | (16, 512) | fused (8, 512) | fused (16, 512),
//            FP64 (4, 256) | (8, 256) | fused (4, 256) | fused (8, 128);
//            then fused 8 (FP64: 4) columns with 3 or 4 CTAs per SM, and (256 <= N <= 512)
//            the TMA-staged pass: 16 (FP64: 8) columns, 16 warps at N = 512, 8 below; the same
//            with warp-shuffle middle and last stages (FP32, N = 512; else as candidate 6)
//   rows:    (RPC, threads) = FP32 (8, 256) | (16, 256) | fused (16, 256) | (32, 512),
//            FP64 (4, 256) | (8, 256) | fused (8, 256) | (16, 512)
constexpr int kFixedCandidates = 4;  // row-pass candidates
constexpr int kColsCandidates = 8;   // strided-pass candidates (4, 5: fused, 8 columns, 3 or 4 CTAs per SM; 6: TMA-staged;
                                     // 7: TMA-staged with warp-shuffle stages)

// cuTensorMapEncodeTiled, looked up once through the runtime (no link-time dependency on
// the driver library); null when the driver does not provide it
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (EncodeTiledFn) nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(f);
  }();
  return fn;
}

// the dynamic shared-memory limit of a kernel, set once per device (any host thread)
inline void set_smem_once(const void *fn, size_t bytes, std::atomic<int> &done_mask) {
  int dev = 0;
  GIC_CUDA(cudaGetDevice(&dev));
  if (done_mask.load() & (1 << (dev & 31))) return;
  GIC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  done_mask.fetch_or(1 << (dev & 31));
}

template <typename T, int N>
struct FixedFft {
  using C = typename Cx<T>::type;
  static constexpr int H = N / 2, S = H + 1;
  static constexpr bool F32 = sizeof(T) == 4;

  // planes and rows of a box (the whole transform: x0 = y0 = 0, nx = ny = N)
  struct Sel {
    int x0, nx, y0, ny;
    bool whole() const { return nx >= N && ny >= N; }
  };
  static Sel whole_sel() { return Sel{0, N, 0, N}; }

  template <int TC, int NT, int SIGN>
  static void cols(Context &ctx, C *d, int A, long long B, const C *tw, T scale, XTab<T> tab, int a0, int na,
                   int m0, int mn, const C *src, C *dst, const C *xsrc, XTab<T> xtab) {
    static std::atomic<int> mask{0};
    const size_t smem = (size_t)N * (TC + 1) * sizeof(C);
    set_smem_once((const void *)k_fft_cols<T, N, TC, NT, SIGN>, smem, mask);
    dim3 grid((unsigned)((B + TC - 1) / TC), (unsigned)na);
    k_fft_cols<T, N, TC, NT, SIGN><<<grid, NT, smem, ctx.stream>>>(d, B, tw, scale, tab, a0, A, m0, mn, src, dst, xsrc,
                                                                   xtab);
    launched();
  }
  template <int TC, int NT, int SIGN, int MINB = 1024 / NT>
  static void cols_fused(Context &ctx, C *d, int A, long long B, const C *tw, T scale, XTab<T> tab, int a0,
                         int na, int m0, int mn, const C *src, C *dst, const C *xsrc, XTab<T> xtab) {
    static std::atomic<int> mask{0}, mask_plain{0};
    // FP32 x passes stage their multipliers' per-coefficient layouts in shared memory
    // (FP64 would lose a resident CTA per SM to the extra shared memory)
    const size_t rows = (size_t)(N / 2 + 1) * TC * sizeof(T);
    const bool stage = F32 && B == (long long)N * S && (tab.col || (dst && xtab.col));
    const size_t smem_max = (size_t)N * TC * sizeof(C) + (F32 ? 2 * rows : 0);
    const size_t smem = (size_t)N * TC * sizeof(C) + (stage ? ((tab.col ? rows : 0) + (dst && xtab.col ? rows : 0)) : 0);
    dim3 grid((unsigned)((B + TC - 1) / TC), (unsigned)na);
    if (src || dst || m0 != 0 || mn < N) {
      set_smem_once((const void *)k_fft_cols_fused<T, N, TC, NT, SIGN, MINB, true>, smem_max, mask);
      k_fft_cols_fused<T, N, TC, NT, SIGN, MINB, true><<<grid, NT, smem, ctx.stream>>>(d, B, tw, scale, tab, a0, A, m0, mn,
                                                                                       src, dst, xsrc, xtab, stage);
    } else {
      set_smem_once((const void *)k_fft_cols_fused<T, N, TC, NT, SIGN, MINB, false>, smem_max, mask_plain);
      k_fft_cols_fused<T, N, TC, NT, SIGN, MINB, false><<<grid, NT, smem, ctx.stream>>>(d, B, tw, scale, tab, a0, A, m0,
                                                                                        mn, src, dst, xsrc, xtab, stage);
    }
    launched();
  }
  // row tiles of RPC rows covering the selection: grid (tiles, planes)
  template <int RPC>
  static dim3 row_grid(const Sel &sel, int &ty0) {
    constexpr int NTILE = N / RPC;
    ty0 = sel.y0 / RPC;
    const int nty = std::min(NTILE, (sel.y0 + sel.ny - 1) / RPC - ty0 + 1);
    return dim3((unsigned)nty, (unsigned)sel.nx);
  }
  template <int RPC, int NT, bool INV>
  static void rows_fused(Context &ctx, C *d, const C *tw, T scale, const Sel &sel) {
    static std::atomic<int> mask{0};
    const size_t smem = (size_t)(INV ? H : S) * RPC * sizeof(C);
    int ty0 = 0;
    const dim3 grid = row_grid<RPC>(sel, ty0);
    if (INV) {
      set_smem_once((const void *)k_fft_rows_c2r_fused<T, H, RPC, NT>, smem, mask);
      k_fft_rows_c2r_fused<T, H, RPC, NT><<<grid, NT, smem, ctx.stream>>>(d, sel.x0, ty0, tw, scale);
    } else {
      set_smem_once((const void *)k_fft_rows_r2c_fused<T, H, RPC, NT>, smem, mask);
      k_fft_rows_r2c_fused<T, H, RPC, NT><<<grid, NT, smem, ctx.stream>>>(d, sel.x0, ty0, tw, scale);
    }
    launched();
  }
  template <int RPC, int NT, bool INV>
  static void rows(Context &ctx, C *d, const C *tw, T scale, const Sel &sel) {
    static std::atomic<int> mask{0};
    const size_t smem = (size_t)S * (RPC + 1) * sizeof(C);
    int ty0 = 0;
    const dim3 grid = row_grid<RPC>(sel, ty0);
    if (INV) {
      set_smem_once((const void *)k_fft_rows_c2r_fixed<T, H, RPC, NT>, smem, mask);
      k_fft_rows_c2r_fixed<T, H, RPC, NT><<<grid, NT, smem, ctx.stream>>>(d, sel.x0, ty0, tw, scale);
    } else {
      set_smem_once((const void *)k_fft_rows_r2c_fixed<T, H, RPC, NT>, smem, mask);
      k_fft_rows_r2c_fixed<T, H, RPC, NT><<<grid, NT, smem, ctx.stream>>>(d, sel.x0, ty0, tw, scale);
    }
    launched();
  }
  // the TMA-staged strided pass (k_fft_cols_tma) for 256 <= N <= 512; false where it does
  // not apply, and the caller runs a fused pass: a forward pass that reads a window of
  // positions only (the fused pass loads just the window), an x pass with a multiplier,
  // an out-of-place source or an epilogue, or no tensor-map encoder
  static constexpr bool kTma = N >= 256 && N <= 512;
  template <int SIGN, bool EXT, bool PAIRS, bool SHUF = false>
  static void launch_tma(Context &ctx, const CUtensorMap &map, const TmaColsArgs<T> &args) {
    constexpr int TC = F32 ? 16 : 8, NCW = N >= 512 ? 16 : 8;
    using SH = TmaColsShape<N, TC, PAIRS>;
    const void *fn = (const void *)k_fft_cols_tma<T, N, TC, NCW, SIGN, EXT, PAIRS, SHUF>;
    const size_t smem = 1024 + (2 * (size_t)SH::SLOT + (size_t)N * TC + N) * sizeof(C) + 2 * sizeof(uint64_t);
    static std::atomic<int> mask{0}, resident{0};
    set_smem_once(fn, smem, mask);
    if (resident.load() == 0) {
      int nb = 0;
      GIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, NCW * 32, smem));
      resident.store(std::max(nb, 1));
    }
    int dev = 0, nsm = 0;
    GIC_CUDA(cudaGetDevice(&dev));
    GIC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int grid = std::min(args.ntiles, resident.load() * nsm);
    k_fft_cols_tma<T, N, TC, NCW, SIGN, EXT, PAIRS, SHUF><<<grid, NCW * 32, smem, ctx.stream>>>(map, args);
    launched();
  }
  // SHUF: the variant with warp-shuffle middle and last stages (FP32, N = 512)
  static constexpr bool kShuf = F32 && N == 512;
  static bool cols_tma(Context &ctx, int sign, C *d, int A, long long B, const C *tw, T scale, XTab<T> tab, int a0,
                       int na, int m0, int mn, const C *src, C *dst, const C *xsrc, XTab<T> xtab, bool shuf = false) {
    if constexpr (!kTma) {
      return false;
    } else {
      if ((sign < 0 && mn < N) || tab || src || dst || xsrc || xtab) return false;
      constexpr int TC = F32 ? 16 : 8;
      const bool pairs = ((size_t)B * sizeof(C)) % 16 != 0;
      if (pairs && !(F32 && B % 2 == 1)) return false;
      EncodeTiledFn enc = encode_tiled_fn();
      if (!enc) return false;
      if (reinterpret_cast<uintptr_t>(d) % 16) return false;
      // the tensor: scalars along a row (two per complex value), rows (or row pairs), planes
      cuuint64_t dims[3], strides[2];
      cuuint32_t box[3], es[3] = {1, 1, 1};
      if (!pairs) {
        dims[0] = (cuuint64_t)(2 * B);
        dims[1] = (cuuint64_t)N;
        strides[0] = (cuuint64_t)(B * (long long)sizeof(C));
        box[0] = 2 * TC;
        box[1] = (cuuint32_t)std::min(N, 256);
      } else {
        dims[0] = (cuuint64_t)(4 * B);
        dims[1] = (cuuint64_t)(N / 2);
        strides[0] = (cuuint64_t)(2 * B * (long long)sizeof(C));
        box[0] = 2 * (TC + 2);
        box[1] = (cuuint32_t)std::min(N / 2, 256);
      }
      dims[2] = (cuuint64_t)A;
      strides[1] = (cuuint64_t)((long long)N * B * (long long)sizeof(C));
      box[2] = 1;
      CUtensorMap map;
      if (enc(&map, F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, d, dims,
              strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
      TmaColsArgs<T> args{};
      args.data = d;
      args.B = B;
      args.A = A;
      args.a0 = a0;
      args.ntb = (int)((B + TC - 1) / TC);
      args.ntiles = args.ntb * na;
      args.tw = tw;
      args.scale = scale;
      args.sm0 = m0;
      args.smn = mn;
      args.err = ctx.fft.wait_flag();
      args.wait_cycles = 1ll << 31;
      if (args.ntiles <= 0) return true;
      const bool ext = sign > 0 && mn < N;
      if constexpr (kShuf) {
        if (shuf) {
          if (pairs) {
            if (sign > 0) ext ? launch_tma<+1, true, true, true>(ctx, map, args) : launch_tma<+1, false, true, true>(ctx, map, args);
            else ext ? launch_tma<-1, true, true, true>(ctx, map, args) : launch_tma<-1, false, true, true>(ctx, map, args);
          } else {
            if (sign > 0) ext ? launch_tma<+1, true, false, true>(ctx, map, args) : launch_tma<+1, false, false, true>(ctx, map, args);
            else ext ? launch_tma<-1, true, false, true>(ctx, map, args) : launch_tma<-1, false, false, true>(ctx, map, args);
          }
          return true;
        }
      }
      if (pairs) {
        if constexpr (F32) {
          if (sign > 0) ext ? launch_tma<+1, true, true>(ctx, map, args) : launch_tma<+1, false, true>(ctx, map, args);
          else ext ? launch_tma<-1, true, true>(ctx, map, args) : launch_tma<-1, false, true>(ctx, map, args);
        }
      } else {
        if (sign > 0) ext ? launch_tma<+1, true, false>(ctx, map, args) : launch_tma<+1, false, false>(ctx, map, args);
        else ext ? launch_tma<-1, true, false>(ctx, map, args) : launch_tma<-1, false, false>(ctx, map, args);
      }
      return true;
    }
  }
  // a0, na: the planes (a0 + i) mod A, i < na, of the strided pass (na < 0: all A);
  // m0, mn: the positions along the transform read (forward) or written (inverse)
  // src: an out-of-place inverse x pass reads the columns other than kz = 0, N/2 from src
  // dst, xsrc, xtab: a forward x pass writes xtab[q] xsrc + result to dst instead of in place
  static void cols_cfg(Context &ctx, int cfg, int sign, C *d, int A, long long B, const C *tw, T scale,
                       XTab<T> tab = {}, int a0 = 0, int na = -1, int m0 = 0, int mn = N,
                       const C *src = nullptr, C *dst = nullptr, const C *xsrc = nullptr, XTab<T> xtab = {}) {
    if (na < 0) na = A;
    if (cfg == 6 || cfg == 7) {
      // TMA-staged (7: with warp-shuffle middle and last stages where built), else the fused
      // 16- (FP64: 8-) column pass
      if (cols_tma(ctx, sign, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab, cfg == 7)) return;
      cfg = 3;
    }
    if (cfg == 4) {
      // fused, 8 columns, registers capped for 3 CTAs of 512 threads per SM (48 warps)
      if (sign > 0) cols_fused<F32 ? 8 : 4, 512, +1, 3>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
      else cols_fused<F32 ? 8 : 4, 512, -1, 3>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
      return;
    }
    if (cfg == 5) {
      // fused, 8 columns, registers capped for 4 CTAs of 512 threads per SM (64 warps)
      if (sign > 0) cols_fused<F32 ? 8 : 4, 512, +1, 4>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
      else cols_fused<F32 ? 8 : 4, 512, -1, 4>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
      return;
    }
    if (cfg == 2) {
      if (sign > 0) cols_fused<F32 ? 8 : 4, F32 ? 512 : 256, +1>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
      else cols_fused<F32 ? 8 : 4, F32 ? 512 : 256, -1>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
    } else if (cfg == 3) {
      if (sign > 0) cols_fused<F32 ? 16 : 8, F32 ? 512 : 128, +1>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
      else cols_fused<F32 ? 16 : 8, F32 ? 512 : 128, -1>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
    } else if (cfg == 0) {
      if (sign > 0) cols<F32 ? 8 : 4, 256, +1>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
      else cols<F32 ? 8 : 4, 256, -1>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
    } else {
      if (sign > 0) cols<F32 ? 16 : 8, F32 ? 512 : 256, +1>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
      else cols<F32 ? 16 : 8, F32 ? 512 : 256, -1>(ctx, d, A, B, tw, scale, tab, a0, na, m0, mn, src, dst, xsrc, xtab);
    }
  }
  static void rows_cfg(Context &ctx, int cfg, bool inv, C *d, const C *tw, T scale, const Sel &sel = whole_sel()) {
    if (cfg == 2) {
      if (inv) rows_fused<F32 ? 16 : 8, 256, true>(ctx, d, tw, scale, sel);
      else rows_fused<F32 ? 16 : 8, 256, false>(ctx, d, tw, scale, sel);
    } else if (cfg == 3) {
      if (inv) rows<F32 ? 32 : 16, 512, true>(ctx, d, tw, scale, sel);
      else rows<F32 ? 32 : 16, 512, false>(ctx, d, tw, scale, sel);
    } else if (cfg == 0) {
      if (inv) rows<F32 ? 8 : 4, 256, true>(ctx, d, tw, scale, sel);
      else rows<F32 ? 8 : 4, 256, false>(ctx, d, tw, scale, sel);
    } else {
      if (inv) rows<F32 ? 16 : 8, 256, true>(ctx, d, tw, scale, sel);
      else rows<F32 ? 16 : 8, 256, false>(ctx, d, tw, scale, sel);
    }
  }
  // plane pass (N >= 256 in FP32, N >= 512 in FP64): column tiles and row tiles sized for 512 threads and about
  // 64 KB of shared memory, two CTAs per SM; `group` planes per step of the ticket order
  static constexpr bool kPlanes = F32 ? N >= 256 : N >= 512;
  static constexpr int kPlaneVariants = 3;
  template <bool INV>
  static void planes(Context &ctx, C *d, const C *tw, T scale, int variant) {
    if constexpr (kPlanes) {
      constexpr int PTC = F32 ? (N >= 1024 ? 8 : 16) : (N >= 1024 ? 4 : 8);
      constexpr int PRPC = F32 ? (N >= 1024 ? 16 : 32) : (N >= 1024 ? 8 : 16);
      constexpr int PNT = 512;
      static std::atomic<int> mask{0};
      static std::atomic<int> resident{0};
      const void *fn = (const void *)k_fft_planes<T, N, PTC, PRPC, PNT, INV>;
      const size_t smem = std::max((size_t)N * PTC, (size_t)S * (PRPC + 1)) * sizeof(C);
      set_smem_once(fn, smem, mask);
      int dev = 0, nsm = 0;
      GIC_CUDA(cudaGetDevice(&dev));
      GIC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      if (resident.load() == 0) {
        int nb = 0;
        GIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, PNT, smem));
        resident.store(std::max(nb, 1));
      }
      using PT = PlaneTasks<N, PTC, PRPC>;
      const int ctas = resident.load() * nsm;
      const int group = std::max(1, 2048 / N), ngroups = N / group;
      const int per_step = (PT::NY + PT::NZ) * group;
      // lag: 1, 2 or 4 times the resident CTAs, in ticket steps
      const int lag = std::max(1, std::min(ngroups, ((1 << variant) * ctas + per_step - 1) / per_step));
      const int total = per_step * ngroups;
      ctx.fft.plane_sync.ensure((size_t)(N + 1) * sizeof(unsigned));
      GIC_CUDA(cudaMemsetAsync(ctx.fft.plane_sync.ptr, 0, (size_t)(N + 1) * sizeof(unsigned), ctx.stream));
      k_fft_planes<T, N, PTC, PRPC, PNT, INV><<<std::min(ctas, total), PNT, smem, ctx.stream>>>(
          d, tw, scale, group, lag, ctx.fft.plane_sync.template as<unsigned>(), ctx.fft.wait_flag(),
          ctx.fft.plane_spin_limit, (unsigned)(INV ? PT::NY : PT::NZ) + ctx.fft.plane_wait_extra);
      launched();
    }
  }
  // inverse: the x pass over every column, then the y transforms of the selected
  // planes and the real transforms of the selected rows (output valid there)
  static void c2r(Context &ctx, C *c, const C *tw, T scale, int ccfg, int rcfg, int pv, XTab<T> tab,
                  const Sel &sel, const C *src = nullptr) {
    // the x pass stores the selected planes only, the y pass the selected rows only
    cols_cfg(ctx, ccfg, +1, c, 1, (long long)N * S, tw, (T)1, tab, 0, -1, sel.x0, sel.nx, src);
    if (kPlanes && pv >= 0 && sel.whole()) {
      planes<true>(ctx, c, tw, scale, pv);
      return;
    }
    cols_cfg(ctx, ccfg, +1, c, N, S, tw, (T)1, {}, sel.x0, sel.nx, sel.y0, sel.ny);
    rows_cfg(ctx, rcfg, true, c, tw, scale, sel);
  }
  // forward, input zero outside the selection: the selected rows, the selected
  // planes' y transforms, then the x pass over every column
  static void r2c(Context &ctx, C *c, const C *tw, T scale, int ccfg, int rcfg, int pv, XTab<T> tab,
                  const Sel &sel, C *dst = nullptr, const C *xsrc = nullptr, XTab<T> xtab = {}) {
    if (kPlanes && pv >= 0 && sel.whole()) {
      planes<false>(ctx, c, tw, (T)1, pv);
    } else {
      rows_cfg(ctx, rcfg, false, c, tw, (T)1, sel);
      // rows outside the selection are zero: the y pass does not read them
      cols_cfg(ctx, ccfg, -1, c, N, S, tw, (T)1, {}, sel.x0, sel.nx, sel.y0, sel.ny);
    }
    // planes outside the selection are zero: the x pass does not read them
    cols_cfg(ctx, ccfg, -1, c, 1, (long long)N * S, tw, scale, tab, 0, -1, sel.x0, sel.nx, nullptr, dst, xsrc, xtab);
  }
  // time every candidate on a scratch array of the transform's size
  static void tune(Context &ctx, const C *tw, int &best_cols, int &best_rows, int &best_planes) {
    const size_t bytes = (size_t)N * N * S * sizeof(C);
    auto scratch = ctx.pool.take(bytes);
    C *d = scratch->template as<C>();
    GIC_CUDA(cudaMemsetAsync(d, 0, bytes, ctx.stream));
    cudaEvent_t e0, e1;
    GIC_CUDA(cudaEventCreate(&e0));
    GIC_CUDA(cudaEventCreate(&e1));
    auto time_it = [&](auto &&fn) {
      fn();  // warm-up
      GIC_CUDA(cudaEventRecord(e0, ctx.stream));
      for (int r = 0; r < 3; ++r) fn();
      GIC_CUDA(cudaEventRecord(e1, ctx.stream));
      GIC_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      GIC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      return ms;
    };
    float bc = 1e30f, br = 1e30f;
    // a strided candidate is timed on both of its passes (x, then y over every plane)
    for (int c = 0; c < kColsCandidates; ++c) {
      float t = time_it([&] {
        cols_cfg(ctx, c, +1, d, 1, (long long)N * S, tw, (T)1);
        cols_cfg(ctx, c, +1, d, N, S, tw, (T)1);
      });
      if (t < bc) { bc = t; best_cols = c; }
    }
    for (int r = 0; r < kFixedCandidates; ++r) {
      float t = time_it([&] { rows_cfg(ctx, r, true, d, tw, (T)1); });
      if (t < br) { br = t; best_rows = r; }
    }
    // the plane pass against the best separate y and z passes
    best_planes = -1;
    if (kPlanes) {
      float bp = time_it([&] {
        cols_cfg(ctx, best_cols, +1, d, N, S, tw, (T)1);
        rows_cfg(ctx, best_rows, true, d, tw, (T)1);
      });
      for (int v = 0; v < kPlaneVariants; ++v) {
        float t = time_it([&] { planes<true>(ctx, d, tw, (T)1, v); });
        if (t < bp) { bp = t; best_planes = v; }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx.pool.give(std::move(scratch));
  }
};

// tuning results shared by every context of the process, per device, size and precision
struct SharedTune {
  int device, n;
  bool dbl;
  int cols, rows, planes;
};
std::mutex g_tune_mutex;
std::vector<SharedTune> g_tuned;

// out[f][c] = q[f^2 + ky^2 + kz^2], f <= n/2, c = ky (n/2 + 1) + kz (ky signed)
template <typename T>
__global__ void k_col_table(T *out, const T *q, int n) {
  const int S = n / 2 + 1, H = n / 2, per = n * S;
  const int c = (int)(blockIdx.x * blockDim.x + threadIdx.x), f = (int)blockIdx.y;
  if (c >= per) return;
  const int ky = c / S, kz = c - ky * S, b = ky > H ? ky - n : ky;
  out[(size_t)f * (size_t)per + (size_t)c] = q[(long long)f * f + (long long)b * b + (long long)kz * kz];
}

// Layouts of all registered tables together stay below this many bytes.
constexpr size_t kColTableBytes = size_t(8) << 30;

// The per-coefficient layout of the registered per-|k|^2 table q of an n^3 grid, built
// on first use; nullptr where q is not registered, the layout does not fit, or the
// stream is being captured (the x pass then gathers from q: the same values).
template <typename T>
const T *col_table(Context &ctx, const T *q, int n) {
  if (!q || !ctx.fft.col_tables) return nullptr;
  for (auto &e : ctx.col_tables) {
    if (e->q != (const void *)q || e->n != n || e->elem != (int)sizeof(T)) continue;
    if (e->col.ptr) return e->col.template as<T>();
    if (e->failed) return nullptr;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    GIC_CUDA(cudaStreamIsCapturing(ctx.stream, &st));
    if (st != cudaStreamCaptureStatusNone) return nullptr;
    const size_t per = (size_t)n * (size_t)(n / 2 + 1), bytes = (size_t)(n / 2 + 1) * per * sizeof(T);
    size_t held = 0;
    for (auto &o : ctx.col_tables) held += o->col.bytes;
    const MemAccount *a = t_account;
    if (held + bytes > kColTableBytes || (a && a->limit && a->used.load() + bytes > a->limit)) {
      e->failed = true;
      return nullptr;
    }
    try {
      e->col.ensure(bytes);
    } catch (const Error &) {
      e->failed = true;
      return nullptr;
    }
    k_col_table<T><<<dim3((unsigned)((per + 255) / 256), (unsigned)(n / 2 + 1)), 256, 0, ctx.stream>>>(
        e->col.template as<T>(), q, n);
    launched();
    return e->col.template as<T>();
  }
  return nullptr;
}

template <typename T, int N>
void fixed_transform(Context &ctx, typename Cx<T>::type *c, const typename Cx<T>::type *tw, double scale, bool inverse,
                     const T *tab, const CellBox *box, const typename Cx<T>::type *src, typename Cx<T>::type *dst,
                     const typename Cx<T>::type *xsrc, const T *xtab) {
  FftTables &F = ctx.fft;
  const bool dbl = sizeof(T) == 8;
  int cc = -1, rc = -1, pv = -1;
  for (auto &t : F.tuned)
    if (t.n == N && t.dbl == dbl) {
      cc = t.cols;
      rc = t.rows;
      pv = t.planes;
    }
  // a choice pinned by hand (GIC_FFT_TILE) replaces the tuner
  if (cc < 0 && F.force_cols >= 0 && F.force_rows >= 0) {
    cc = F.force_cols;
    rc = F.force_rows;
    pv = -1;
  }
  if (cc < 0) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    for (auto &t : g_tuned)
      if (t.device == ctx.device && t.n == N && t.dbl == dbl) {
        cc = t.cols;
        rc = t.rows;
        pv = t.planes;
      }
    if (cc < 0) {
      cc = 0;
      rc = 0;
      pv = -1;
      if (N >= 128) FixedFft<T, N>::tune(ctx, tw, cc, rc, pv);
      g_tuned.push_back({ctx.device, N, dbl, cc, rc, pv});
    }
    F.tuned.push_back({N, dbl, cc, rc, pv});
  }
  if (F.force_cols >= 0) cc = F.force_cols;
  if (F.force_rows >= 0) rc = F.force_rows;
  if (F.force_planes >= -1) pv = std::min(F.force_planes, FixedFft<T, N>::kPlaneVariants - 1);
  typename FixedFft<T, N>::Sel sel = FixedFft<T, N>::whole_sel();
  if (box && box->len[0] < N) {
    sel.x0 = ((box->start[0] % N) + N) % N;
    sel.nx = box->len[0];
  }
  if (box && box->len[1] < N) {
    sel.y0 = ((box->start[1] % N) + N) % N;
    sel.ny = box->len[1];
  }
  const XTab<T> t{tab, col_table<T>(ctx, tab, N)}, xt{xtab, col_table<T>(ctx, xtab, N)};
  if (inverse) FixedFft<T, N>::c2r(ctx, c, tw, (T)scale, cc, rc, pv, t, sel, src);
  else FixedFft<T, N>::r2c(ctx, c, tw, (T)scale, cc, rc, pv, t, sel, dst, xsrc, xt);
}

// power-of-two sizes 32..1024 use the fixed-length passes
template <typename T>
bool fixed_dispatch(Context &ctx, typename Cx<T>::type *c, int n, const typename Cx<T>::type *tw, double scale,
                    bool inverse, const T *tab, const CellBox *box, const typename Cx<T>::type *src = nullptr,
                    typename Cx<T>::type *dst = nullptr, const typename Cx<T>::type *xsrc = nullptr,
                    const T *xtab = nullptr) {
  switch (n) {
    case 32: fixed_transform<T, 32>(ctx, c, tw, scale, inverse, tab, box, src, dst, xsrc, xtab); return true;
    case 64: fixed_transform<T, 64>(ctx, c, tw, scale, inverse, tab, box, src, dst, xsrc, xtab); return true;
    case 128: fixed_transform<T, 128>(ctx, c, tw, scale, inverse, tab, box, src, dst, xsrc, xtab); return true;
    case 256: fixed_transform<T, 256>(ctx, c, tw, scale, inverse, tab, box, src, dst, xsrc, xtab); return true;
    case 512: fixed_transform<T, 512>(ctx, c, tw, scale, inverse, tab, box, src, dst, xsrc, xtab); return true;
    case 1024: fixed_transform<T, 1024>(ctx, c, tw, scale, inverse, tab, box, src, dst, xsrc, xtab); return true;
    default: return false;
  }
}

template <typename T>
void strided_pass(Context &ctx, typename Cx<T>::type *data, int A, int L, long long B, int sign, T scale,
                  const typename Cx<T>::type *tw, const T *tab = nullptr) {
  constexpr int TC = sizeof(T) == 4 ? 8 : 4;
  Radix plan = make_plan(L);
  size_t smem = 2ull * L * TC * sizeof(typename Cx<T>::type);
  set_smem<T>((const void *)k_fft_strided<T, TC>, smem);
  dim3 grid((unsigned)((B + TC - 1) / TC), (unsigned)A);
  k_fft_strided<T, TC><<<grid, 256, smem, ctx.stream>>>(data, L, B, plan, sign, tw, scale, tab);
  launched();
}

template <typename T>
int rows_per_cta(int N) {
  size_t row_bytes = (size_t)(N / 2 + 1) * sizeof(typename Cx<T>::type);
  int rpc = (int)std::max<size_t>(1, 16384 / row_bytes);
  return std::min(rpc, 32);
}

}  // namespace

template <typename T>
const T *coefficient_table(Context &ctx, const T *q, int n) {
  return col_table<T>(ctx, q, n);
}
template const float *coefficient_table<float>(Context &, const float *, int);
template const double *coefficient_table<double>(Context &, const double *, int);

int *FftTables::wait_flag() {
  if (!wait_flag_host) {
    void *h = nullptr, *d = nullptr;
    GIC_CUDA(cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped));
    *static_cast<int *>(h) = 0;
    if (cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess) {
      cudaGetLastError();
      cudaFreeHost(h);
      fail(GIC_ERR_CUDA, "cudaHostGetDevicePointer failed");
    }
    wait_flag_host = static_cast<int *>(h);
    wait_flag_dev = static_cast<int *>(d);
  }
  return wait_flag_dev;
}

const void *FftTables::get(int n, bool dbl, cudaStream_t s) {
  for (auto &e : entries)
    if (e->n == n) return dbl ? e->f64.ptr : e->f32.ptr;
  auto e = std::make_unique<Entry>();
  e->n = n;
  std::vector<double2> h64(n);
  std::vector<float2> h32(n);
  for (int m = 0; m < n; ++m) {
    long double ang = -2.0L * 3.141592653589793238462643383279502884L * (long double)m / (long double)n;
    h64[m].x = (double)cosl(ang);
    h64[m].y = (double)sinl(ang);
    h32[m].x = (float)cosl(ang);
    h32[m].y = (float)sinl(ang);
  }
  e->f64.ensure(n * sizeof(double2));
  e->f32.ensure(n * sizeof(float2));
  GIC_CUDA(cudaMemcpyAsync(e->f64.ptr, h64.data(), n * sizeof(double2), cudaMemcpyHostToDevice, s));
  GIC_CUDA(cudaMemcpyAsync(e->f32.ptr, h32.data(), n * sizeof(float2), cudaMemcpyHostToDevice, s));
  GIC_CUDA(cudaStreamSynchronize(s));
  entries.push_back(std::move(e));
  return dbl ? entries.back()->f64.ptr : entries.back()->f32.ptr;
}

template <typename T>
void fft_c2r_3d(Context &ctx, T *data, int n, double scale, const T *pre_tab, const CellBox *box) {
  using C = typename Cx<T>::type;
  if (n < 2 || n % 2) fail(GIC_ERR_INVALID_ARG, "FFT size must be even");
  const C *tw = (const C *)ctx.fft.get(n, sizeof(T) == 8, ctx.stream);
  C *c = reinterpret_cast<C *>(data);
  long long S = n / 2 + 1;
  long long mirror_threads = 2ll * n * n;
  k_mirror<T><<<(unsigned)((mirror_threads + 255) / 256), 256, 0, ctx.stream>>>(c, n);
  launched();
  if (ctx.fft.force_cols != -2 && fixed_dispatch<T>(ctx, c, n, tw, scale, true, pre_tab, box)) return;
  strided_pass<T>(ctx, c, 1, n, (long long)n * S, +1, (T)1, tw, pre_tab);
  strided_pass<T>(ctx, c, n, n, S, +1, (T)1, tw);
  int rpc = rows_per_cta<T>(n);
  Radix plan = make_plan(n / 2);
  size_t smem = 2ull * rpc * S * sizeof(C);
  set_smem<T>((const void *)k_fft_rows_c2r<T>, smem);
  long long nrows = (long long)n * n;
  k_fft_rows_c2r<T><<<(unsigned)((nrows + rpc - 1) / rpc), 256, smem, ctx.stream>>>(c, nrows, n, rpc, plan, tw,
                                                                                   (T)scale);
  launched();
}

template <typename T>
void fft_r2c_3d(Context &ctx, T *data, int n, double scale, const T *post_tab, const CellBox *box) {
  using C = typename Cx<T>::type;
  if (n < 2 || n % 2) fail(GIC_ERR_INVALID_ARG, "FFT size must be even");
  const C *tw = (const C *)ctx.fft.get(n, sizeof(T) == 8, ctx.stream);
  C *c = reinterpret_cast<C *>(data);
  long long S = n / 2 + 1;
  if (ctx.fft.force_cols != -2 && fixed_dispatch<T>(ctx, c, n, tw, scale, false, post_tab, box)) return;
  int rpc = rows_per_cta<T>(n);
  Radix plan = make_plan(n / 2);
  size_t smem = 2ull * rpc * S * sizeof(C);
  set_smem<T>((const void *)k_fft_rows_r2c<T>, smem);
  long long nrows = (long long)n * n;
  k_fft_rows_r2c<T><<<(unsigned)((nrows + rpc - 1) / rpc), 256, smem, ctx.stream>>>(c, nrows, n, rpc, plan, tw,
                                                                                   (T)1);
  launched();
  strided_pass<T>(ctx, c, n, n, S, -1, (T)1, tw);
  strided_pass<T>(ctx, c, 1, n, (long long)n * S, -1, (T)scale, tw, post_tab);
}

bool fft_prunes(const Context &ctx, int n) {
  return ctx.fft.force_cols != -2 && n >= 32 && n <= 1024 && (n & (n - 1)) == 0;
}

bool take_fft_wait_error(Context &ctx) {
  volatile int *f = ctx.fft.wait_flag_host;
  if (!f || *f == 0) return false;
  ctx.last_error = *f == 4   ? "block means (k_fold_rows): a wait for the fine rows' bulk copies gave up; the coarse "
                               "field is invalid"
                  : *f >= 3 ? "FFT TMA-staged strided pass: a wait for a tile's bulk copy gave up; results of the "
                              "transform are invalid"
                            : "FFT plane pass: a wait for another CTA's tiles gave up; results of the transform are "
                              "invalid";
  *f = 0;
  return true;
}

// dst = xtab[q] x + (the forward transform of data, times post_tab): the x pass writes the sum
template <typename T>
__global__ void k_fft_add_epilogue(typename Cx<T>::type *dst, const typename Cx<T>::type *data,
                                   const typename Cx<T>::type *x, const T *xtab, int n) {
  const size_t S = (size_t)(n / 2 + 1);
  const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (size_t)n * n * S) return;
  const int kx = (int)(id / ((size_t)n * S));
  dst[id] = cadd(cscale(x[id], qtab(xtab, n, kx, (long long)(id - (size_t)kx * n * S))), data[id]);
}

template <typename T>
void fft_r2c_3d_add(Context &ctx, T *data, int n, double scale, const T *post_tab, const CellBox *box, T *dst,
                    const T *x, const T *xtab) {
  using C = typename Cx<T>::type;
  if (n < 2 || n % 2) fail(GIC_ERR_INVALID_ARG, "FFT size must be even");
  C *c = reinterpret_cast<C *>(data);
  if (fft_prunes(ctx, n)) {
    const C *tw = (const C *)ctx.fft.get(n, sizeof(T) == 8, ctx.stream);
    fixed_dispatch<T>(ctx, c, n, tw, scale, false, post_tab, box, nullptr, reinterpret_cast<C *>(dst),
                      reinterpret_cast<const C *>(x), xtab);
    return;
  }
  fft_r2c_3d<T>(ctx, data, n, scale, post_tab, box);
  const size_t m = (size_t)n * n * (n / 2 + 1);
  k_fft_add_epilogue<T><<<(unsigned)((m + 255) / 256), 256, 0, ctx.stream>>>(
      reinterpret_cast<C *>(dst), c, reinterpret_cast<const C *>(x), xtab, n);
  launched();
}

template void fft_r2c_3d_add<float>(Context &, float *, int, double, const float *, const CellBox *, float *,
                                    const float *, const float *);
template void fft_r2c_3d_add<double>(Context &, double *, int, double, const double *, const CellBox *, double *,
                                     const double *, const double *);

template <typename T>
void fft_c2r_3d_from(Context &ctx, T *dst, const T *src, int n, double scale, const T *pre_tab, const CellBox *box) {
  using C = typename Cx<T>::type;
  if (n < 2 || n % 2) fail(GIC_ERR_INVALID_ARG, "FFT size must be even");
  if (!fft_prunes(ctx, n)) {
    // runtime-length passes: copy, then transform in place
    GIC_CUDA(cudaMemcpyAsync(dst, src, (size_t)n * n * (n / 2 + 1) * sizeof(C), cudaMemcpyDeviceToDevice, ctx.stream));
    fft_c2r_3d<T>(ctx, dst, n, scale, pre_tab, box);
    return;
  }
  const C *tw = (const C *)ctx.fft.get(n, sizeof(T) == 8, ctx.stream);
  C *d = reinterpret_cast<C *>(dst);
  const C *s = reinterpret_cast<const C *>(src);
  long long mirror_threads = 2ll * n * n;
  k_mirror_from<T><<<(unsigned)((mirror_threads + 255) / 256), 256, 0, ctx.stream>>>(d, s, n);
  launched();
  fixed_dispatch<T>(ctx, d, n, tw, scale, true, pre_tab, box, s);
}

template void fft_c2r_3d_from<float>(Context &, float *, const float *, int, double, const float *, const CellBox *);
template void fft_c2r_3d_from<double>(Context &, double *, const double *, int, double, const double *,
                                      const CellBox *);
template void fft_c2r_3d<float>(Context &, float *, int, double, const float *, const CellBox *);
template void fft_c2r_3d<double>(Context &, double *, int, double, const double *, const CellBox *);
template void fft_r2c_3d<float>(Context &, float *, int, double, const float *, const CellBox *);
template void fft_r2c_3d<double>(Context &, double *, int, double, const double *, const CellBox *);

}  // namespace gic
