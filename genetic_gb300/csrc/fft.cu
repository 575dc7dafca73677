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
#include <cmath>
#include <algorithm>

namespace gic {
namespace {

template <typename T> struct Cx;
template <> struct Cx<float> { using type = float2; };
template <> struct Cx<double> { using type = double2; };

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
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
                                              int ns_log, int sign, const typename Cx<T>::type *tw, T scale) {
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
        for (int r = 0; r < R; ++r) gout[(size_t)(d + r * Ns) * (size_t)B + c] = cscale(v[r], scale);
      }
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) dst[(d + r * Ns) * TC + c] = v[r];
    }
  }
}

template <typename T, int TC>
__global__ void __launch_bounds__(256) k_fft_strided(typename Cx<T>::type *data, int L, long long B,
                                                     Radix plan, int sign, const typename Cx<T>::type *tw,
                                                     T scale) {
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
  C *src = buf0, *dst = buf1;
  int Ns = 1, ns_log = 0;
  for (int s = 0; s < plan.n; ++s) {
    int R = plan.r[s];
    C *g = (s == plan.n - 1) ? base : nullptr;
    if (R == 8) strided_stage<T, 8, TC>(src, dst, g, B, tcv, L, Ns, ns_log, sign, tw, scale);
    else if (R == 4) strided_stage<T, 4, TC>(src, dst, g, B, tcv, L, Ns, ns_log, sign, tw, scale);
    else if (R == 2) strided_stage<T, 2, TC>(src, dst, g, B, tcv, L, Ns, ns_log, sign, tw, scale);
    else strided_stage<T, 3, TC>(src, dst, g, B, tcv, L, Ns, ns_log, sign, tw, scale);
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

template <typename T>
void set_smem(const void *fn, size_t bytes) {
  static size_t current = 0;
  (void)current;
  GIC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
}

template <typename T>
void strided_pass(Context &ctx, typename Cx<T>::type *data, int A, int L, long long B, int sign, T scale,
                  const typename Cx<T>::type *tw) {
  constexpr int TC = sizeof(T) == 4 ? 8 : 4;
  Radix plan = make_plan(L);
  size_t smem = 2ull * L * TC * sizeof(typename Cx<T>::type);
  set_smem<T>((const void *)k_fft_strided<T, TC>, smem);
  dim3 grid((unsigned)((B + TC - 1) / TC), (unsigned)A);
  k_fft_strided<T, TC><<<grid, 256, smem, ctx.stream>>>(data, L, B, plan, sign, tw, scale);
  launched();
}

template <typename T>
int rows_per_cta(int N) {
  size_t row_bytes = (size_t)(N / 2 + 1) * sizeof(typename Cx<T>::type);
  int rpc = (int)std::max<size_t>(1, 16384 / row_bytes);
  return std::min(rpc, 32);
}

}  // namespace

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
void fft_c2r_3d(Context &ctx, T *data, int n, double scale) {
  using C = typename Cx<T>::type;
  if (n < 2 || n % 2) fail(GIC_ERR_INVALID_ARG, "FFT size must be even");
  const C *tw = (const C *)ctx.fft.get(n, sizeof(T) == 8, ctx.stream);
  C *c = reinterpret_cast<C *>(data);
  long long S = n / 2 + 1;
  long long mirror_threads = 2ll * n * n;
  k_mirror<T><<<(unsigned)((mirror_threads + 255) / 256), 256, 0, ctx.stream>>>(c, n);
  launched();
  strided_pass<T>(ctx, c, 1, n, (long long)n * S, +1, (T)1, tw);
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
void fft_r2c_3d(Context &ctx, T *data, int n, double scale) {
  using C = typename Cx<T>::type;
  if (n < 2 || n % 2) fail(GIC_ERR_INVALID_ARG, "FFT size must be even");
  const C *tw = (const C *)ctx.fft.get(n, sizeof(T) == 8, ctx.stream);
  C *c = reinterpret_cast<C *>(data);
  long long S = n / 2 + 1;
  int rpc = rows_per_cta<T>(n);
  Radix plan = make_plan(n / 2);
  size_t smem = 2ull * rpc * S * sizeof(C);
  set_smem<T>((const void *)k_fft_rows_r2c<T>, smem);
  long long nrows = (long long)n * n;
  k_fft_rows_r2c<T><<<(unsigned)((nrows + rpc - 1) / rpc), 256, smem, ctx.stream>>>(c, nrows, n, rpc, plan, tw,
                                                                                   (T)1);
  launched();
  strided_pass<T>(ctx, c, n, n, S, -1, (T)1, tw);
  strided_pass<T>(ctx, c, 1, n, (long long)n * S, -1, (T)scale, tw);
}

template void fft_c2r_3d<float>(Context &, float *, int, double);
template void fft_c2r_3d<double>(Context &, double *, int, double);
template void fft_r2c_3d<float>(Context &, float *, int, double);
template void fft_r2c_3d<double>(Context &, double *, int, double);

}  // namespace gic
