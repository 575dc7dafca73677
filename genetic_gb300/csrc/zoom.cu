// Zoom-level combination (genetIC/src/simulation/particles/multilevelgenerator.hpp:104-124,
// genetIC/src/simulation/field/field.hpp:816-831 with FILTER_ON_COARSE_GRID):
// on level l >= 1 the fine fields keep only their high-pass part (applied in the
// fused k-space kernel), and the low-pass-filtered fields of level l-1, in real
// space, are interpolated onto every fine cell and added.
//
// Interpolation (field.hpp:483-509, 598-617; tools/numerics/tricubic.hpp): the 4^3
// coarse cells around the fine centroid define a tricubic whose derivatives are
// central differences -- the tensor product of 1-D Catmull-Rom cubics, so the
// value is sum_abc w_a(tx) w_b(ty) w_c(tz) F[i0-1+a][j0-1+b][k0-1+c].  Indices
// wrap when the coarse grid is the periodic base grid and clamp otherwise.
// One thread per fine cell does all four fields (delta, psi_x, psi_y, psi_z).
#include "gic_internal.h"
#include <atomic>
#include <cmath>

namespace gic {
namespace {

template <typename T>
__device__ __forceinline__ void catmull_rom(T t, T (&w)[4]) {
  T t2 = t * t, t3 = t2 * t;
  w[0] = -(t - 1) * (t - 1) * t / 2;
  w[1] = (2 - 5 * t2 + 3 * t3) / 2;
  w[2] = t * (1 + 4 * t - 3 * t2) / 2;
  w[3] = (t - 1) * t2 / 2;
}

__device__ __forceinline__ double wrap_coord(double x, double period) {
  x = fmod(x, period);
  if (x < 0) x += period;
  return x;
}

// Per axis and fine index: first stencil cell i0 - 1 (wrapped or clamped later)
// and the fractional offset t of the fine centroid, evaluated in double once
// per grid line (field.hpp:483-500): loc = centroid - coarse offset, wrapped into
// the periodic domain; u = loc / dx_coarse - 0.5; i0 = floor(u); t = u - i0.
template <typename T>
__global__ void k_interp_axes(int nf, double dxf, double f0, double f1, double f2, double o0, double o1, double o2,
                              double dxc, double period, int nc, int *base, T *frac, int *ubase) {
  int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= 3 * nf) return;
  int a = id / nf, x = id % nf;
  double fo = a == 0 ? f0 : (a == 1 ? f1 : f2);
  double co = a == 0 ? o0 : (a == 1 ? o1 : o2);
  double lu = (double)x * dxf + fo + dxf / 2 - co;
  double l = wrap_coord(lu, period);
  double u = l / dxc - 0.5;
  double f = floor(u);
  base[id] = (int)f;
  frac[id] = (T)(u - f);
  // the same base counted from the unwrapped position: monotonic along the axis
  ubase[id] = (int)f + (int)floor(lu / period) * nc;
}

template <typename T, int NF>
struct FieldPtrs {
  const T *src[NF];
  T *dst[NF];
  int assign;  // 1: dst = interpolation (dst need not be initialised), 0: dst += it
};

// Direct form (any geometry): one thread per fine cell, 64 coarse values per field.
template <typename T, int NF>
__global__ void __launch_bounds__(256) k_interp_add_direct(FieldPtrs<T, NF> fp, int nc, int wrap,
                                                           const int *__restrict__ base, const T *__restrict__ frac,
                                                           int nf) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t m = (size_t)nf * nf * nf;
  if (i >= m) return;
  size_t row = i / nf;
  int pos[3] = {(int)(row / nf), (int)(row % nf), (int)(i % nf)};
  T w[3][4];
  int idx[3][4];
  for (int a = 0; a < 3; ++a) {
    catmull_rom<T>(__ldg(frac + a * nf + pos[a]), w[a]);
    int b0 = __ldg(base + a * nf + pos[a]);
    for (int c = 0; c < 4; ++c) {
      int v = b0 - 1 + c;
      idx[a][c] = wrap ? ((v % nc) + nc) % nc : min(max(v, 0), nc - 1);
    }
  }
  const size_t rs = (size_t)(2 * (nc / 2 + 1));
  T s[NF];
  for (int f = 0; f < NF; ++f) s[f] = 0;
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) {
      size_t rowi = ((size_t)idx[0][a] * nc + idx[1][b]) * rs;
      for (int c = 0; c < 4; ++c) {
        T wt = w[0][a] * w[1][b] * w[2][c];
        for (int f = 0; f < NF; ++f) s[f] += wt * __ldg(fp.src[f] + rowi + idx[2][c]);
      }
    }
  size_t dst = row * (size_t)(2 * (nf / 2 + 1)) + pos[2];
  for (int f = 0; f < NF; ++f) fp.dst[f][dst] = fp.assign ? s[f] : fp.dst[f][dst] + s[f];
}

// Separable form: a CTA owns one fine x plane and TY fine y rows.  Three contractions,
// each done once: the four coarse x planes of the stencil into P[cy][cz], then z into
// Q[cy][z] = sum_c wz_c(z) P[cy][pz(z) + c] for every coarse row cy of the block and
// fine z, then every fine (y, z) is sum_b wy_b(y) Q[py(y) + b][z].  The sums run in the
// order of the direct 4 x 4 contraction of P, so the values are the same.
template <typename T, int NF, int TY>
__global__ void __launch_bounds__(256) k_interp_add_sep(FieldPtrs<T, NF> fp, int nc, int wrap,
                                                        const int *__restrict__ base, const T *__restrict__ frac,
                                                        const int *__restrict__ ubase, int nf, int maxcz, int maxcy) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T *P = reinterpret_cast<T *>(smraw);
  const int x = blockIdx.y;
  const int y0 = blockIdx.x * TY;
  const int ylast = min(y0 + TY, nf) - 1;
  auto cw = [&](int v) { return wrap ? ((v % nc) + nc) % nc : min(max(v, 0), nc - 1); };
  T wx[4];
  catmull_rom<T>(__ldg(frac + x), wx);
  int ixw[4];
  int bx = __ldg(base + x);
#pragma unroll
  for (int a = 0; a < 4; ++a) ixw[a] = cw(bx - 1 + a);
  const int cy0 = __ldg(ubase + nf + y0) - 1;
  const int ny = min(__ldg(ubase + nf + ylast) + 3 - cy0, maxcy);
  const int cz0 = __ldg(ubase + 2 * nf) - 1;
  const int nz = min(__ldg(ubase + 2 * nf + nf - 1) + 3 - cz0, maxcz);
  T *Q = P + (size_t)NF * maxcy * maxcz;  // [NF][maxcy][nf]
  const size_t rs = (size_t)(2 * (nc / 2 + 1));
  const int tile = ny * nz;
  // cw without a division for the indices within one period of the grid
  auto cwf = [&](int v) {
    if (!wrap) return min(max(v, 0), nc - 1);
    if (v >= 0 && v < nc) return v;
    if (v < 0 && v >= -nc) return v + nc;
    if (v >= nc && v < 2 * nc) return v - nc;
    return ((v % nc) + nc) % nc;
  };
  // a warp per coarse row of the tile, its lanes along z
  const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31), nwarps = (int)(blockDim.x >> 5);
  for (int cyi = warp; cyi < ny; cyi += nwarps) {
    const int cy = cwf(cy0 + cyi);
    size_t k0[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) k0[a] = ((size_t)ixw[a] * nc + cy) * rs;
    for (int czi = lane; czi < nz; czi += 32) {
      const int cz = cwf(cz0 + czi);
      T v[NF];
#pragma unroll
      for (int f = 0; f < NF; ++f) v[f] = 0;
#pragma unroll
      for (int a = 0; a < 4; ++a) {
#pragma unroll
        for (int f = 0; f < NF; ++f) v[f] += wx[a] * __ldg(fp.src[f] + k0[a] + cz);
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) P[f * tile + cyi * nz + czi] = v[f];
    }
  }
  __shared__ T wys[TY][4];
  __shared__ int pys[TY];
  for (int r = threadIdx.x; r <= ylast - y0; r += blockDim.x) {
    catmull_rom<T>(__ldg(frac + nf + y0 + r), wys[r]);
    pys[r] = __ldg(ubase + nf + y0 + r) - 1 - cy0;
  }
  __syncthreads();
  for (int z = threadIdx.x; z < nf; z += blockDim.x) {
    T wz[4];
    catmull_rom<T>(__ldg(frac + 2 * nf + z), wz);
    const int pz = __ldg(ubase + 2 * nf + z) - 1 - cz0;
    for (int cy = 0; cy < ny; ++cy) {
      const int rowp = cy * nz + pz;
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        T q = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) q += wz[c] * P[f * tile + rowp + c];
        Q[((size_t)f * maxcy + cy) * nf + z] = q;
      }
    }
  }
  __syncthreads();
  const size_t frs = (size_t)(2 * (nf / 2 + 1));
  // fine cells: a thread owns z columns and walks the block's rows U at a time, their
  // destination loads issued before the sums (the read-modify-write is otherwise
  // latency-bound); the rows' y weights come from shared memory
  constexpr int U = 4;
  const int nrows = ylast - y0 + 1;
  for (int z = threadIdx.x; z < nf; z += blockDim.x) {
    for (int r0 = 0; r0 < nrows; r0 += U) {
      T cur[U][NF];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const size_t at = ((size_t)x * nf + (y0 + r0 + u)) * frs + z;
#pragma unroll
        for (int f = 0; f < NF; ++f) cur[u][f] = (r0 + u < nrows && !fp.assign) ? fp.dst[f][at] : (T)0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int r = r0 + u;
        if (r >= nrows) break;
        const int py = pys[r];
        T s[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) s[f] = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
#pragma unroll
          for (int f = 0; f < NF; ++f) s[f] += wys[r][b] * Q[((size_t)f * maxcy + py + b) * nf + z];
        }
        const size_t at = ((size_t)x * nf + (y0 + r)) * frs + z;
#pragma unroll
        for (int f = 0; f < NF; ++f) fp.dst[f][at] = fp.assign ? s[f] : cur[u][f] + s[f];
      }
    }
  }
}

// The same with the direct 4 x 4 contraction of P per fine cell (smaller shared memory:
// P only), for geometries whose Q does not fit.
template <typename T, int NF, int TY>
__global__ void __launch_bounds__(256) k_interp_add_tile(FieldPtrs<T, NF> fp, int nc, int wrap,
                                                        const int *__restrict__ base, const T *__restrict__ frac,
                                                        const int *__restrict__ ubase, int nf, int maxcz) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T *P = reinterpret_cast<T *>(smraw);
  const int x = blockIdx.y;
  const int y0 = blockIdx.x * TY;
  const int ylast = min(y0 + TY, nf) - 1;
  auto cw = [&](int v) { return wrap ? ((v % nc) + nc) % nc : min(max(v, 0), nc - 1); };
  T wx[4];
  catmull_rom<T>(__ldg(frac + x), wx);
  int ixw[4];
  int bx = __ldg(base + x);
#pragma unroll
  for (int a = 0; a < 4; ++a) ixw[a] = cw(bx - 1 + a);
  const int cy0 = __ldg(ubase + nf + y0) - 1;
  const int ny = __ldg(ubase + nf + ylast) + 3 - cy0;
  const int cz0 = __ldg(ubase + 2 * nf) - 1;
  const int nz = min(__ldg(ubase + 2 * nf + nf - 1) + 3 - cz0, maxcz);
  const size_t rs = (size_t)(2 * (nc / 2 + 1));
  const int tile = ny * nz;
  for (int e = threadIdx.x; e < tile; e += blockDim.x) {
    int cy = cw(cy0 + e / nz), cz = cw(cz0 + e % nz);
    T v[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) v[f] = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      size_t k = ((size_t)ixw[a] * nc + cy) * rs + cz;
#pragma unroll
      for (int f = 0; f < NF; ++f) v[f] += wx[a] * __ldg(fp.src[f] + k);
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) P[f * tile + e] = v[f];
  }
  __syncthreads();
  const size_t frs = (size_t)(2 * (nf / 2 + 1));
  const int cnt = (ylast - y0 + 1) * nf;
  for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
    int y = y0 + e / nf, z = e % nf;
    T wy[4], wz[4];
    catmull_rom<T>(__ldg(frac + nf + y), wy);
    catmull_rom<T>(__ldg(frac + 2 * nf + z), wz);
    int py = __ldg(ubase + nf + y) - 1 - cy0;
    int pz = __ldg(ubase + 2 * nf + z) - 1 - cz0;
    T s[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) s[f] = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      int rowp = (py + b) * nz + pz;
      T q[NF];
#pragma unroll
      for (int f = 0; f < NF; ++f) q[f] = 0;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
#pragma unroll
        for (int f = 0; f < NF; ++f) q[f] += wz[c] * P[f * tile + rowp + c];
      }
#pragma unroll
      for (int f = 0; f < NF; ++f) s[f] += wy[b] * q[f];
    }
    size_t dst = ((size_t)x * nf + y) * frs + z;
#pragma unroll
    for (int f = 0; f < NF; ++f) fp.dst[f][dst] = fp.assign ? s[f] : fp.dst[f][dst] + s[f];
  }
}

}  // namespace

// Add the tricubic interpolation of NF real fields of grid `coarse` onto the
// NF real fields of grid `fine` (any two levels, coarse cells larger).
template <typename T, int NF>
void interp_add(Context &ctx, const Level &coarse, const T *const *src, const Level &fine, T *const *dst, bool assign) {
  size_t m = fine.ncells();
  int wrap = (coarse.box == coarse.periodic) ? 1 : 0;
  int nf = fine.n;
  ctx.geom.ensure(3 * (size_t)nf * (2 * sizeof(int) + sizeof(T)));
  int *base = ctx.geom.as<int>();
  int *ubase = base + 3 * nf;
  T *frac = reinterpret_cast<T *>(ubase + 3 * nf);
  k_interp_axes<T><<<(3 * nf + 127) / 128, 128, 0, ctx.stream>>>(nf, fine.dx, fine.x0[0], fine.x0[1], fine.x0[2],
                                                                coarse.x0[0], coarse.x0[1], coarse.x0[2], coarse.dx,
                                                                coarse.periodic, coarse.n, base, frac, ubase);
  launched();
  double ratio = fine.dx / coarse.dx;
  int span = (int)std::ceil(nf * ratio) + 6;
  // fine rows per CTA: more rows amortise the coarse contractions, within 96 KB of P and Q
  constexpr int TY = NF == 1 ? 32 : 16;
  int ny = (int)std::ceil(TY * ratio) + 6;
  size_t smem = (size_t)NF * ny * ((size_t)span + nf) * sizeof(T);
  FieldPtrs<T, NF> fp;
  fp.assign = assign ? 1 : 0;
  for (int f = 0; f < NF; ++f) {
    fp.src[f] = src[f];
    fp.dst[f] = dst[f];
  }
  if (ratio <= 1.0 && smem <= 96 * 1024) {
    // raise the kernel's shared-memory limit to the 96 KB ceiling once per device
    static std::atomic<int> mask{0};
    int dev = 0;
    GIC_CUDA(cudaGetDevice(&dev));
    if (!(mask.load() & (1 << (dev & 31)))) {
      GIC_CUDA(cudaFuncSetAttribute((const void *)k_interp_add_sep<T, NF, TY>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
      mask.fetch_or(1 << (dev & 31));
    }
    dim3 grid((nf + TY - 1) / TY, nf);
    k_interp_add_sep<T, NF, TY><<<grid, 256, smem, ctx.stream>>>(fp, coarse.n, wrap, base, frac, ubase, nf, span, ny);
    launched();
  } else if (ratio <= 1.0 && (size_t)NF * ((size_t)std::ceil(8 * ratio) + 6) * span * sizeof(T) <= 96 * 1024) {
    constexpr int TY8 = 8;
    const int ny8 = (int)std::ceil(TY8 * ratio) + 6;
    const size_t smem8 = (size_t)NF * ny8 * span * sizeof(T);
    static std::atomic<int> mask{0};
    int dev = 0;
    GIC_CUDA(cudaGetDevice(&dev));
    if (!(mask.load() & (1 << (dev & 31)))) {
      GIC_CUDA(cudaFuncSetAttribute((const void *)k_interp_add_tile<T, NF, TY8>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
      mask.fetch_or(1 << (dev & 31));
    }
    dim3 grid((nf + TY8 - 1) / TY8, nf);
    k_interp_add_tile<T, NF, TY8><<<grid, 256, smem8, ctx.stream>>>(fp, coarse.n, wrap, base, frac, ubase, nf, span);
    launched();
  } else {
    k_interp_add_direct<T, NF><<<(unsigned)((m + 255) / 256), 256, 0, ctx.stream>>>(fp, coarse.n, wrap, base, frac,
                                                                                   nf);
    launched();
  }
}

// the fields of `mask` (bit f: delta, psi_x, psi_y, psi_z): all four, the three
// displacements, or delta alone
template <typename T>
void interp_add_fields(Context &ctx, const Level &coarse, T *const src[4], Level &fine, unsigned mask) {
  T *dst[4] = {fine.field[0].as<T>(), fine.field[1].as<T>(), fine.field[2].as<T>(), fine.field[3].as<T>()};
  const T *s[4] = {src[0], src[1], src[2], src[3]};
  if (mask == 15u) interp_add<T, 4>(ctx, coarse, s, fine, dst);
  else if (mask == 14u) interp_add<T, 3>(ctx, coarse, s + 1, fine, dst + 1);
  else if (mask == 1u) interp_add<T, 1>(ctx, coarse, s, fine, dst);
  else fail(GIC_ERR_INTERNAL, "unsupported field mask for the zoom interpolation");
}

template void interp_add_fields<float>(Context &, const Level &, float *const[4], Level &, unsigned);
template void interp_add_fields<double>(Context &, const Level &, double *const[4], Level &, unsigned);
template void interp_add<float, 1>(Context &, const Level &, const float *const *, const Level &, float *const *, bool);
template void interp_add<double, 1>(Context &, const Level &, const double *const *, const Level &, double *const *, bool);
template void interp_add<float, 3>(Context &, const Level &, const float *const *, const Level &, float *const *, bool);
template void interp_add<double, 3>(Context &, const Level &, const double *const *, const Level &, double *const *, bool);

}  // namespace gic
