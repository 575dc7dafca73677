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
                              double dxc, double period, int *base, T *frac) {
  int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= 3 * nf) return;
  int a = id / nf, x = id % nf;
  double fo = a == 0 ? f0 : (a == 1 ? f1 : f2);
  double co = a == 0 ? o0 : (a == 1 ? o1 : o2);
  double l = wrap_coord((double)x * dxf + fo + dxf / 2 - co, period);
  double u = l / dxc - 0.5;
  double f = floor(u);
  base[id] = (int)f;
  frac[id] = (T)(u - f);
}

template <typename T>
__global__ void __launch_bounds__(256) k_interp_add4(const T *__restrict__ c0, const T *__restrict__ c1,
                                                     const T *__restrict__ c2, const T *__restrict__ c3, int nc,
                                                     int wrap, const int *__restrict__ base,
                                                     const T *__restrict__ frac, T *f0, T *f1, T *f2, T *f3,
                                                     int nf) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t m = (size_t)nf * nf * nf;
  if (i >= m) return;
  size_t row = i / nf;
  int z = (int)(i % nf), y = (int)(row % nf), x = (int)(row / nf);
  int pos[3] = {x, y, z};
  T w[3][4];
  int idx[3][4];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    catmull_rom<T>(__ldg(frac + a * nf + pos[a]), w[a]);
    int b0 = __ldg(base + a * nf + pos[a]);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int v = b0 - 1 + c;
      if (wrap) {
        v = v < 0 ? v + nc : (v >= nc ? v - nc : v);
      } else {
        v = min(max(v, 0), nc - 1);
      }
      idx[a][c] = v;
    }
  }
  const size_t rs = (size_t)(2 * (nc / 2 + 1));
  T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    T p0 = 0, p1 = 0, p2 = 0, p3 = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      size_t rowi = ((size_t)idx[0][a] * nc + idx[1][b]) * rs;
      T q0 = 0, q1 = 0, q2 = 0, q3 = 0;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        size_t k = rowi + idx[2][c];
        T wc = w[2][c];
        q0 += wc * __ldg(c0 + k);
        q1 += wc * __ldg(c1 + k);
        q2 += wc * __ldg(c2 + k);
        q3 += wc * __ldg(c3 + k);
      }
      T wb = w[1][b];
      p0 += wb * q0;
      p1 += wb * q1;
      p2 += wb * q2;
      p3 += wb * q3;
    }
    T wa = w[0][a];
    s0 += wa * p0;
    s1 += wa * p1;
    s2 += wa * p2;
    s3 += wa * p3;
  }
  size_t dst = row * (size_t)(2 * (nf / 2 + 1)) + z;
  f0[dst] += s0;
  f1[dst] += s1;
  f2[dst] += s2;
  f3[dst] += s3;
}

}  // namespace

template <typename T>
void interp_add4(Context &ctx, const Level &coarse, T *const src[4], Level &fine) {
  size_t m = fine.ncells();
  int wrap = (coarse.box == coarse.periodic) ? 1 : 0;
  int nf = fine.n;
  ctx.geom.ensure(3 * (size_t)nf * (sizeof(int) + sizeof(T)));
  int *base = ctx.geom.as<int>();
  T *frac = reinterpret_cast<T *>(base + 3 * nf);
  k_interp_axes<T><<<(3 * nf + 127) / 128, 128, 0, ctx.stream>>>(nf, fine.dx, fine.x0[0], fine.x0[1], fine.x0[2],
                                                                coarse.x0[0], coarse.x0[1], coarse.x0[2], coarse.dx,
                                                                coarse.periodic, base, frac);
  k_interp_add4<T><<<(unsigned)((m + 255) / 256), 256, 0, ctx.stream>>>(
      src[0], src[1], src[2], src[3], coarse.n, wrap, base, frac, fine.field[0].as<T>(), fine.field[1].as<T>(),
      fine.field[2].as<T>(), fine.field[3].as<T>(), nf);
  launched(2);
}

template void interp_add4<float>(Context &, const Level &, float *const[4], Level &);
template void interp_add4<double>(Context &, const Level &, double *const[4], Level &);

}  // namespace gic
