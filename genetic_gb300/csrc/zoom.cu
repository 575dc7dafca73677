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

template <typename T>
__global__ void k_interp_add4(const T *__restrict__ c0, const T *__restrict__ c1, const T *__restrict__ c2,
                              const T *__restrict__ c3, int nc, double dxc, double ox, double oy, double oz,
                              double period, int wrap, T *f0, T *f1, T *f2, T *f3, int nf, double dxf, double fx,
                              double fy, double fz) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t m = (size_t)nf * nf * nf;
  if (i >= m) return;
  size_t row = i / nf;
  int z = (int)(i % nf), y = (int)(row % nf), x = (int)(row / nf);
  double loc[3] = {(double)x * dxf + fx + dxf / 2 - ox, (double)y * dxf + fy + dxf / 2 - oy,
                   (double)z * dxf + fz + dxf / 2 - oz};
  int base[3];
  T w[3][4];
  for (int a = 0; a < 3; ++a) {
    double l = wrap_coord(loc[a], period);
    double u = l / dxc - 0.5;
    double f = floor(u);
    base[a] = (int)f;
    catmull_rom<T>((T)(u - f), w[a]);
  }
  int ix[4], iy[4], iz[4];
  for (int a = 0; a < 4; ++a) {
    int vx = base[0] - 1 + a, vy = base[1] - 1 + a, vz = base[2] - 1 + a;
    if (wrap) {
      vx = (vx % nc + nc) % nc;
      vy = (vy % nc + nc) % nc;
      vz = (vz % nc + nc) % nc;
    } else {
      vx = min(max(vx, 0), nc - 1);
      vy = min(max(vy, 0), nc - 1);
      vz = min(max(vz, 0), nc - 1);
    }
    ix[a] = vx;
    iy[a] = vy;
    iz[a] = vz;
  }
  const size_t rs = (size_t)(2 * (nc / 2 + 1));
  T s0 = 0, s1 = 0, s2 = 0, s3 = 0;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    T p0 = 0, p1 = 0, p2 = 0, p3 = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      size_t rowi = ((size_t)ix[a] * nc + iy[b]) * rs;
      T q0 = 0, q1 = 0, q2 = 0, q3 = 0;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        size_t k = rowi + iz[c];
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
  k_interp_add4<T><<<(unsigned)((m + 255) / 256), 256, 0, ctx.stream>>>(
      src[0], src[1], src[2], src[3], coarse.n, coarse.dx, coarse.x0[0], coarse.x0[1], coarse.x0[2], coarse.periodic,
      wrap, fine.field[0].as<T>(), fine.field[1].as<T>(), fine.field[2].as<T>(), fine.field[3].as<T>(), fine.n,
      fine.dx, fine.x0[0], fine.x0[1], fine.x0[2]);
  launched();
}

template void interp_add4<float>(Context &, const Level &, float *const[4], Level &);
template void interp_add4<double>(Context &, const Level &, double *const[4], Level &);

}  // namespace gic
