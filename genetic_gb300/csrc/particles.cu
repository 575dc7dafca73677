// Zel'dovich (and 2LPT) particles of one level: position = cell centroid + psi, wrapped
// into the periodic domain, velocity = psi * 100 sqrt(Om/a^3 + OL) sqrt(a)
// (f = 1), as ZeldovichParticleEvaluator evaluates them one index at a time
// (genetIC/src/simulation/particles/zeldovich.hpp:87-124,
//  genetIC/src/cosmology/parameters.hpp:84-106, generator.hpp:49-53,
//  grid.hpp:659-669 centroid, grid.hpp:519-531 wrap).
// Here every cell of the level is evaluated in one pass over the three
// real-space displacement fields: positions in double, velocities in the
// working precision.
#include "gic_internal.h"
#include <cstring>
#include <cmath>

namespace gic {
namespace {

// fmod(x, period) then + period if negative, as grid.hpp:527-531; for
// -period < x < 2 period this equals the branch below exactly (x - period is
// exact there), which avoids a double-precision remainder per coordinate.
__device__ __forceinline__ double wrap_coord(double x, double period) {
  if (x >= period && x < 2 * period) return x - period;
  if (x < 0 && x > -period) return x + period;
  if (x >= 0 && x < period) return x;
  x = fmod(x, period);
  if (x < 0) x += period;
  return x;
}

// cell centroids along one axis: coord * dx + offset + dx / 2 (grid.hpp:659-669)
__global__ void k_centroids(int n, double dx, double x0, double y0, double z0, double *c) {
  int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= 3 * n) return;
  int a = id / n, i = id % n;
  double o = a == 0 ? x0 : (a == 1 ? y0 : z0);
  c[id] = (double)i * dx + o + dx / 2;
}

// float -> double by bit manipulation (exact; keeps the conversion off the
// double-precision pipe).  Zero and subnormal floats map to (signed) zero
// scaled exactly; inf/nan keep their class.
__device__ __forceinline__ double f2d_bits(float f) {
  unsigned u = __float_as_uint(f);
  unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  unsigned e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  if (e == 0) {
    if (m == 0) return __longlong_as_double((long long)sign);
    // subnormal float: normalise
    int sh = __clz(m) - 8;
    m = (m << sh) & 0x7FFFFFu;
    unsigned long long ed = (unsigned long long)(1 - 127 - sh + 1023);
    return __longlong_as_double((long long)(sign | (ed << 52) | ((unsigned long long)m << 29)));
  }
  unsigned long long ed = e == 0xFFu ? 0x7FFull : (unsigned long long)(e - 127 + 1023);
  return __longlong_as_double((long long)(sign | (ed << 52) | ((unsigned long long)m << 29)));
}

__device__ __forceinline__ double to_double(float v) { return f2d_bits(v); }
__device__ __forceinline__ double to_double(double v) { return v; }

// wrap_coord with the common in-range case decided by integer compares on the
// bit patterns (non-negative doubles order like their bits)
__device__ __forceinline__ double wrap_fast(double x, double period, long long period_bits) {
  long long b = __double_as_longlong(x);
  if (b >= 0 && b < period_bits) return x;  // 0 <= x < period (and x != -0)
  return wrap_coord(x, period);
}

// LPT2: second-order displacements q2 are added, pos = q + psi + psi2 and
// vel = ratio (psi + 2 psi2) (f2 = 2 with genetIC's f = 1).
// A CTA per row (x, y) of n cells, 256 of them at a time: each thread evaluates one
// particle into shared memory, then the CTA writes the 256 particles' positions and
// velocities as contiguous runs (3 components per particle, interleaved).
template <typename T, bool LPT2>
__global__ void __launch_bounds__(256) k_particles(const T *__restrict__ px, const T *__restrict__ py,
                                                   const T *__restrict__ pz, const T *__restrict__ qx,
                                                   const T *__restrict__ qy, const T *__restrict__ qz, int n,
                                                   const double *__restrict__ cen, double period, T ratio,
                                                   double *pos, T *vel) {
  __shared__ double sp[3 * 256];
  __shared__ T sv[3 * 256];
  const unsigned row = blockIdx.x;
  const int x = (int)(row / (unsigned)n), y = (int)(row - (unsigned)x * (unsigned)n);
  const size_t src_row = (size_t)row * (size_t)(2 * (n / 2 + 1));
  const double cx = __ldg(cen + x), cy = __ldg(cen + n + y);
  const long long pb = __double_as_longlong(period);
  const int t = threadIdx.x;
  for (int z0 = 0; z0 < n; z0 += 256) {
    const int z = z0 + t;
    if (z < n) {
      const size_t src = src_row + z;
      T sx = px[src], sy = py[src], sz = pz[src];
      if (LPT2) {
        T tx = qx[src], ty = qy[src], tz = qz[src];
        sv[3 * t + 0] = (sx + 2 * tx) * ratio;
        sv[3 * t + 1] = (sy + 2 * ty) * ratio;
        sv[3 * t + 2] = (sz + 2 * tz) * ratio;
        sx += tx;
        sy += ty;
        sz += tz;
      } else {
        sv[3 * t + 0] = sx * ratio;
        sv[3 * t + 1] = sy * ratio;
        sv[3 * t + 2] = sz * ratio;
      }
      sp[3 * t + 0] = wrap_fast(to_double(sx) + cx, period, pb);
      sp[3 * t + 1] = wrap_fast(to_double(sy) + cy, period, pb);
      sp[3 * t + 2] = wrap_fast(to_double(sz) + __ldg(cen + 2 * n + z), period, pb);
    }
    __syncthreads();
    const size_t o = 3 * ((size_t)row * n + z0);
    const int cnt = 3 * min(256, n - z0);
    for (int e = t; e < cnt; e += 256) {
      pos[o + e] = sp[e];
      vel[o + e] = sv[e];
    }
    __syncthreads();
  }
}

// The mean of each s^3 block of a level's real field (SubSampleEvaluator,
// genetIC/src/simulation/field/evaluator.hpp:180-207 with SubSampleGrid::forEachSubcell,
// genetIC/src/simulation/grid/virtualgrid.hpp:576-605: the sum over x, then y, then z,
// divided by the count) into an (n/s)^3 field; both in the padded real layout.
template <typename T>
__global__ void k_block_average(const T *__restrict__ src, int n, int s, T *__restrict__ dst, int nv) {
  const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (size_t)nv * nv * nv) return;
  const int z = (int)(id % nv);
  const size_t r = id / nv;
  const int y = (int)(r % nv), x = (int)(r / nv);
  const size_t srow = 2 * (size_t)(n / 2 + 1);
  T acc = 0;
  for (int i = 0; i < s; ++i)
    for (int j = 0; j < s; ++j)
      for (int k = 0; k < s; ++k) acc += src[((size_t)(x * s + i) * n + (y * s + j)) * srow + (size_t)(z * s + k)];
  dst[((size_t)x * nv + y) * (2 * (size_t)(nv / 2 + 1)) + z] = acc / (T)(s * s * s);
}

// Geometry of a resolution-matching grid (strays): V is level l's resolution over the
// region of level l-1 (nv cells per side from vx0), the zoom window starts at cell w0 of V
// (cyclic in V, nw cells per side); the coarse level has nc cells of dxc from cx0.
struct Matched {
  int nv, nw, nc, wrap_coarse;
  int w0[3];
  double dxv, vx0[3], dxc, cx0[3], period;
};

__device__ __forceinline__ void catmull_rom_w(double t, double (&w)[4]) {
  const double t2 = t * t, t3 = t2 * t;
  w[0] = -(t - 1) * (t - 1) * t / 2;
  w[1] = (2 - 5 * t2 + 3 * t3) / 2;
  w[2] = t * (1 + 4 * t - 3 * t2) / 2;
  w[3] = (t - 1) * t2 / 2;
}

// genetIC's ResolutionMatchingEvaluator (evaluator.hpp:208-256) per requested cell of the
// resolution-matching grid: inside the zoom window the level's own displacement, outside it
// the coarse level's displacement tricubic-interpolated at the cell's centroid (the
// supersampled low-resolution grid, virtualgrid.hpp:250-255; wrapped when the coarse level
// is the periodic base, clamped otherwise).  Position = centroid + displacement, wrapped.
template <typename T>
__global__ void k_matched_particles(const unsigned long long *cells, size_t count, Matched g, const T *fx, const T *fy,
                                    const T *fz, const T *cxf, const T *cyf, const T *czf, T ratio, double *pos,
                                    T *vel) {
  const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= count) return;
  const unsigned long long c = cells[id];
  const int v[3] = {(int)(c / ((unsigned long long)g.nv * g.nv)), (int)((c / g.nv) % g.nv), (int)(c % g.nv)};
  int w[3];
  bool inside = true;
  double cen[3];
  for (int a = 0; a < 3; ++a) {
    w[a] = ((v[a] - g.w0[a]) % g.nv + g.nv) % g.nv;
    inside = inside && w[a] < g.nw;
    cen[a] = (double)v[a] * g.dxv + g.vx0[a] + g.dxv / 2;
  }
  T d[3];
  if (inside) {
    const size_t at = ((size_t)w[0] * g.nw + w[1]) * (size_t)(2 * (g.nw / 2 + 1)) + w[2];
    d[0] = fx[at];
    d[1] = fy[at];
    d[2] = fz[at];
  } else {
    int base[3];
    double wt[3][4];
    for (int a = 0; a < 3; ++a) {
      double l = fmod(cen[a] - g.cx0[a], g.period);
      if (l < 0) l += g.period;
      const double u = l / g.dxc - 0.5, f = floor(u);
      base[a] = (int)f - 1;
      catmull_rom_w(u - f, wt[a]);
    }
    const size_t crow = 2 * (size_t)(g.nc / 2 + 1);
    double acc[3] = {0, 0, 0};
    for (int i = 0; i < 4; ++i) {
      int ix = base[0] + i;
      ix = g.wrap_coarse ? ((ix % g.nc) + g.nc) % g.nc : min(max(ix, 0), g.nc - 1);
      for (int j = 0; j < 4; ++j) {
        int iy = base[1] + j;
        iy = g.wrap_coarse ? ((iy % g.nc) + g.nc) % g.nc : min(max(iy, 0), g.nc - 1);
        const double wij = wt[0][i] * wt[1][j];
        for (int k = 0; k < 4; ++k) {
          int iz = base[2] + k;
          iz = g.wrap_coarse ? ((iz % g.nc) + g.nc) % g.nc : min(max(iz, 0), g.nc - 1);
          const size_t at = ((size_t)ix * g.nc + iy) * crow + iz;
          const double ww = wij * wt[2][k];
          acc[0] += ww * (double)cxf[at];
          acc[1] += ww * (double)cyf[at];
          acc[2] += ww * (double)czf[at];
        }
      }
    }
    for (int a = 0; a < 3; ++a) d[a] = (T)acc[a];
  }
  for (int a = 0; a < 3; ++a) {
    pos[3 * id + a] = wrap_coord((double)d[a] + cen[a], g.period);
    vel[3 * id + a] = d[a] * ratio;
  }
}

template <typename T>
__global__ void k_widen(const T *src, double *dst, size_t count) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dst[i] = to_double(src[i]);
}

}  // namespace

double velocity_to_offset_ratio(const Cosmo &c) {
  double f = 1.0;
  return f * 100. * std::sqrt(c.om / (c.a * c.a * c.a) + c.ol) * std::sqrt(c.a);
}

template <typename T>
static void particles_typed(Context &ctx, Level &L, int order) {
  size_t m = L.ncells();
  // an asynchronous fetch may still be reading the current pair: write the other one, after
  // (on the device) any fetch still reading that
  if (L.fetching) {
    L.pos.swap(L.pos_alt);
    L.vel.swap(L.vel_alt);
    std::swap(L.fetched, L.fetched_alt);
    std::swap(L.fetching, L.fetching_alt);
    if (L.fetching) {
      GIC_CUDA(cudaStreamWaitEvent(ctx.stream, L.fetched, 0));
      L.fetching = false;
    }
  }
  L.pos.ensure(3 * m * sizeof(double));
  L.vel.ensure(3 * m * sizeof(T));
  T ratio = (T)velocity_to_offset_ratio(ctx.cosmo);
  ctx.geom.ensure(3 * (size_t)L.n * sizeof(double));
  double *cen = ctx.geom.as<double>();
  k_centroids<<<(3 * L.n + 127) / 128, 128, 0, ctx.stream>>>(L.n, L.dx, L.x0[0], L.x0[1], L.x0[2], cen);
  const unsigned grid = (unsigned)((size_t)L.n * L.n);  // a CTA per row of cells
  if (order == 2)
    k_particles<T, true><<<grid, 256, 0, ctx.stream>>>(L.field[1].as<T>(), L.field[2].as<T>(), L.field[3].as<T>(),
                                                       L.field2[0].as<T>(), L.field2[1].as<T>(), L.field2[2].as<T>(),
                                                       L.n, cen, L.periodic, ratio, L.pos.as<double>(), L.vel.as<T>());
  else
    k_particles<T, false><<<grid, 256, 0, ctx.stream>>>(L.field[1].as<T>(), L.field[2].as<T>(), L.field[3].as<T>(),
                                                        nullptr, nullptr, nullptr, L.n, cen, L.periodic, ratio,
                                                        L.pos.as<double>(), L.vel.as<T>());
  launched(2);
}

void fetch_particles_async(Context &ctx, Level &L, double *host_pos, void *host_vel) {
  if (!L.pos.ptr || !L.vel.ptr) fail(GIC_ERR_NOT_READY, "particles have not been generated");
  if (!ctx.copy_stream) {
    GIC_CUDA(cudaStreamCreateWithFlags(&ctx.copy_stream, cudaStreamNonBlocking));
    GIC_CUDA(cudaEventCreateWithFlags(&ctx.copy_ready, cudaEventDisableTiming));
  }
  if (!L.fetched) {
    GIC_CUDA(cudaEventCreateWithFlags(&L.fetched, cudaEventDisableTiming));
    GIC_CUDA(cudaEventCreateWithFlags(&L.fetched_alt, cudaEventDisableTiming));
  }
  const size_t m = L.ncells();
  GIC_CUDA(cudaEventRecord(ctx.copy_ready, ctx.stream));
  GIC_CUDA(cudaStreamWaitEvent(ctx.copy_stream, ctx.copy_ready, 0));
  if (host_pos)
    GIC_CUDA(cudaMemcpyAsync(host_pos, L.pos.ptr, 3 * m * sizeof(double), cudaMemcpyDeviceToHost, ctx.copy_stream));
  if (host_vel)
    GIC_CUDA(cudaMemcpyAsync(host_vel, L.vel.ptr, 3 * m * (ctx.dbl() ? sizeof(double) : sizeof(float)),
                             cudaMemcpyDeviceToHost, ctx.copy_stream));
  GIC_CUDA(cudaEventRecord(L.fetched, ctx.copy_stream));
  L.fetching = true;
}

__global__ void k_copy_words(const unsigned *__restrict__ src, unsigned *__restrict__ dst, size_t n) {
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

void read_small(Context &ctx, const void *dev, size_t bytes, void *host) {
  if (bytes == 0) return;
  if (bytes > kReadbackBytes || bytes % 4 || reinterpret_cast<uintptr_t>(dev) % 4) {
    GIC_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx.stream));
    GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    return;
  }
  Context::Mapped &m = ctx.readback;
  if (!m.host) {
    GIC_CUDA(cudaHostAlloc(&m.host, kReadbackBytes, cudaHostAllocMapped));
    if (cudaHostGetDevicePointer(&m.dev, m.host, 0) != cudaSuccess) {
      cudaGetLastError();
      cudaFreeHost(m.host);
      m.host = nullptr;
      fail(GIC_ERR_CUDA, "cudaHostGetDevicePointer failed");
    }
  }
  k_copy_words<<<1, 256, 0, ctx.stream>>>(static_cast<const unsigned *>(dev), static_cast<unsigned *>(m.dev), bytes / 4);
  launched();
  GIC_CUDA(cudaStreamSynchronize(ctx.stream));
  std::memcpy(host, m.host, bytes);
}

void finish_fetches(Context &ctx) {
  if (ctx.copy_stream) GIC_CUDA(cudaStreamSynchronize(ctx.copy_stream));
  for (auto &L : ctx.levels) L->fetching = L->fetching_alt = false;
  ctx.records_pending[0] = ctx.records_pending[1] = false;
}


// genetIC's grafic writer (io/grafic.hpp:160-200, GraficOutput::writeGrid) on one grid of the
// grafic stack: for every cell (x, y, z) of the z-slabs [z0, z0 + nz), the particle of cell
// (x, y, z) - roll of the (virtual) level (CenteredGrid's index map; roll = 0 for the other
// grids), as the writer's floats: velocity * vel_factor, displacement * pos_factor
// (getParticleNoOffset: the displacement, vel = displacement * velocityToOffsetRatio, in
// double), the overdensity, and the cell's id + id_offset; every output [nz][n][n] with x
// fastest, the order of a slab's record.  Sources: padded real fields of n^3.
template <typename T, bool LPT2>
__global__ void k_grafic_slabs(const T *__restrict__ px, const T *__restrict__ py, const T *__restrict__ pz,
                               const T *__restrict__ qx, const T *__restrict__ qy, const T *__restrict__ qz,
                               const T *__restrict__ delta, int n, int z0, int nz, int rx, int ry, int rz, double ratio,
                               double vel_factor, double pos_factor, float *vel, float *pos, float *dlt,
                               unsigned long long *ids, unsigned long long id_offset) {
  const size_t m = (size_t)nz * n * n;
  const size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= m) return;
  const int x = (int)(o % n);
  const size_t r = o / n;
  const int y = (int)(r % n), z = z0 + (int)(r / n);
  const int ux = ((x - rx) % n + n) % n, uy = ((y - ry) % n + n) % n, uz = ((z - rz) % n + n) % n;
  const size_t src = ((size_t)ux * n + uy) * (size_t)(2 * (n / 2 + 1)) + uz;
  if (vel || pos) {
    const T *p[3] = {px, py, pz};
    const T *q[3] = {qx, qy, qz};
    for (int a = 0; a < 3; ++a) {
      T d = p[a][src], v = d;
      if (LPT2) {
        const T e = q[a][src];
        v = d + 2 * e;  // as the particle kernel forms the second-order velocity
        d += e;
      }
      if (vel) vel[a * m + o] = (float)(((double)v * ratio) * vel_factor);
      if (pos) pos[a * m + o] = (float)((double)d * pos_factor);
    }
  }
  if (dlt) dlt[o] = (float)delta[src];
  if (ids) ids[o] = id_offset + ((unsigned long long)ux * n + uy) * (unsigned long long)n + (unsigned long long)uz;
}

// Particles of a virtual grid over level L's region (genetIC's supersample / subsample):
// factor > 1, (n factor)^3 cells whose displacements are the level's interpolated at
// their centroids (SuperSampleEvaluator, evaluator.hpp:96-130: the tricubic of
// field.hpp:483-509, wrapped on the periodic base level, clamped on a zoom level);
// factor < -1, (n / |factor|)^3 cells averaging |factor|^3 cells each.  Positions
// (centroid + displacement, wrapped) and velocities go to host_pos / host_vel (doubles).
template <typename T>
static void resampled_typed(Context &ctx, const Level &L, int factor, double *host_pos, double *host_vel) {
  const bool super = factor > 1;
  const int s = super ? factor : -factor;
  Level V;
  V.n = super ? L.n * s : L.n / s;
  V.box = L.box;
  V.dx = L.box / V.n;
  for (int a = 0; a < 3; ++a) V.x0[a] = L.x0[a];
  V.periodic = L.periodic;
  const size_t real = (size_t)V.n * V.n * 2 * (size_t)(V.n / 2 + 1), m = V.ncells();
  std::unique_ptr<DevBuf> f[3] = {ctx.pool.take(real * sizeof(T)), ctx.pool.take(real * sizeof(T)),
                                  ctx.pool.take(real * sizeof(T))};
  T *dst[3] = {f[0]->as<T>(), f[1]->as<T>(), f[2]->as<T>()};
  if (super) {
    const T *src[3] = {L.field[1].as<T>(), L.field[2].as<T>(), L.field[3].as<T>()};
    interp_add<T, 3>(ctx, L, src, V, dst, true);
  } else {
    for (int a = 0; a < 3; ++a)
      k_block_average<T><<<(unsigned)((m + 255) / 256), 256, 0, ctx.stream>>>(L.field[1 + a].as<T>(), L.n, s, dst[a],
                                                                             V.n);
    launched(3);
  }
  auto pos = ctx.pool.take(3 * m * sizeof(double));
  auto vel = ctx.pool.take(3 * m * sizeof(T));
  auto cen = ctx.pool.take(3 * (size_t)V.n * sizeof(double));
  k_centroids<<<(3 * V.n + 127) / 128, 128, 0, ctx.stream>>>(V.n, V.dx, V.x0[0], V.x0[1], V.x0[2], cen->as<double>());
  k_particles<T, false><<<(unsigned)((size_t)V.n * V.n), 256, 0, ctx.stream>>>(
      dst[0], dst[1], dst[2], nullptr, nullptr, nullptr, V.n, cen->as<double>(), V.periodic,
      (T)velocity_to_offset_ratio(ctx.cosmo), pos->as<double>(), vel->as<T>());
  launched(2);
  GIC_CUDA(cudaMemcpyAsync(host_pos, pos->ptr, 3 * m * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
  if (sizeof(T) == sizeof(double)) {
    GIC_CUDA(cudaMemcpyAsync(host_vel, vel->ptr, 3 * m * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
  } else {
    // widen in the positions' buffer, once they are on the host
    GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    k_widen<T><<<(unsigned)((3 * m + 255) / 256), 256, 0, ctx.stream>>>(vel->as<T>(), pos->as<double>(), 3 * m);
    launched();
    GIC_CUDA(cudaMemcpyAsync(host_vel, pos->ptr, 3 * m * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
  }
  GIC_CUDA(cudaStreamSynchronize(ctx.stream));
  for (auto &b : f) ctx.pool.give(std::move(b));
  ctx.pool.give(std::move(pos));
  ctx.pool.give(std::move(vel));
  ctx.pool.give(std::move(cen));
}


template <typename T>
static void grafic_typed(Context &ctx, int level, const gic_grafic_grid &g, int z0, int nz, float *host_vel,
                         float *host_pos, float *host_delta, unsigned long long *host_ids) {
  Level &L = *ctx.levels[level];
  if (host_delta) ensure_delta(ctx);
  const bool lpt2 = L.have_lpt2;
  const int f = g.factor, s = f > 1 ? f : (f < -1 ? -f : 1);
  const bool super = f > 1, sub = f < -1;
  const int n = super ? L.n * s : (sub ? L.n / s : L.n);
  // the (virtual) grid's padded real fields: delta, psi (and psi2) of level L, interpolated
  // tricubically (supersampled) or averaged over blocks (subsampled) as in particles of those grids
  const int nsrc = lpt2 ? 7 : 4;
  const T *src[7] = {L.field[0].as<T>(), L.field[1].as<T>(), L.field[2].as<T>(), L.field[3].as<T>(),
                     L.field2[0].as<T>(), L.field2[1].as<T>(), L.field2[2].as<T>()};
  std::unique_ptr<DevBuf> virt[7];
  if (super || sub) {
    Level V;
    V.n = n;
    V.box = L.box;
    V.dx = L.box / n;
    for (int a = 0; a < 3; ++a) V.x0[a] = L.x0[a];
    V.periodic = L.periodic;
    const size_t real = (size_t)n * n * 2 * (size_t)(n / 2 + 1), m = V.ncells();
    T *dst[7];
    for (int k = 0; k < nsrc; ++k) {
      virt[k] = ctx.pool.take(real * sizeof(T));
      dst[k] = virt[k]->as<T>();
    }
    for (int k = 0; k < nsrc; ++k) {
      if (k == 0 && !host_delta) continue;
      if (super) {
        const T *one[1] = {src[k]};
        T *out[1] = {dst[k]};
        interp_add<T, 1>(ctx, L, one, V, out, true);
      } else {
        k_block_average<T><<<(unsigned)((m + 255) / 256), 256, 0, ctx.stream>>>(src[k], L.n, s, dst[k], n);
        launched();
      }
    }
    for (int k = 0; k < nsrc; ++k) src[k] = dst[k];
  }
  const size_t m = (size_t)nz * n * n;
  auto dv = ctx.pool.take(std::max<size_t>(1, 7 * m) * sizeof(float));
  auto di = ctx.pool.take(std::max<size_t>(1, m) * sizeof(unsigned long long));
  float *vel = host_vel ? dv->as<float>() : nullptr, *pos = host_pos ? dv->as<float>() + 3 * m : nullptr,
        *dl = host_delta ? dv->as<float>() + 6 * m : nullptr;
  unsigned long long *id = host_ids ? di->as<unsigned long long>() : nullptr;
  const double ratio = velocity_to_offset_ratio(ctx.cosmo);
  const unsigned blocks = (unsigned)((m + 255) / 256);
  if (lpt2)
    k_grafic_slabs<T, true><<<blocks, 256, 0, ctx.stream>>>(src[1], src[2], src[3], src[4], src[5], src[6], src[0], n,
                                                           z0, nz, g.roll[0], g.roll[1], g.roll[2], ratio, g.vel_factor,
                                                           g.pos_factor, vel, pos, dl, id, g.id_offset);
  else
    k_grafic_slabs<T, false><<<blocks, 256, 0, ctx.stream>>>(src[1], src[2], src[3], nullptr, nullptr, nullptr, src[0],
                                                            n, z0, nz, g.roll[0], g.roll[1], g.roll[2], ratio,
                                                            g.vel_factor, g.pos_factor, vel, pos, dl, id, g.id_offset);
  launched();
  if (host_vel) GIC_CUDA(cudaMemcpyAsync(host_vel, vel, 3 * m * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
  if (host_pos) GIC_CUDA(cudaMemcpyAsync(host_pos, pos, 3 * m * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
  if (host_delta) GIC_CUDA(cudaMemcpyAsync(host_delta, dl, m * sizeof(float), cudaMemcpyDeviceToHost, ctx.stream));
  if (host_ids)
    GIC_CUDA(cudaMemcpyAsync(host_ids, id, m * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx.stream));
  GIC_CUDA(cudaStreamSynchronize(ctx.stream));
  for (auto &b : virt)
    if (b) ctx.pool.give(std::move(b));
  ctx.pool.give(std::move(dv));
  ctx.pool.give(std::move(di));
}

void grafic_pack(Context &ctx, const gic_grafic_grid &g, int z0, int nz, float *host_vel, float *host_pos,
                 float *host_delta, unsigned long long *host_ids) {
  if (g.level < 0 || g.level >= (int)ctx.levels.size()) fail(GIC_ERR_INVALID_ARG, "no such level");
  const Level &L = *ctx.levels[g.level];
  if (!L.have_fields) fail(GIC_ERR_NOT_READY, "fields have not been computed");
  const int f = g.factor;
  if (f == 0 || f == -1 || (f < -1 && L.n % (-f)) || (f > 1 && (long long)L.n * f > 2048))
    fail(GIC_ERR_INVALID_ARG, "factor must be 1, >= 2 (supersampled, at most 2048 cells per side) or <= -2 "
                              "dividing the level's cells per side (subsampled)");
  const int n = f > 1 ? L.n * f : (f < -1 ? L.n / -f : L.n);
  if (z0 < 0 || nz < 0 || z0 + nz > n) fail(GIC_ERR_INVALID_ARG, "slab range outside the grid");
  if (nz == 0) return;
  if (ctx.dbl()) grafic_typed<double>(ctx, g.level, g, z0, nz, host_vel, host_pos, host_delta, host_ids);
  else grafic_typed<float>(ctx, g.level, g, z0, nz, host_vel, host_pos, host_delta, host_ids);
}

void resampled_particles(Context &ctx, const Level &L, int factor, double *host_pos, double *host_vel) {
  if (!L.have_fields) fail(GIC_ERR_NOT_READY, "displacement fields not computed");
  if (ctx.dbl())
    resampled_typed<double>(ctx, L, factor, host_pos, host_vel);
  else
    resampled_typed<float>(ctx, L, factor, host_pos, host_vel);
}

template <typename T>
static void matched_typed(Context &ctx, const Level &F, const Level &Cl, const unsigned long long *host_cells,
                          size_t count, double *host_pos, double *host_vel) {
  Matched g{};
  const int r = (int)std::lround(Cl.dx / F.dx);
  g.nv = Cl.n * r;
  g.nw = F.n;
  g.nc = Cl.n;
  g.wrap_coarse = Cl.box == Cl.periodic ? 1 : 0;
  g.dxv = F.dx;
  g.dxc = Cl.dx;
  g.period = F.periodic;
  for (int a = 0; a < 3; ++a) {
    g.vx0[a] = Cl.x0[a];
    g.cx0[a] = Cl.x0[a];
    // the window's lower corner in cells of the matching grid (virtualgrid.hpp:257-259)
    g.w0[a] = (int)std::lround((F.x0[a] - Cl.x0[a]) / F.dx);
  }
  auto cells = ctx.pool.take(count * sizeof(unsigned long long));
  auto pos = ctx.pool.take(3 * count * sizeof(double));
  auto vel = ctx.pool.take(3 * count * sizeof(T));
  GIC_CUDA(cudaMemcpyAsync(cells->ptr, host_cells, count * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                           ctx.stream));
  k_matched_particles<T><<<(unsigned)((count + 255) / 256), 256, 0, ctx.stream>>>(
      cells->as<unsigned long long>(), count, g, F.field[1].as<T>(), F.field[2].as<T>(), F.field[3].as<T>(),
      Cl.field[1].as<T>(), Cl.field[2].as<T>(), Cl.field[3].as<T>(), (T)velocity_to_offset_ratio(ctx.cosmo),
      pos->as<double>(), vel->as<T>());
  launched();
  GIC_CUDA(cudaMemcpyAsync(host_pos, pos->ptr, 3 * count * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
  if (sizeof(T) == sizeof(double)) {
    GIC_CUDA(cudaMemcpyAsync(host_vel, vel->ptr, 3 * count * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
  } else {
    GIC_CUDA(cudaStreamSynchronize(ctx.stream));
    k_widen<T><<<(unsigned)((3 * count + 255) / 256), 256, 0, ctx.stream>>>(vel->as<T>(), pos->as<double>(), 3 * count);
    launched();
    GIC_CUDA(cudaMemcpyAsync(host_vel, pos->ptr, 3 * count * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
  }
  GIC_CUDA(cudaStreamSynchronize(ctx.stream));
  ctx.pool.give(std::move(cells));
  ctx.pool.give(std::move(pos));
  ctx.pool.give(std::move(vel));
}

void matched_particles(Context &ctx, int level, const unsigned long long *cells, size_t count, double *pos,
                       double *vel) {
  const Level &F = *ctx.levels[level], &Cl = *ctx.levels[level - 1];
  if (!F.have_fields || !Cl.have_fields) fail(GIC_ERR_NOT_READY, "displacement fields not computed");
  const unsigned long long nv = (unsigned long long)Cl.n * (unsigned long long)std::lround(Cl.dx / F.dx);
  const unsigned long long total = nv * nv * nv;
  for (size_t i = 0; i < count; ++i)
    if (cells[i] >= total) fail(GIC_ERR_INVALID_ARG, "cell index beyond the resolution-matching grid");
  if (count == 0) return;
  if (ctx.dbl())
    matched_typed<double>(ctx, F, Cl, cells, count, pos, vel);
  else
    matched_typed<float>(ctx, F, Cl, cells, count, pos, vel);
}

void make_particles(Context &ctx, Level &L, int order) {
  if (!L.have_fields) fail(GIC_ERR_NOT_READY, "displacement fields not computed");
  if (order == 2 && !L.have_lpt2) fail(GIC_ERR_NOT_READY, "second-order displacements not computed");
  if (ctx.dbl())
    particles_typed<double>(ctx, L, order);
  else
    particles_typed<float>(ctx, L, order);
}

}  // namespace gic
