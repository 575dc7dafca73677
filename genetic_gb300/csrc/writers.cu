// Tipsy particle records of one level or a two-level zoom, in genetIC's particle-mapper
// order, packed on the host (threads) or on the device.
//
// The records are TipsyParticle::dark (genetIC/src/io/tipsy.hpp:61-63) as
// TipsyOutput::saveNextBlockOfTipsyParticles fills them (tipsy.hpp:109-145):
//   mass = m * mass_factor, (x, y, z) = pos * pos_factor - 0.5, eps = soft * pos_factor,
//   (vx, vy, vz) = vel * vel_factor, phi = 0,
// each product and difference rounded in double (no fused multiply-add) and then to float.
// The order is that of OneLevelParticleMapper (cell order) and TwoLevelParticleMapper
// (genetIC/src/simulation/particles/mapper/twolevelmapper.hpp:262-320, 869-893): the
// level-0 cells that are not replaced, in cell order, then for every replaced level-0
// cell in ascending order the r^3 level-1 cells it covers, x, y, z ascending
// (Grid::insertCubeIdsIntoVector, grid.hpp:704-729, iterateOverCube, coordinate.hpp:197-208).
#include "gic_internal.h"

#include <algorithm>
#include <thread>
#include <vector>

namespace gic {
namespace {

constexpr int kRowWords = 32;  // a row of at most 1024 cells as a bit mask

// the map as the kernels and the host loops read it
struct MapView {
  int nlevels, n0, n1, ratio, org[3];
  unsigned long long n_replaced, n_kept, per_block;  // per_block = ratio^3
  const unsigned long long *replaced;                // ascending level-0 cell ids
};

struct TipsyConst {
  double mass[2], eps[2], pf, vf, mf;
};

__host__ __device__ inline int popc32(unsigned v) {
#ifdef __CUDA_ARCH__
  return __popc(v);
#else
  return __builtin_popcount(v);
#endif
}

// products and differences rounded separately, as the reference's host build does
__host__ __device__ inline double mul_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;  // this translation unit is compiled with -ffp-contract=off
#endif
}
__host__ __device__ inline double sub_rn(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}

// position of cell z of a row among the row's kept cells, or -1 when it is replaced;
// w: the row's replaced cells as bits, pre[k] = replaced cells in words below k
__host__ __device__ inline int row_rank(const unsigned *w, const int *pre, int z) {
  const int k = z >> 5;
  const unsigned bit = 1u << (z & 31);
  if (w[k] & bit) return -1;
  return z - pre[k] - popc32(w[k] & (bit - 1u));
}

// level-1 cell of the j-th fine particle (j < n_replaced * ratio^3)
__host__ __device__ inline unsigned long long fine_cell(const MapView &m, unsigned long long j) {
  const unsigned long long parent = m.replaced[j / m.per_block];
  const unsigned s = (unsigned)(j % m.per_block), r = (unsigned)m.ratio;
  const long long n0 = m.n0;
  long long p[3] = {(long long)(parent / (unsigned long long)(n0 * n0)), (long long)((parent / n0) % n0),
                    (long long)(parent % n0)};
  for (int a = 0; a < 3; ++a) {
    p[a] -= m.org[a];
    if (p[a] < 0) p[a] += n0;
  }
  const unsigned long long fx = (unsigned long long)p[0] * r + s / (r * r);
  const unsigned long long fy = (unsigned long long)p[1] * r + (s / r) % r;
  const unsigned long long fz = (unsigned long long)p[2] * r + s % r;
  return (fx * m.n1 + fy) * m.n1 + fz;
}

template <typename V>
__host__ __device__ inline void tipsy_record(gic_tipsy_dark &o, const double *pos, const V *vel, unsigned long long cell,
                                             int level, const TipsyConst &c) {
  const double *p = pos + 3 * cell;
  const V *v = vel + 3 * cell;
  o.mass = (float)mul_rn(c.mass[level], c.mf);
  o.x = (float)sub_rn(mul_rn(p[0], c.pf), 0.5);
  o.y = (float)sub_rn(mul_rn(p[1], c.pf), 0.5);
  o.z = (float)sub_rn(mul_rn(p[2], c.pf), 0.5);
  o.vx = (float)mul_rn((double)v[0], c.vf);
  o.vy = (float)mul_rn((double)v[1], c.vf);
  o.vz = (float)mul_rn((double)v[2], c.vf);
  o.eps = (float)mul_rn(c.eps[level], c.pf);
  o.phi = 0.f;
}

// the map's view, checked; replaced cells must lie under the level-1 grid, as
// TwoLevelParticleMapper requires (calculateHiresParticleList throws otherwise)
MapView check_map(const gic_particle_map *m) {
  if (!m) fail(GIC_ERR_INVALID_ARG, "null map");
  MapView v{};
  v.nlevels = m->nlevels;
  if (v.nlevels != 1 && v.nlevels != 2) fail(GIC_ERR_INVALID_ARG, "a tipsy map has one or two levels");
  v.n0 = m->n[0];
  if (v.n0 < 1 || v.n0 > 32 * kRowWords) fail(GIC_ERR_INVALID_ARG, "level 0 needs 1 to 1024 cells per side");
  const unsigned long long n03 = (unsigned long long)v.n0 * v.n0 * v.n0;
  v.ratio = 1;
  v.per_block = 1;
  if (v.nlevels == 1) {
    if (m->n_replaced) fail(GIC_ERR_INVALID_ARG, "a single level replaces no cells");
    v.n_kept = n03;
    return v;
  }
  v.n1 = m->n[1];
  v.ratio = m->ratio;
  if (v.ratio < 1 || v.n1 < v.ratio || v.n1 % v.ratio) fail(GIC_ERR_INVALID_ARG, "level 1 needs a multiple of ratio cells per side");
  for (int a = 0; a < 3; ++a) {
    v.org[a] = m->origin[a];
    if (v.org[a] < 0 || v.org[a] >= v.n0) fail(GIC_ERR_INVALID_ARG, "the level-1 origin is a level-0 cell coordinate");
  }
  v.n_replaced = m->n_replaced;
  if (v.n_replaced > n03 || (v.n_replaced && !m->replaced)) fail(GIC_ERR_INVALID_ARG, "bad list of replaced cells");
  v.replaced = m->replaced;
  const long long span = v.n1 / v.ratio, n0 = v.n0;
  for (unsigned long long k = 0; k < v.n_replaced; ++k) {
    const unsigned long long c = v.replaced[k];
    if (c >= n03 || (k && c <= v.replaced[k - 1]))
      fail(GIC_ERR_INVALID_ARG, "replaced cells must be ascending level-0 cell ids");
    const long long p[3] = {(long long)(c / (unsigned long long)(n0 * n0)), (long long)((c / n0) % n0), (long long)(c % n0)};
    for (int a = 0; a < 3; ++a) {
      long long d = p[a] - v.org[a];
      if (d < 0) d += n0;
      if (d >= span) fail(GIC_ERR_INVALID_ARG, "Requested zoom region falls outside high resolution grid");
    }
  }
  v.n_kept = n03 - v.n_replaced;
  v.per_block = (unsigned long long)v.ratio * v.ratio * v.ratio;
  return v;
}

unsigned long long map_size(const MapView &v) { return v.n_kept + v.n_replaced * v.per_block; }

TipsyConst tipsy_const(const gic_particle_map *m) {
  TipsyConst c{};
  for (int l = 0; l < 2; ++l) {
    c.mass[l] = m->mass[l];
    c.eps[l] = m->eps[l];
  }
  c.pf = m->pos_factor;
  c.vf = m->vel_factor;
  c.mf = m->mass_factor;
  return c;
}

// per level-0 row (x, y): the first replaced entry of the row (rep_begin, one more
// entry at the end) and the kept cells before the row
void row_tables(const MapView &v, std::vector<unsigned long long> &rep_begin, std::vector<unsigned long long> &kept_before) {
  const unsigned long long rows = (unsigned long long)v.n0 * v.n0;
  rep_begin.resize(rows + 1);
  kept_before.resize(rows);
  unsigned long long k = 0;
  for (unsigned long long row = 0; row < rows; ++row) {
    rep_begin[row] = k;
    kept_before[row] = row * v.n0 - k;
    while (k < v.n_replaced && v.replaced[k] < (row + 1) * v.n0) ++k;
  }
  rep_begin[rows] = k;
}

// the replaced cells of a row as bits, and the counts below each word
inline void row_mask(const MapView &v, unsigned long long row, unsigned long long rb, unsigned long long re, unsigned *w,
                     int *pre) {
  for (int q = 0; q < kRowWords; ++q) w[q] = 0;
  for (unsigned long long k = rb; k < re; ++k) {
    const int z = (int)(v.replaced[k] - row * v.n0);
    w[z >> 5] |= 1u << (z & 31);
  }
  int s = 0;
  for (int q = 0; q < kRowWords; ++q) {
    pre[q] = s;
    s += popc32(w[q]);
  }
}

// every particle of [first, first + count) in mapper order, on `threads` host threads
// (0: all cores): f(o, level, cell) with o the particle's index in the map
template <typename F>
void for_each_particle(const MapView &v, unsigned long long first, unsigned long long count, int threads, const F &f) {
  std::vector<unsigned long long> rep_begin, kept_before;
  row_tables(v, rep_begin, kept_before);
  const unsigned long long rows = (unsigned long long)v.n0 * v.n0, end = first + count;
  auto kept_rows = [&](unsigned long long r0, unsigned long long r1) {
    unsigned w[kRowWords];
    int pre[kRowWords];
    for (unsigned long long row = r0; row < r1; ++row) {
      const unsigned long long rb = rep_begin[row], re = rep_begin[row + 1], kb = kept_before[row];
      if (kb + (v.n0 - (re - rb)) <= first || kb >= end) continue;
      row_mask(v, row, rb, re, w, pre);
      for (int z = 0; z < v.n0; ++z) {
        const int rk = row_rank(w, pre, z);
        if (rk < 0) continue;
        const unsigned long long o = kb + (unsigned long long)rk;
        if (o >= first && o < end) f(o, 0, row * v.n0 + z);
      }
    }
  };
  const unsigned long long f0 = std::max(first, v.n_kept), f1 = std::max(end, v.n_kept);
  auto fine = [&](unsigned long long o0, unsigned long long o1) {
    for (unsigned long long o = o0; o < o1; ++o) f(o, 1, fine_cell(v, o - v.n_kept));
  };
  int nt = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&, t] {
      kept_rows(rows * t / nt, rows * (t + 1) / nt);
      if (f1 > f0) fine(f0 + (f1 - f0) * t / nt, f0 + (f1 - f0) * (t + 1) / nt);
    });
  for (auto &th : pool) th.join();
}

template <typename V>
__global__ void k_tipsy_kept(gic_tipsy_dark *out, unsigned long long first, unsigned long long count, MapView v,
                             const unsigned long long *rep_begin, const unsigned long long *kept_before, const double *pos,
                             const V *vel, TipsyConst c) {
  // a CTA per level-0 row
  const unsigned long long row = blockIdx.x;
  __shared__ unsigned w[kRowWords];
  __shared__ int pre[kRowWords];
  if (threadIdx.x < kRowWords) w[threadIdx.x] = 0;
  __syncthreads();
  const unsigned long long rb = rep_begin[row], re = rep_begin[row + 1];
  for (unsigned long long k = rb + threadIdx.x; k < re; k += blockDim.x) {
    const int z = (int)(v.replaced[k] - row * v.n0);
    atomicOr(&w[z >> 5], 1u << (z & 31));
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int q = 0; q < kRowWords; ++q) {
      pre[q] = s;
      s += __popc(w[q]);
    }
  }
  __syncthreads();
  const unsigned long long kb = kept_before[row];
  for (int z = threadIdx.x; z < v.n0; z += blockDim.x) {
    const int rk = row_rank(w, pre, z);
    if (rk < 0) continue;
    const unsigned long long o = kb + (unsigned long long)rk;
    if (o < first || o - first >= count) continue;
    tipsy_record(out[o - first], pos, vel, row * v.n0 + z, 0, c);
  }
}

template <typename V>
__global__ void k_tipsy_fine(gic_tipsy_dark *out, unsigned long long first, unsigned long long o0, unsigned long long o1,
                             MapView v, const double *pos, const V *vel, TipsyConst c) {
  const unsigned long long o = o0 + (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= o1) return;
  tipsy_record(out[o - first], pos, vel, fine_cell(v, o - v.n_kept), 1, c);
}

}  // namespace

unsigned long long tipsy_count(const gic_particle_map *m) { return map_size(check_map(m)); }

static void check_window(const MapView &v, unsigned long long first, unsigned long long count, const void *out) {
  const unsigned long long total = map_size(v);
  if (first > total || count > total - first) fail(GIC_ERR_INVALID_ARG, "records outside the map");
  if (count && !out) fail(GIC_ERR_INVALID_ARG, "null output");
}

void tipsy_pack_host(const gic_particle_map *m, const double *const *pos, const double *const *vel, unsigned long long first,
                     unsigned long long count, gic_tipsy_dark *out, int threads) {
  const MapView v = check_map(m);
  check_window(v, first, count, out);
  if (!pos || !vel || !pos[0] || !vel[0] || (v.nlevels == 2 && (!pos[1] || !vel[1])))
    fail(GIC_ERR_INVALID_ARG, "null particle arrays");
  if (!count) return;
  const TipsyConst c = tipsy_const(m);
  for_each_particle(v, first, count, threads, [&](unsigned long long o, int l, unsigned long long cell) {
    tipsy_record(out[o - first], pos[l], vel[l], cell, l, c);
  });
}

void gadget_pack_host(const gic_particle_map *m, const double *const *pos, const double *const *vel,
                      unsigned long long first, unsigned long long count, float *pos_out, float *vel_out,
                      unsigned long long *ids, float *mass_out, int threads) {
  const MapView v = check_map(m);
  const void *any = pos_out ? (const void *)pos_out : vel_out ? (const void *)vel_out : ids ? (const void *)ids
                                                                                         : (const void *)mass_out;
  check_window(v, first, count, any);
  auto arrays_ok = [&](const double *const *a) { return a && a[0] && (v.nlevels == 1 || a[1]); };
  if ((pos_out && !arrays_ok(pos)) || (vel_out && !arrays_ok(vel))) fail(GIC_ERR_INVALID_ARG, "null particle arrays");
  if (!count) return;
  const float mass[2] = {(float)m->mass[0], (float)m->mass[1]};
  for_each_particle(v, first, count, threads, [&](unsigned long long o, int l, unsigned long long cell) {
    const unsigned long long k = o - first;
    for (int a = 0; a < 3; ++a) {
      if (pos_out) pos_out[3 * k + a] = (float)pos[l][3 * cell + a];
      if (vel_out) vel_out[3 * k + a] = (float)vel[l][3 * cell + a];
    }
    if (ids) ids[k] = o;
    if (mass_out) mass_out[k] = mass[l];
  });
}

template <typename V>
static void launch_tipsy(Context &C, const MapView &dv, const TipsyConst &c, unsigned long long first, unsigned long long count,
                         const unsigned long long *rep_begin, const unsigned long long *kept_before, gic_tipsy_dark *out) {
  const Level &L0 = *C.levels[0];
  if (first < dv.n_kept) {
    k_tipsy_kept<V><<<(unsigned)((unsigned long long)dv.n0 * dv.n0), 256, 0, C.stream>>>(
        out, first, count, dv, rep_begin, kept_before, L0.pos.as<double>(), L0.vel.as<V>(), c);
    launched();
  }
  const unsigned long long o0 = std::max(first, dv.n_kept), o1 = first + count;
  if (dv.nlevels == 2 && o1 > o0) {
    const Level &L1 = *C.levels[1];
    k_tipsy_fine<V><<<(unsigned)((o1 - o0 + 255) / 256), 256, 0, C.stream>>>(out, first, o0, o1, dv, L1.pos.as<double>(),
                                                                             L1.vel.as<V>(), c);
    launched();
  }
}

void tipsy_pack_device(Context &C, const gic_particle_map *m, unsigned long long first, unsigned long long count,
                       gic_tipsy_dark *host_out) {
  const MapView v = check_map(m);
  check_window(v, first, count, host_out);
  if ((int)C.levels.size() < v.nlevels) fail(GIC_ERR_NOT_READY, "the map has more levels than the context");
  for (int l = 0; l < v.nlevels; ++l) {
    const Level &L = *C.levels[l];
    if (L.n != m->n[l]) fail(GIC_ERR_INVALID_ARG, "map and level sizes differ");
    if (!L.pos.ptr || !L.vel.ptr) fail(GIC_ERR_NOT_READY, "particles have not been generated");
  }
  if (!count) return;
  std::vector<unsigned long long> rep_begin, kept_before;
  row_tables(v, rep_begin, kept_before);
  const size_t rows = (size_t)v.n0 * v.n0, u = sizeof(unsigned long long);
  auto drep = C.pool.take(std::max<size_t>(1, v.n_replaced) * u), dbeg = C.pool.take((rows + 1) * u),
       dkept = C.pool.take(rows * u), dout = C.pool.take((size_t)count * sizeof(gic_tipsy_dark));
  if (v.n_replaced)
    GIC_CUDA(cudaMemcpyAsync(drep->ptr, v.replaced, v.n_replaced * u, cudaMemcpyHostToDevice, C.stream));
  GIC_CUDA(cudaMemcpyAsync(dbeg->ptr, rep_begin.data(), (rows + 1) * u, cudaMemcpyHostToDevice, C.stream));
  GIC_CUDA(cudaMemcpyAsync(dkept->ptr, kept_before.data(), rows * u, cudaMemcpyHostToDevice, C.stream));
  MapView dv = v;
  dv.replaced = drep->as<unsigned long long>();
  const TipsyConst c = tipsy_const(m);
  gic_tipsy_dark *out = dout->as<gic_tipsy_dark>();
  if (C.dbl())
    launch_tipsy<double>(C, dv, c, first, count, dbeg->as<unsigned long long>(), dkept->as<unsigned long long>(), out);
  else
    launch_tipsy<float>(C, dv, c, first, count, dbeg->as<unsigned long long>(), dkept->as<unsigned long long>(), out);
  GIC_CUDA(cudaMemcpyAsync(host_out, out, (size_t)count * sizeof(gic_tipsy_dark), cudaMemcpyDeviceToHost, C.stream));
  GIC_CUDA(cudaStreamSynchronize(C.stream));
  for (auto *b : {&drep, &dbeg, &dkept, &dout}) C.pool.give(std::move(*b));
}

}  // namespace gic
