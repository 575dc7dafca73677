// Particle output in genetIC's particle-mapper order: tipsy records packed on the device
// (one level or a two-level zoom) or by host threads (any depth), and gadget blocks packed
// by host threads.
//
// The tipsy records are TipsyParticle::dark (genetIC/src/io/tipsy.hpp:61-63) as
// TipsyOutput::saveNextBlockOfTipsyParticles fills them (tipsy.hpp:109-145):
//   mass = m * mass_factor, (x, y, z) = pos * pos_factor - 0.5, eps = soft * pos_factor,
//   (vx, vy, vz) = vel * vel_factor, phi = 0,
// each product and difference rounded in double (no fused multiply-add) and then to float.
// The gadget blocks are GadgetOutput's (io/gadget.hpp:481-520) for one particle type:
// Coordinate<float> of positions and velocities, the map index as id, float masses.
// The order is that of OneLevelParticleMapper (cell order) and of TwoLevelParticleMapper
// (genetIC/src/simulation/particles/mapper/twolevelmapper.hpp:262-320, 869-893): the
// level-0 cells that are not replaced, in cell order, then for every replaced level-0
// cell in ascending order the r^3 level-1 cells it covers, x, y, z ascending
// (Grid::insertCubeIdsIntoVector, grid.hpp:704-729, iterateOverCube, coordinate.hpp:197-208).
// Deeper zooms nest one TwoLevelParticleMapper per level (ic.hpp:1150-1185).
#include "gic_internal.h"

#include <algorithm>
#include <thread>
#include <vector>

namespace gic {
namespace {

constexpr int kRowWords = 32;  // a row of at most 1024 cells as a bit mask
constexpr int kMaxLevels = GIC_MAP_MAX_LEVELS;

// the map as the kernels and the host loops read it
struct MapView {
  int nlevels, n0, n1, ratio, org[3];
  unsigned long long n_replaced, n_kept, per_block;  // per_block = ratio^3
  const unsigned long long *replaced;                // ascending level-0 cell ids
};

struct TipsyConst {
  double mass[kMaxLevels], eps[kMaxLevels], pf, vf, mf;
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

// cell s (x, y, z ascending) of the ratio^3 block that parent cell `parent` of a grid of
// np cells per side covers on a grid of nc cells whose corner is parent cell `org`
__host__ __device__ inline unsigned long long block_cell(int np, int nc, int ratio, const int *org,
                                                        unsigned long long parent, unsigned s) {
  const unsigned r = (unsigned)ratio;
  const long long n0 = np;
  long long p[3] = {(long long)(parent / (unsigned long long)(n0 * n0)), (long long)((parent / n0) % n0),
                    (long long)(parent % n0)};
  for (int a = 0; a < 3; ++a) {
    p[a] -= org[a];
    if (p[a] < 0) p[a] += n0;
  }
  const unsigned long long fx = (unsigned long long)p[0] * r + s / (r * r);
  const unsigned long long fy = (unsigned long long)p[1] * r + (s / r) % r;
  const unsigned long long fz = (unsigned long long)p[2] * r + s % r;
  return (fx * (unsigned long long)nc + fy) * (unsigned long long)nc + fz;
}

// level-1 cell of the j-th fine particle (j < n_replaced * ratio^3)
__host__ __device__ inline unsigned long long fine_cell(const MapView &m, unsigned long long j) {
  return block_cell(m.n0, m.n1, m.ratio, m.org, m.replaced[j / m.per_block], (unsigned)(j % m.per_block));
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

// every level of a map, checked: replaced cells ascending, each under the next level's
// grid (TwoLevelParticleMapper's calculateHiresParticleList throws otherwise) and under a
// replaced cell of the level above (its consistency assertion, twolevelmapper.hpp:287-302)
struct LevelMap {
  int n, ratio, org[3];
  const unsigned long long *rep;
  unsigned long long nrep;
};
struct MapFull {
  int nlevels;
  LevelMap lv[kMaxLevels];
  unsigned long long total;
};

bool contains(const unsigned long long *a, unsigned long long n, unsigned long long v) {
  return std::binary_search(a, a + n, v);
}

MapFull check_full(const gic_particle_map *m) {
  if (!m) fail(GIC_ERR_INVALID_ARG, "null map");
  MapFull f{};
  f.nlevels = m->nlevels;
  if (f.nlevels < 1 || f.nlevels > kMaxLevels) fail(GIC_ERR_INVALID_ARG, "a particle map has 1 to 8 levels");
  for (int l = 0; l < f.nlevels; ++l) {
    LevelMap &L = f.lv[l];
    L.n = m->n[l];
    if (L.n < 1 || (l == 0 && L.n > 32 * kRowWords)) fail(GIC_ERR_INVALID_ARG, "level 0 needs 1 to 1024 cells per side");
    L.ratio = l ? m->ratio[l] : 1;
    if (l) {
      const LevelMap &P = f.lv[l - 1];
      if (L.ratio < 1 || L.n < L.ratio || L.n % L.ratio)
        fail(GIC_ERR_INVALID_ARG, "each zoom level needs a multiple of its ratio cells per side");
      for (int a = 0; a < 3; ++a) {
        L.org[a] = m->origin[l][a];
        if (L.org[a] < 0 || L.org[a] >= P.n) fail(GIC_ERR_INVALID_ARG, "a level's origin is a cell coordinate of the level above");
      }
    }
    L.nrep = m->n_replaced[l];
    L.rep = m->replaced[l];
    const unsigned long long n3 = (unsigned long long)L.n * L.n * L.n;
    if (L.nrep && (l == f.nlevels - 1)) fail(GIC_ERR_INVALID_ARG, "the finest level replaces no cells");
    if (L.nrep > n3 || (L.nrep && !L.rep)) fail(GIC_ERR_INVALID_ARG, "bad list of replaced cells");
  }
  for (int l = 0; l + 1 < f.nlevels; ++l) {
    const LevelMap &L = f.lv[l], &C = f.lv[l + 1];
    const unsigned long long n3 = (unsigned long long)L.n * L.n * L.n;
    const long long span = C.n / C.ratio, n0 = L.n;
    for (unsigned long long k = 0; k < L.nrep; ++k) {
      const unsigned long long c = L.rep[k];
      if (c >= n3 || (k && c <= L.rep[k - 1])) fail(GIC_ERR_INVALID_ARG, "replaced cells must be ascending cell ids");
      const long long p[3] = {(long long)(c / (unsigned long long)(n0 * n0)), (long long)((c / n0) % n0), (long long)(c % n0)};
      for (int a = 0; a < 3; ++a) {
        long long d = p[a] - C.org[a];
        if (d < 0) d += n0;
        if (d >= span) fail(GIC_ERR_INVALID_ARG, "Requested zoom region falls outside high resolution grid");
      }
      if (l) {
        // the parent on level l-1 must itself be replaced: the cell is a particle of the mapper
        const LevelMap &P = f.lv[l - 1];
        const long long q[3] = {(p[0] / L.ratio + L.org[0]) % P.n, (p[1] / L.ratio + L.org[1]) % P.n,
                                (p[2] / L.ratio + L.org[2]) % P.n};
        const unsigned long long parent = ((unsigned long long)q[0] * P.n + q[1]) * P.n + q[2];
        if (!contains(P.rep, P.nrep, parent))
          fail(GIC_ERR_INVALID_ARG, "a replaced cell is not a particle of the level above's zoom");
      }
    }
  }
  // particles per level: level 0's cells, or the blocks of the level above, less those replaced
  f.total = 0;
  for (int l = 0; l < f.nlevels; ++l) {
    const LevelMap &L = f.lv[l];
    const unsigned long long have =
        l ? f.lv[l - 1].nrep * (unsigned long long)L.ratio * L.ratio * L.ratio : (unsigned long long)L.n * L.n * L.n;
    f.total += have - L.nrep;
  }
  return f;
}

// the one- or two-level view the streaming host loop and the kernels use
MapView view2(const MapFull &f) {
  MapView v{};
  v.nlevels = f.nlevels;
  v.n0 = f.lv[0].n;
  v.ratio = 1;
  v.per_block = 1;
  const unsigned long long n03 = (unsigned long long)v.n0 * v.n0 * v.n0;
  v.n_kept = n03;
  if (f.nlevels == 2) {
    v.n1 = f.lv[1].n;
    v.ratio = f.lv[1].ratio;
    for (int a = 0; a < 3; ++a) v.org[a] = f.lv[1].org[a];
    v.n_replaced = f.lv[0].nrep;
    v.replaced = f.lv[0].rep;
    v.n_kept = n03 - v.n_replaced;
    v.per_block = (unsigned long long)v.ratio * v.ratio * v.ratio;
  }
  return v;
}

MapView check_map(const gic_particle_map *m) {
  const MapFull f = check_full(m);
  if (f.nlevels > 2) fail(GIC_ERR_INVALID_ARG, "the device packer takes maps of one or two levels");
  return view2(f);
}

unsigned long long map_size(const MapView &v) { return v.n_kept + v.n_replaced * v.per_block; }

TipsyConst tipsy_const(const gic_particle_map *m) {
  TipsyConst c{};
  for (int l = 0; l < kMaxLevels; ++l) {
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

// the mapper order of three or more levels, written out: level 0's cells, then per zoom
// level the order so far without the replaced cells of the level above, followed by
// the blocks of those cells in ascending id
void build_order(const MapFull &f, std::vector<unsigned char> &lev, std::vector<unsigned long long> &cell) {
  const unsigned long long n3 = (unsigned long long)f.lv[0].n * f.lv[0].n * f.lv[0].n;
  lev.assign(n3, 0);
  cell.resize(n3);
  for (unsigned long long c = 0; c < n3; ++c) cell[c] = c;
  for (int l = 1; l < f.nlevels; ++l) {
    const LevelMap &P = f.lv[l - 1], &L = f.lv[l];
    size_t w = 0;
    for (size_t i = 0; i < cell.size(); ++i)
      if (!(lev[i] == l - 1 && contains(P.rep, P.nrep, cell[i]))) {
        lev[w] = lev[i];
        cell[w] = cell[i];
        ++w;
      }
    lev.resize(w);
    cell.resize(w);
    const unsigned per = (unsigned)(L.ratio * L.ratio * L.ratio);
    for (unsigned long long k = 0; k < P.nrep; ++k)
      for (unsigned s = 0; s < per; ++s) {
        lev.push_back((unsigned char)l);
        cell.push_back(block_cell(P.n, L.n, L.ratio, L.org, P.rep[k], s));
      }
  }
}

// every particle of [first, first + count) of any map in mapper order: f(o, level, cell)
template <typename F>
void for_each_particle_full(const MapFull &mf, unsigned long long first, unsigned long long count, int threads,
                            const F &f) {
  if (mf.nlevels <= 2) {
    for_each_particle(view2(mf), first, count, threads, f);
    return;
  }
  std::vector<unsigned char> lev;
  std::vector<unsigned long long> cell;
  build_order(mf, lev, cell);
  int nt = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
  std::vector<std::thread> pool;
  for (int t = 0; t < nt; ++t)
    pool.emplace_back([&, t] {
      for (unsigned long long o = first + count * t / nt; o < first + count * (t + 1) / nt; ++o) f(o, lev[o], cell[o]);
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

// Gadget blocks on the device.  File index = mapper index + shift (each level's particles
// are one run of the mapper order; the file holds them by gadget type).  Outputs for file
// indices [first, first + count); a level's part of that window is mapper range [lo, hi).
struct GadgetOut {
  float *pos, *vel, *mass;
  unsigned long long *ids;
  unsigned long long first;
};

template <typename V>
__device__ __forceinline__ void gadget_emit(const GadgetOut &g, unsigned long long k, unsigned long long o,
                                            const double *pos, const V *vel, unsigned long long cell, float mass) {
  for (int c = 0; c < 3; ++c) {
    if (g.pos) g.pos[3 * k + c] = (float)pos[3 * cell + c];
    if (g.vel) g.vel[3 * k + c] = (float)vel[3 * cell + c];
  }
  if (g.ids) g.ids[k] = o;
  if (g.mass) g.mass[k] = mass;
}

template <typename V>
__global__ void k_gadget_kept(GadgetOut g, unsigned long long lo, unsigned long long hi, unsigned long long shift,
                              MapView v, const unsigned long long *rep_begin, const unsigned long long *kept_before,
                              const double *pos, const V *vel, float mass) {
  // a CTA per level-0 row, as k_tipsy_kept
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
    if (o < lo || o >= hi) continue;
    gadget_emit(g, o + shift - g.first, o, pos, vel, row * v.n0 + z, mass);
  }
}

template <typename V>
__global__ void k_gadget_fine(GadgetOut g, unsigned long long lo, unsigned long long hi, unsigned long long shift,
                              MapView v, const double *pos, const V *vel, float mass) {
  const unsigned long long o = lo + (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= hi) return;
  gadget_emit(g, o + shift - g.first, o, pos, vel, fine_cell(v, o - v.n_kept), mass);
}

}  // namespace

unsigned long long tipsy_count(const gic_particle_map *m) { return check_full(m).total; }

// TipsyOutput's factors (tipsy.hpp:200-239): the particle masses summed one by one in
// mapper order (where each level's particles form one run, in level order), then
// mass_factor = Om / sum, pos_factor = 1 / box, vel_factor = a^-1/2 / dKmsUnit
void tipsy_factors(const gic_particle_map *m, double omega_m, double hubble, double scalefactor, double box,
                   double *pos_factor, double *vel_factor, double *mass_factor) {
  const MapFull f = check_full(m);
  if (!(box > 0) || !(hubble > 0) || !(scalefactor > 0)) fail(GIC_ERR_INVALID_ARG, "box, hubble and a must be positive");
  double tot = 0;
  for (int l = 0; l < f.nlevels; ++l) {
    const LevelMap &L = f.lv[l];
    const unsigned long long have =
        l ? f.lv[l - 1].nrep * (unsigned long long)L.ratio * L.ratio * L.ratio : (unsigned long long)L.n * L.n * L.n;
    const double ml = m->mass[l];
    for (unsigned long long i = 0; i < have - L.nrep; ++i) tot += ml;
  }
  const double mf = omega_m / tot;
  const double kpc = box * 1000 / hubble;
  const double msol = 1e10 / hubble / mf;
  const double kms = std::sqrt(4.3022682e-6 * msol / kpc);
  if (mass_factor) *mass_factor = mf;
  if (pos_factor) *pos_factor = 1. / box;
  if (vel_factor) *vel_factor = std::pow(scalefactor, -0.5) / kms;
}

static void check_window(unsigned long long total, unsigned long long first, unsigned long long count, const void *out) {
  if (first > total || count > total - first) fail(GIC_ERR_INVALID_ARG, "records outside the map");
  if (count && !out) fail(GIC_ERR_INVALID_ARG, "null output");
}

void tipsy_pack_host(const gic_particle_map *m, const double *const *pos, const double *const *vel, unsigned long long first,
                     unsigned long long count, gic_tipsy_dark *out, int threads) {
  const MapFull f = check_full(m);
  check_window(f.total, first, count, out);
  bool ok = pos && vel;
  for (int l = 0; ok && l < f.nlevels; ++l) ok = pos[l] && vel[l];
  if (!ok) fail(GIC_ERR_INVALID_ARG, "null particle arrays");
  if (!count) return;
  const TipsyConst c = tipsy_const(m);
  for_each_particle_full(f, first, count, threads, [&](unsigned long long o, int l, unsigned long long cell) {
    tipsy_record(out[o - first], pos[l], vel[l], cell, l, c);
  });
}

// each level's particles in mapper order: one run per level, in level order
static void level_runs(const MapFull &f, unsigned long long *start, unsigned long long *len) {
  unsigned long long at = 0;
  for (int l = 0; l < f.nlevels; ++l) {
    const LevelMap &L = f.lv[l];
    const unsigned long long have =
        l ? f.lv[l - 1].nrep * (unsigned long long)L.ratio * L.ratio * L.ratio : (unsigned long long)L.n * L.n * L.n;
    start[l] = at;
    len[l] = have - L.nrep;
    at += len[l];
  }
}

void gadget_pack_host(const gic_particle_map *m, const double *const *pos, const double *const *vel,
                      const int *level_types, unsigned long long first, unsigned long long count, float *pos_out,
                      float *vel_out, unsigned long long *ids, float *mass_out, int threads) {
  const MapFull f = check_full(m);
  if (level_types)
    for (int l = 0; l < f.nlevels; ++l)
      if (level_types[l] < 0 || level_types[l] > 5) fail(GIC_ERR_INVALID_ARG, "gadget particle types are 0 to 5");
  const void *any = pos_out ? (const void *)pos_out : vel_out ? (const void *)vel_out : ids ? (const void *)ids
                                                                                         : (const void *)mass_out;
  check_window(f.total, first, count, any);
  auto arrays_ok = [&](const double *const *a) {
    bool ok = a != nullptr;
    for (int l = 0; ok && l < f.nlevels; ++l) ok = a[l] != nullptr;
    return ok;
  };
  if ((pos_out && !arrays_ok(pos)) || (vel_out && !arrays_ok(vel))) fail(GIC_ERR_INVALID_ARG, "null particle arrays");
  if (!count) return;
  float mass[kMaxLevels];
  for (int l = 0; l < kMaxLevels; ++l) mass[l] = (float)m->mass[l];
  // the file holds the types in order 0..5, each type's particles in mapper order
  // (GadgetOutput::genericSaveBlock, gadget.hpp:285-312); a level's particles are one
  // run in mapper order, so a file range of a level is a mapper range
  unsigned long long start[kMaxLevels], len[kMaxLevels], file_at[kMaxLevels];
  level_runs(f, start, len);
  unsigned long long at = 0;
  for (int t = 0; t < 6; ++t)
    for (int l = 0; l < f.nlevels; ++l)
      if ((level_types ? level_types[l] : 1) == t) {
        file_at[l] = at;
        at += len[l];
      }
  const unsigned long long end = first + count;
  for (int l = 0; l < f.nlevels; ++l) {
    const unsigned long long a = std::max(first, file_at[l]), b = std::min(end, file_at[l] + len[l]);
    if (b <= a) continue;
    const unsigned long long shift = file_at[l] - start[l];  // file index = mapper index + shift
    for_each_particle_full(f, a - shift, b - a, threads, [&](unsigned long long o, int lv, unsigned long long cell) {
      const unsigned long long k = o + shift - first;
      for (int c = 0; c < 3; ++c) {
        if (pos_out) pos_out[3 * k + c] = (float)pos[lv][3 * cell + c];
        if (vel_out) vel_out[3 * k + c] = (float)vel[lv][3 * cell + c];
      }
      if (ids) ids[k] = o;
      if (mass_out) mass_out[k] = mass[lv];
    });
  }
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

template <typename V>
static void launch_gadget(Context &C, const MapView &dv, const GadgetOut &g, const unsigned long long *lo,
                          const unsigned long long *hi, const unsigned long long *shift, const float *mass,
                          const unsigned long long *rep_begin, const unsigned long long *kept_before) {
  if (hi[0] > lo[0]) {
    const Level &L0 = *C.levels[0];
    k_gadget_kept<V><<<(unsigned)((unsigned long long)dv.n0 * dv.n0), 256, 0, C.stream>>>(
        g, lo[0], hi[0], shift[0], dv, rep_begin, kept_before, L0.pos.as<double>(), L0.vel.as<V>(), mass[0]);
    launched();
  }
  if (dv.nlevels == 2 && hi[1] > lo[1]) {
    const Level &L1 = *C.levels[1];
    k_gadget_fine<V><<<(unsigned)((hi[1] - lo[1] + 255) / 256), 256, 0, C.stream>>>(g, lo[1], hi[1], shift[1], dv,
                                                                                    L1.pos.as<double>(), L1.vel.as<V>(),
                                                                                    mass[1]);
    launched();
  }
}

void gadget_pack_device(Context &C, const gic_particle_map *m, const int *level_types, unsigned long long first,
                        unsigned long long count, float *pos_out, float *vel_out, unsigned long long *ids,
                        float *mass_out) {
  const MapView v = check_map(m);
  if (level_types)
    for (int l = 0; l < v.nlevels; ++l)
      if (level_types[l] < 0 || level_types[l] > 5) fail(GIC_ERR_INVALID_ARG, "gadget particle types are 0 to 5");
  const void *any = pos_out ? (const void *)pos_out : vel_out ? (const void *)vel_out : ids ? (const void *)ids
                                                                                         : (const void *)mass_out;
  check_window(map_size(v), first, count, any);
  if ((int)C.levels.size() < v.nlevels) fail(GIC_ERR_NOT_READY, "the map has more levels than the context");
  for (int l = 0; l < v.nlevels; ++l) {
    const Level &L = *C.levels[l];
    if (L.n != m->n[l]) fail(GIC_ERR_INVALID_ARG, "map and level sizes differ");
    if (!L.pos.ptr || !L.vel.ptr) fail(GIC_ERR_NOT_READY, "particles have not been generated");
  }
  if (!count) return;
  // mapper runs of the levels, their file positions by type, the window per level
  const unsigned long long start[2] = {0, v.n_kept}, len[2] = {v.n_kept, v.n_replaced * v.per_block};
  unsigned long long file_at[2] = {0, 0}, at = 0, lo[2] = {0, 0}, hi[2] = {0, 0}, shift[2] = {0, 0};
  for (int t = 0; t < 6; ++t)
    for (int l = 0; l < v.nlevels; ++l)
      if ((level_types ? level_types[l] : 1) == t) {
        file_at[l] = at;
        at += len[l];
      }
  const unsigned long long end = first + count;
  for (int l = 0; l < v.nlevels; ++l) {
    const unsigned long long a = std::max(first, file_at[l]), b = std::min(end, file_at[l] + len[l]);
    shift[l] = file_at[l] - start[l];
    if (b > a) {
      lo[l] = a - shift[l];
      hi[l] = b - shift[l];
    }
  }
  float mass[2] = {(float)m->mass[0], (float)m->mass[1]};
  std::vector<unsigned long long> rep_begin, kept_before;
  row_tables(v, rep_begin, kept_before);
  const size_t rows = (size_t)v.n0 * v.n0, u = sizeof(unsigned long long);
  auto drep = C.pool.take(std::max<size_t>(1, v.n_replaced) * u), dbeg = C.pool.take((rows + 1) * u),
       dkept = C.pool.take(rows * u);
  auto dpos = C.pool.take(pos_out ? 3 * count * sizeof(float) : 1), dvel = C.pool.take(vel_out ? 3 * count * sizeof(float) : 1),
       dids = C.pool.take(ids ? count * u : 1), dmass = C.pool.take(mass_out ? count * sizeof(float) : 1);
  if (v.n_replaced)
    GIC_CUDA(cudaMemcpyAsync(drep->ptr, v.replaced, v.n_replaced * u, cudaMemcpyHostToDevice, C.stream));
  GIC_CUDA(cudaMemcpyAsync(dbeg->ptr, rep_begin.data(), (rows + 1) * u, cudaMemcpyHostToDevice, C.stream));
  GIC_CUDA(cudaMemcpyAsync(dkept->ptr, kept_before.data(), rows * u, cudaMemcpyHostToDevice, C.stream));
  MapView dv = v;
  dv.replaced = drep->as<unsigned long long>();
  GadgetOut g{pos_out ? dpos->as<float>() : nullptr, vel_out ? dvel->as<float>() : nullptr,
              mass_out ? dmass->as<float>() : nullptr, ids ? dids->as<unsigned long long>() : nullptr, first};
  if (C.dbl())
    launch_gadget<double>(C, dv, g, lo, hi, shift, mass, dbeg->as<unsigned long long>(), dkept->as<unsigned long long>());
  else
    launch_gadget<float>(C, dv, g, lo, hi, shift, mass, dbeg->as<unsigned long long>(), dkept->as<unsigned long long>());
  if (pos_out) GIC_CUDA(cudaMemcpyAsync(pos_out, g.pos, 3 * count * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
  if (vel_out) GIC_CUDA(cudaMemcpyAsync(vel_out, g.vel, 3 * count * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
  if (ids) GIC_CUDA(cudaMemcpyAsync(ids, g.ids, count * u, cudaMemcpyDeviceToHost, C.stream));
  if (mass_out) GIC_CUDA(cudaMemcpyAsync(mass_out, g.mass, count * sizeof(float), cudaMemcpyDeviceToHost, C.stream));
  GIC_CUDA(cudaStreamSynchronize(C.stream));
  for (auto *b : {&drep, &dbeg, &dkept, &dpos, &dvel, &dids, &dmass}) C.pool.give(std::move(*b));
}

void tipsy_pack_device(Context &C, const gic_particle_map *m, unsigned long long first, unsigned long long count,
                       gic_tipsy_dark *host_out, bool async) {
  const MapView v = check_map(m);
  check_window(map_size(v), first, count, host_out);
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
       dkept = C.pool.take(rows * u);
  std::unique_ptr<DevBuf> dout;
  int slot = -1;
  if (async) {
    // alternate two record buffers; one a copy may still be reading is waited for on the device
    slot = C.records_next;
    C.records_next ^= 1;
    if (!C.copy_stream) {
      GIC_CUDA(cudaStreamCreateWithFlags(&C.copy_stream, cudaStreamNonBlocking));
      GIC_CUDA(cudaEventCreateWithFlags(&C.copy_ready, cudaEventDisableTiming));
    }
    if (!C.records_read[slot]) GIC_CUDA(cudaEventCreateWithFlags(&C.records_read[slot], cudaEventDisableTiming));
    if (C.records_pending[slot]) GIC_CUDA(cudaStreamWaitEvent(C.stream, C.records_read[slot], 0));
    C.records[slot].ensure((size_t)count * sizeof(gic_tipsy_dark));
  } else {
    dout = C.pool.take((size_t)count * sizeof(gic_tipsy_dark));
  }
  if (v.n_replaced)
    GIC_CUDA(cudaMemcpyAsync(drep->ptr, v.replaced, v.n_replaced * u, cudaMemcpyHostToDevice, C.stream));
  GIC_CUDA(cudaMemcpyAsync(dbeg->ptr, rep_begin.data(), (rows + 1) * u, cudaMemcpyHostToDevice, C.stream));
  GIC_CUDA(cudaMemcpyAsync(dkept->ptr, kept_before.data(), rows * u, cudaMemcpyHostToDevice, C.stream));
  MapView dv = v;
  dv.replaced = drep->as<unsigned long long>();
  const TipsyConst c = tipsy_const(m);
  gic_tipsy_dark *out = async ? C.records[slot].as<gic_tipsy_dark>() : dout->as<gic_tipsy_dark>();
  if (C.dbl())
    launch_tipsy<double>(C, dv, c, first, count, dbeg->as<unsigned long long>(), dkept->as<unsigned long long>(), out);
  else
    launch_tipsy<float>(C, dv, c, first, count, dbeg->as<unsigned long long>(), dkept->as<unsigned long long>(), out);
  if (async) {
    GIC_CUDA(cudaEventRecord(C.copy_ready, C.stream));
    GIC_CUDA(cudaStreamWaitEvent(C.copy_stream, C.copy_ready, 0));
    GIC_CUDA(cudaMemcpyAsync(host_out, out, (size_t)count * sizeof(gic_tipsy_dark), cudaMemcpyDeviceToHost,
                             C.copy_stream));
    GIC_CUDA(cudaEventRecord(C.records_read[slot], C.copy_stream));
    C.records_pending[slot] = true;
    // the tables are read by kernels on C.stream only: later users of the pool are ordered after them
    for (auto *b : {&drep, &dbeg, &dkept}) C.pool.give(std::move(*b));
    return;
  }
  GIC_CUDA(cudaMemcpyAsync(host_out, out, (size_t)count * sizeof(gic_tipsy_dark), cudaMemcpyDeviceToHost, C.stream));
  GIC_CUDA(cudaStreamSynchronize(C.stream));
  for (auto *b : {&drep, &dbeg, &dkept, &dout}) C.pool.give(std::move(*b));
}

}  // namespace gic
