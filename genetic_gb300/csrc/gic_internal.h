// Internal declarations of the GB300 field-realisation library (not part of the C-ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <cmath>
#include <vector>
#include <memory>
#include <atomic>
#include <utility>
#include "../../include/gicgpu.h"

namespace gic {

struct Error {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string &msg);
// check the last launch and count it (gic_launch_count)
void launched(int kernels = 1);
unsigned long long launch_count();
void count_launches(unsigned long long kernels);  // kernels run by a graph launch
void cuda_check(cudaError_t e, const char *what);
#define GIC_CUDA(call) ::gic::cuda_check((call), #call)

// Device memory charged to a context, against its gic_device_opts.mem_limit.  A
// context's API calls (and a batch's workers) make its account the thread's current
// one; a DevBuf is charged to the account current when it grows and credited back
// when it is released.
struct MemAccount {
  std::atomic<size_t> used{0};
  size_t limit = 0;  // bytes; 0 = no limit
  // A captured CUDA graph holds device pointers: every allocation gets a serial number,
  // and `frees` counts the releases (or regrowths) of buffers whose serial is at most
  // graph_serial, the last serial when the context's realisation was captured (all
  // buffers before any capture).  Buffers made after a capture cannot be in its graph.
  std::atomic<unsigned long long> serial{0};
  std::atomic<unsigned long long> graph_serial{~0ull};
  std::atomic<unsigned long long> frees{0};
};
extern thread_local MemAccount *t_account;
struct AccountScope {
  MemAccount *prev;
  explicit AccountScope(MemAccount &a) : prev(t_account) { t_account = &a; }
  ~AccountScope() { t_account = prev; }
  AccountScope(const AccountScope &) = delete;
  AccountScope &operator=(const AccountScope &) = delete;
};

// Owning device allocation.
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  MemAccount *acct = nullptr;
  unsigned long long serial = 0;  // allocation number in acct
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) {
      cudaFree(ptr);
      if (acct && serial <= acct->graph_serial.load()) acct->frees++;
    }
    if (acct) acct->used -= bytes;
    acct = nullptr;
    ptr = nullptr;
    bytes = 0;
  }
  void ensure(size_t nbytes) {  // grow-only
    if (nbytes <= bytes && ptr) return;
    release();
    if (nbytes == 0) return;
    MemAccount *a = t_account;
    if (a && a->limit && a->used.load() + nbytes > a->limit)
      fail(GIC_ERR_OOM, "device allocation of " + std::to_string(nbytes) + " bytes would exceed the context's mem_limit of " +
                            std::to_string(a->limit) + " bytes (" + std::to_string(a->used.load()) + " in use)");
    cudaError_t e = cudaMalloc(&ptr, nbytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      ptr = nullptr;
      fail(GIC_ERR_OOM, "cudaMalloc of " + std::to_string(nbytes) + " bytes failed");
    }
    bytes = nbytes;
    if (a) {
      a->used += nbytes;
      acct = a;
      serial = ++a->serial;
    }
  }
  template <typename T> T *as() const { return static_cast<T *>(ptr); }
  void swap(DevBuf &o) {
    std::swap(ptr, o.ptr);
    std::swap(bytes, o.bytes);
    std::swap(acct, o.acct);
    std::swap(serial, o.serial);
  }
};

// Device buffers kept between calls: the fields of the modification algebra take
// them here and give them back, so repeated applications allocate nothing.
struct BufPool {
  std::vector<std::unique_ptr<DevBuf>> free;
  std::unique_ptr<DevBuf> take(size_t nbytes) {
    int best = -1;
    for (int i = 0; i < (int)free.size(); ++i)
      if (free[i]->bytes >= nbytes && (best < 0 || free[i]->bytes < free[best]->bytes)) best = i;
    if (best >= 0) {
      std::unique_ptr<DevBuf> b = std::move(free[best]);
      free.erase(free.begin() + best);
      return b;
    }
    auto b = std::make_unique<DevBuf>();
    try {
      b->ensure(nbytes);
    } catch (const Error &) {
      free.clear();  // give idle buffers back to the device and try once more
      b->ensure(nbytes);
    }
    return b;
  }
  void give(std::unique_ptr<DevBuf> b) {
    if (b) free.push_back(std::move(b));
  }
};

// scratch of the modification algebra (one user at a time; each buffer is used
// within a single operation)
struct GeomEntry;
struct ModScratch {
  DevBuf tab, tabf, conv, masks, tmp_src, win, cells, geom, t1, t2, t3, reduce, compact, csum, fold, btab;
  DevBuf gram;  // the correction's coefficients, formed on the device
  int btab_n = 0, btab_r = 0;  // the (N, r) btab holds the block filter of
  std::vector<std::unique_ptr<GeomEntry>> geom_cache;
  const unsigned char *cur_masks = nullptr;  // the masks of the last window setup (in geom_cache)
};

// One grid level: N^3 cells of a cube of side `box` whose lower corner is x0.
struct Level {
  int n = 0;
  double box = 0, x0[3] = {0, 0, 0}, dx = 0;
  double periodic = 0;  // size of the periodic simulation domain (box of level 0)
  size_t ncomplex() const { return (size_t)n * n * (n / 2 + 1); }
  size_t ncells() const { return (size_t)n * n * n; }
  double kmin() const;
  // half-spectrum (complex) fields, element type by precision; in place with the
  // padded real layout of an r2c transform (row stride 2(n/2+1) reals)
  DevBuf noise;          // white noise (unit variance per real d.o.f.)
  DevBuf field[4];       // delta, psi_x, psi_y, psi_z
  DevBuf sqrtp;          // double sqrt(P_grid) per integer |k|^2
  DevBuf sqrtp_dm;       // the same with the dark-matter transfer column
  DevBuf tab_main;       // sqrt(P_grid), times the high-pass filter on zoom levels
  DevBuf tab_lp_src;     // sqrt(P_grid) * low-pass (source side of the next zoom)
  DevBuf tab_lp;         // low-pass filter alone
  DevBuf tab_main_f, tab_lp_src_f, tab_lp_f;  // float copies of the three (float fields)
  DevBuf field2[3];      // second-order displacements psi2_x, psi2_y, psi2_z (real)
  DevBuf pos, vel;       // particles: pos double[3M], vel (precision)[3M]
  // asynchronous fetches (gic_fetch_particles_async): while one may still be reading pos/vel,
  // the next particles go to the other pair (swapped in); `fetched` is recorded on the copy
  // stream after a fetch of the current pair, fetched_alt likewise for the other pair
  DevBuf pos_alt, vel_alt;
  cudaEvent_t fetched = nullptr, fetched_alt = nullptr;
  bool fetching = false, fetching_alt = false;
  bool have_noise = false;
  bool have_fields = false;  // displacements in real space
  bool have_delta = false;   // delta in real space (made on demand)
  bool have_lpt2 = false;
  Level() = default;
  Level(const Level &) = delete;
  Level &operator=(const Level &) = delete;
  ~Level() {
    if (fetched) cudaEventDestroy(fetched);
    if (fetched_alt) cudaEventDestroy(fetched_alt);
  }
};

struct Cosmo {
  double om, ol, ob, h, s8, ns, z, a;
};

// Device-resident transfer function: natural cubic spline of ln T vs ln k.
struct Transfer {
  int nrows = 0;
  DevBuf lnk, lnT_all, c_all, lnT_dm, c_dm;  // doubles
  double lnk_min = 0, lnk_max = 0;
  double amplitude = 0;  // (sigma8/sigma8_pre * D(a)/D(1))^2
  double sigma8_pre = 0;
  bool ready = false;
  // FNV-1a hash of the table and the cosmology it was normalised with: a repeated
  // gic_set_transfer with the same inputs finds the state already built
  uint64_t inputs_hash = 0;
};

struct FftTables {
  // twiddles w^m = exp(-2 pi i m / n), m < n, per size and precision
  struct Entry {
    int n;
    DevBuf f32, f64;
  };
  std::vector<std::unique_ptr<Entry>> entries;
  const void *get(int n, bool dbl, cudaStream_t s);
  // tile widths of the fixed-length passes chosen by timing the candidates on
  // first use, per size and precision (the choice does not change any result)
  // planes: variant of the plane pass that replaces the y and z passes, or -1 (none)
  struct Tuned {
    int n;
    bool dbl;
    int cols, rows, planes;
  };
  std::vector<Tuned> tuned;
  int force_cols = -1, force_rows = -1;  // >= 0: use this candidate (tests)
  int force_planes = -2;                 // -2: tuned, -1: separate y and z passes, >= 0: this variant
  bool col_tables = true;                // false: x passes gather their multipliers by |k|^2
  // plane pass: N plane counters and a ticket, zeroed before each launch; a word of
  // mapped host memory the kernel sets when one of its waits gives up
  DevBuf plane_sync;
  int *wait_flag_host = nullptr, *wait_flag_dev = nullptr;
  // polls per wait before it gives up (100 ns apart: about 0.4 s), and a count added to
  // each wait's target (0; tests set 1 so that no wait can finish)
  unsigned plane_spin_limit = 1u << 22;
  unsigned plane_wait_extra = 0;
  int *wait_flag();
  FftTables() = default;
  FftTables(const FftTables &) = delete;
  FftTables &operator=(const FftTables &) = delete;
  ~FftTables() {
    if (wait_flag_host) cudaFreeHost(wait_flag_host);
  }
};

struct RngScratch {
  DevBuf raw, gauss, owner, segtab, segentry, segbase, blkmap, blkentry, blkbase, streams, chunkmul, flags, tailq;
  int chunkmul_count = 0;
};

// A box of an n^3 grid's cells: per axis the cyclic range [start, start + len) mod n.
// Given to a forward transform, its input is zero outside the box; given to an
// inverse transform, only its output inside the box is wanted.  The fixed-length
// transforms then skip the x planes and y rows outside it (the z range is not used);
// the values they produce for the box are the same bits as the whole transform's.
struct CellBox {
  int start[3] = {0, 0, 0}, len[3] = {0, 0, 0};
  static CellBox whole(int n) {
    CellBox b;
    for (int a = 0; a < 3; ++a) b.len[a] = n;
    return b;
  }
  // per axis [lo - margin, hi + margin) of a cyclic axis of n cells (any lo, hi)
  void set_axis(int a, long long lo, long long hi, int margin, int n) {
    long long len_ = hi - lo + 2ll * margin;
    if (len_ >= n || len_ <= 0) {
      start[a] = 0;
      len[a] = n;
      return;
    }
    start[a] = (int)((((lo - margin) % n) + n) % n);
    len[a] = (int)len_;
  }
};
// a linear modification awaiting application (kind 0 overdensity, 1-3 velocity x,y,z)
// geometry derived from the levels alone (window masks, deinterpolation axes), kept per key
struct GeomEntry {
  std::vector<double> key;
  DevBuf dev, aux;
  std::vector<int> host;
  CellBox box;
  int umin[3] = {0, 0, 0}, ncu[3] = {0, 0, 0}, roff[3] = {0, 0, 0};  // per-axis tables in aux
};
struct ModRequest {
  int kind;
  std::vector<unsigned long long> cells;  // flagged cells of the finest level
  double target;
  // made at first use and kept: the cells on the device, their box on the finest level
  // (with the stencils' reach) and, for angular momenta, their wrapped centre
  std::shared_ptr<DevBuf> dcells;
  CellBox box;
  bool have_box = false;
  // the list position of every cell of `box` (-1 where not flagged), when the box is small
  // enough to hold one: the localisation kernels' lookups
  std::shared_ptr<DevBuf> dmap;
  double centre[3] = {0, 0, 0};
  bool have_centre = false;
};

// variance of the high-passed dark-matter overdensity over flagged cells
struct QuadRequest {
  std::vector<std::vector<unsigned long long>> cells;  // flagged cells per level (sorted)
  std::vector<std::unique_ptr<DevBuf>> dcells;         // their device copies
  double scale = 0, target = 0, precision = 0.001;
  int init_steps = 10;
};

// A per-|k|^2 table of the modification algebra, kept across calls: it depends on its
// specification (filters, scalars, level), on the transfer function and on the
// cosmology, so the cache is emptied when those or the levels change.
struct CachedTable {
  std::vector<unsigned char> key;
  DevBuf d, f;  // the table and its float copy
};

struct Context {
  MemAccount account;  // first: destroyed after every buffer charged to it
  int device = 0;
  // set while a batch captures this context's realisation into a CUDA graph: no host
  // synchronisation or host-memory copies; the noise draw's stream descriptors are
  // uploaded (upload_noise_streams) before each replay and its underrun flag read after
  bool defer_checks = false;
  int precision = GIC_FP64;
  cudaStream_t stream = nullptr;
  // copies of gic_fetch_particles_async, ordered after `stream` by copy_ready
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ready = nullptr;
  // small results (flags, inner products) come back through mapped pinned host memory that a
  // kernel writes: a cudaMemcpy would queue behind a large transfer on the copy engine
  struct Mapped {
    void *host = nullptr, *dev = nullptr;
    Mapped() = default;
    Mapped(const Mapped &) = delete;
    Mapped &operator=(const Mapped &) = delete;
    ~Mapped() {
      if (host) cudaFreeHost(host);
    }
  } readback;
  DevBuf small;  // scratch of reductions whose partial sums are read back
  // the device record buffers of asynchronous tipsy packs, and the copy that last read each
  DevBuf records[2];
  cudaEvent_t records_read[2] = {nullptr, nullptr};
  bool records_pending[2] = {false, false};
  int records_next = 0;
  std::string last_error;
  std::vector<std::unique_ptr<Level>> levels;
  Cosmo cosmo{};
  bool have_cosmo = false;
  Transfer transfer;
  FftTables fft;
  RngScratch rng;
  DevBuf reduce;  // small scratch for reductions
  DevBuf zoom_scratch[4];  // low-passed coarse fields during zoom combination
  DevBuf geom;             // per-axis interpolation / centroid tables
  DevBuf lpt2_tab, lpt2_tabt;  // the 2LPT multiplier table (double) and its typed copy
  std::vector<ModRequest> mods;
  std::vector<QuadRequest> quads;
  BufPool pool;
  ModScratch modscratch;
  std::vector<std::unique_ptr<CachedTable>> table_cache;
  // Per-coefficient layouts of per-|k|^2 tables for the x passes of power-of-two
  // transforms (n >= 256), built on first use by col_table (fft.cu).  The owner of a
  // registered table keeps it unchanged at its address until drop_col_tables drops the
  // registrations of its kind (`cache`: the modification algebra's cached tables).
  struct ColTable {
    const void *q = nullptr;
    int n = 0, elem = 0;
    bool cache = false;
    bool failed = false;  // no room for the layout: the x pass gathers from q
    DevBuf col;
  };
  std::vector<std::unique_ptr<ColTable>> col_tables;
  void register_col_table(const void *q, int n, int elem, bool cache) {
    if (!q || n < 256 || (n & (n - 1))) return;
    for (auto &e : col_tables)
      if (e->q == q && e->n == n && e->elem == elem) return;
    auto e = std::make_unique<ColTable>();
    e->q = q;
    e->n = n;
    e->elem = elem;
    e->cache = cache;
    col_tables.push_back(std::move(e));
  }
  void drop_col_tables(bool cache_only) {
    std::vector<std::unique_ptr<ColTable>> keep;
    for (auto &e : col_tables)
      if (cache_only && !e->cache) keep.push_back(std::move(e));
    col_tables.swap(keep);
  }
  void clear_table_cache() {
    drop_col_tables(true);
    table_cache.clear();
  }
  bool dbl() const { return precision == GIC_FP64; }
};

// (row, kz) of this thread's element of an n x n x (n/2 + 1) half spectrum, for a 1-D
// launch of hs_elements(n) threads: flat indexing gives every warp one contiguous
// span, so each sector is written whole by one warp (rows of n/2 + 1 coefficients
// are not sector-aligned, and a (row, kz-chunk) grid splits sectors between CTAs)
#ifdef __CUDACC__
__device__ __forceinline__ bool hs_cell(int n, unsigned &row, int &iz) {
  const unsigned S = (unsigned)(n / 2 + 1);
  const unsigned long long e = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned long long total = (unsigned long long)n * (unsigned long long)n * S;
  if (e >= total) return false;
  if (total <= 0xFFFFFFFFull) {
    const unsigned e32 = (unsigned)e;
    row = e32 / S;
    iz = (int)(e32 - row * S);
  } else {
    row = (unsigned)(e / S);
    iz = (int)(e - (unsigned long long)row * S);
  }
  return true;
}
#endif
inline unsigned long long hs_elements(int n) { return (unsigned long long)n * n * (n / 2 + 1); }

// A table of nq doubles in the fields' precision: the table itself (T = double) or a
// float copy made in `shadow` (T = float).  Float kernels read float tables: converting
// a double per element would occupy the FP64 pipe, a few percent of the FP32 rate.
template <typename T>
const T *typed_table(Context &ctx, DevBuf &shadow, const double *tab, size_t nq);
// the level tables in the fields' precision (their float copies are made with them)
// The per-coefficient layout col[f][ky (n/2 + 1) + kz] = q[|k|^2] (f = |kx| <= n/2) of a
// per-|k|^2 table q of an n^3 grid registered with Context::register_col_table, built on
// first use; nullptr where q is not registered or the layout has no room.
template <typename T>
const T *coefficient_table(Context &ctx, const T *q, int n);
template <typename T>
const T *tab_main(const Level &L);
template <typename T>
const T *tab_lp_src(const Level &L);
template <typename T>
const T *tab_lp(const Level &L);

// fft.cu
// cells of the coarse level that the fine level covers, `margin` extra cells each side
inline CellBox footprint_box(const Level &fine, const Level &coarse, int margin) {
  CellBox b = CellBox::whole(coarse.n);
  for (int a = 0; a < 3; ++a) {
    double rel = std::fmod(fine.x0[a] - coarse.x0[a], coarse.periodic);
    if (rel < 0) rel += coarse.periodic;
    const long long lo = (long long)std::floor(rel / coarse.dx);
    const long long hi = (long long)std::ceil((rel + (double)fine.n * fine.dx) / coarse.dx);
    b.set_axis(a, lo, hi, margin, coarse.n);
  }
  return b;
}
// pre_tab / post_tab: optional per-|k|^2 multiplier applied to the half spectrum
// before the inverse / after the forward transform, fused into the x pass; in the
// transform's precision (typed_table gives a float copy of a double table)
template <typename T>
void fft_c2r_3d(Context &ctx, T *data, int n, double scale, const T *pre_tab = nullptr,
                const CellBox *box = nullptr);
template <typename T>
void fft_r2c_3d(Context &ctx, T *data, int n, double scale, const T *post_tab = nullptr,
                const CellBox *box = nullptr);
// the inverse transform of src (unchanged) into dst: the first pass reads src, so no
// copy of the spectrum is made (the runtime-length passes copy, then transform)
template <typename T>
void fft_c2r_3d_from(Context &ctx, T *dst, const T *src, int n, double scale, const T *pre_tab = nullptr,
                     const CellBox *box = nullptr);
// dst = xtab[q] x + the forward transform of data (times post_tab); data is overwritten
// (the sum is formed by the x pass as it stores, one read and write of a field less than
// a separate multiply-add)
template <typename T>
void fft_r2c_3d_add(Context &ctx, T *data, int n, double scale, const T *post_tab, const CellBox *box, T *dst,
                    const T *x, const T *xtab);
// whether transforms of size n honour a box (the fixed-length passes), so that a forward
// transform reads only the box's x planes and its input need be valid there only
bool fft_prunes(const Context &ctx, int n);
// after the stream has synchronised: true (with ctx.last_error set) when a wait of the
// plane pass gave up since the last check; clears the flag
bool take_fft_wait_error(Context &ctx);

// rng.cu
void draw_noise_all(Context &ctx, unsigned long long seed, int mode);
void gaussian_stream(Context &ctx, unsigned long long seed, size_t n, double *host);

// kspace.cu
void transfer_setup(Context &ctx, const double *table, int nrows, int ncols);
void build_sqrtp_table(Context &ctx, Level &L);
void build_sqrtp_table_species(Context &ctx, Level &L, int dm);
// field masks of the real-space field maps (bit f: Level::field[f])
constexpr unsigned kFieldDelta = 1u, kFieldsPsi = 14u;
// Zel'dovich fields of a level in real space (the particles need the displacements
// only; delta is made on demand by ensure_delta), and the low-passed coarser level
// interpolated in (zoom levels)
void za_fields(Context &ctx, int level, unsigned mask = kFieldsPsi);
void zoom_combine(Context &ctx, int level, unsigned mask = kFieldsPsi);
// delta of every level in real space, if the displacements were computed since it last was
void ensure_delta(Context &ctx);
void lpt2_fields(Context &ctx);
// tab_main of level li (sqrt(P) times its high-pass) and the low-pass tables of a coarse level
void level_tables(Context &ctx, int li);
void noise_op(Context &ctx, int op, double param);
void preconditioner_table(Context &ctx, const Level &L, double power, DevBuf &out);
// splice every level's noise with a new real-space draw of new_seed (flagged cells
// per level keep the new field); returns the CG iterations per level
std::vector<int> splice(Context &ctx, unsigned long long new_seed, const std::vector<std::vector<unsigned long long>> &cells);
void lowpass_tables(Context &ctx, int coarse_index);

// zoom.cu
template <typename T, int NF>
void interp_add(Context &ctx, const Level &coarse, const T *const *src, const Level &fine, T *const *dst,
                bool assign = false);

// modify.cu
double modification_value(Context &ctx, ModRequest &m);
double noise_chi2(Context &ctx);
double variance_value(Context &ctx, QuadRequest &q);
void apply_modifications(Context &ctx, double *chi2_before, double *chi2_after);
// realisation maps on real-space white noise and their adjoints (device arrays, compact N^3)
void field_from_noise(Context &ctx, int level, int what, const void *const *noise, void *out);
void field_from_noise_adjoint(Context &ctx, int level, int what, const void *grad_out, void *const *grad_noise);
double variance_gradient(Context &ctx, QuadRequest &q, const void *const *noise, void *const *grad, bool exact);
void noise_real(Context &ctx, int level, void *out);

// particles.cu
double velocity_to_offset_ratio(const Cosmo &c);
void make_particles(Context &ctx, Level &L, int order = 1);
// asynchronous particle fetches: enqueue the copies of a level's particles on the copy
// stream; finish_fetches waits for every one and releases the buffer pairs
void fetch_particles_async(Context &ctx, Level &L, double *host_pos, void *host_vel);
void finish_fetches(Context &ctx);
// copies `bytes` (a multiple of 4, at most kReadbackBytes) of device memory to host memory
// through the mapped readback buffer, after the work queued on ctx.stream; synchronises
// ctx.stream.  Larger or unaligned reads use a plain copy.
constexpr size_t kReadbackBytes = 64 * 1024;
void read_small(Context &ctx, const void *dev, size_t bytes, void *host);
// the descriptors of the noise streams of (seed, mode) for the context's levels, in the
// layout a deferred draw was captured with, copied to the device on the context's stream
void upload_noise_streams(Context &ctx, unsigned long long seed, int mode);
// after a deferred draw: whether a stream ran short of raw numbers (the draw must be redone)
bool noise_underrun(Context &ctx);
// particles of a virtual grid over L's region: factor > 1 supersampled, < -1 subsampled
void resampled_particles(Context &ctx, const Level &L, int factor, double *host_pos, double *host_vel);
// the grafic writer's per-cell floats of one grid of its stack (see gic_grafic_pack)
void grafic_pack(Context &ctx, const gic_grafic_grid &g, int z0, int nz, float *host_vel, float *host_pos,
                 float *host_delta, unsigned long long *host_ids);
// particles of listed cells of a zoom level's resolution-matching grid (strays)
void matched_particles(Context &ctx, int level, const unsigned long long *cells, size_t count, double *pos,
                       double *vel);

}  // namespace gic

// the opaque handle of the C ABI
namespace gic {
// tipsy records (writers.cu)
unsigned long long tipsy_count(const gic_particle_map *m);
void tipsy_factors(const gic_particle_map *m, double omega_m, double hubble, double scalefactor, double box,
                   double *pos_factor, double *vel_factor, double *mass_factor);
void tipsy_pack_host(const gic_particle_map *m, const double *const *pos, const double *const *vel, unsigned long long first,
                     unsigned long long count, gic_tipsy_dark *out, int threads);
void gadget_pack_host(const gic_particle_map *m, const double *const *pos, const double *const *vel,
                      const int *level_types, unsigned long long first, unsigned long long count, float *pos_out,
                      float *vel_out, unsigned long long *ids, float *mass_out, int threads);
void gadget_pack_device(Context &C, const gic_particle_map *m, const int *level_types, unsigned long long first,
                        unsigned long long count, float *pos_out, float *vel_out, unsigned long long *ids,
                        float *mass_out);
// async: the copy to host_out is queued on the copy stream (pinned host_out, valid until
// finish_fetches); the records are packed into one of two device buffers, the next pack
// into the other (after, on the device, any copy still reading it)
void tipsy_pack_device(Context &C, const gic_particle_map *m, unsigned long long first, unsigned long long count,
                       gic_tipsy_dark *host_out, bool async = false);
// the message of the last failure of a call without a context (this thread)
std::string &host_error();
}  // namespace gic

struct gic_ctx {
  gic::Context impl;
};
