// C ABI entry points (include/gicgpu.h).  Each call validates its arguments,
// runs on the context's CUDA stream, synchronises before returning and turns
// every failure into a status code plus a message.
#include "gic_internal.h"
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <new>
#include <atomic>


namespace gic {

[[noreturn]] void fail(int code, const std::string &msg) { throw Error{code, msg}; }

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(e == cudaErrorMemoryAllocation ? GIC_ERR_OOM : GIC_ERR_CUDA,
         std::string(what) + ": " + cudaGetErrorString(e));
  }
}

static std::atomic<unsigned long long> g_launches{0};

void launched(int kernels) {
  cuda_check(cudaGetLastError(), "kernel launch");
  g_launches.fetch_add((unsigned long long)kernels, std::memory_order_relaxed);
}

unsigned long long launch_count() { return g_launches.load(); }
void count_launches(unsigned long long kernels) { g_launches.fetch_add(kernels, std::memory_order_relaxed); }

namespace {

template <typename T>
__global__ void k_unpad_real(const T *src, double *dst, int n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t m = (size_t)n * n * n;
  if (i >= m) return;
  size_t row = i / n, z = i % n;
  dst[i] = (double)src[row * (size_t)(2 * (n / 2 + 1)) + z];
}

template <typename T>
__global__ void k_to_double(const T *src, double *dst, size_t count) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dst[i] = (double)src[i];
}

template <typename T>
__global__ void k_from_double(const double *src, T *dst, size_t count) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dst[i] = (T)src[i];
}

// sum over the half spectrum of w |c|^2, w = 1 on the kz = 0, N/2 planes, else 2
template <typename T>
__global__ void k_chi2_partial(const T *c, int n, double *partial) {
  __shared__ double red[256];
  const int H = n / 2, S = H + 1;
  size_t nc = (size_t)n * n * S;
  double acc = 0;
  for (size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x; id < nc; id += (size_t)gridDim.x * blockDim.x) {
    int kz = (int)(id % S);
    double re = (double)c[2 * id], im = (double)c[2 * id + 1];
    double w = (kz == 0 || kz == H) ? 1.0 : 2.0;
    acc += w * (re * re + im * im);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

Level &level_at(Context &c, int level) {
  if (level < 0 || level >= (int)c.levels.size()) fail(GIC_ERR_INVALID_ARG, "no such level");
  return *c.levels[level];
}

void use_device(Context &c) { GIC_CUDA(cudaSetDevice(c.device)); }

template <typename T>
void fetch_typed(Context &c, Level &L, int what, double *host) {
  cudaStream_t s = c.stream;
  static thread_local DevBuf *unused = nullptr;
  (void)unused;
  if (what == GIC_FIELD_NOISE) {
    if (!L.have_noise) fail(GIC_ERR_NOT_READY, "white noise has not been drawn");
    size_t count = 2 * L.ncomplex();
    if (sizeof(T) == 8) {
      GIC_CUDA(cudaMemcpyAsync(host, L.noise.ptr, count * sizeof(double), cudaMemcpyDeviceToHost, s));
    } else {
      c.reduce.ensure(count * sizeof(double));
      k_to_double<T><<<(unsigned)((count + 255) / 256), 256, 0, s>>>(L.noise.as<T>(), c.reduce.as<double>(), count);
      launched();
      GIC_CUDA(cudaMemcpyAsync(host, c.reduce.ptr, count * sizeof(double), cudaMemcpyDeviceToHost, s));
    }
  } else {
    if (!L.have_fields) fail(GIC_ERR_NOT_READY, "fields have not been computed");
    if (what >= GIC_FIELD_PSI2_X && !L.have_lpt2) fail(GIC_ERR_NOT_READY, "second-order fields have not been computed");
    if (what == GIC_FIELD_DELTA) ensure_delta(c);
    DevBuf &src = what >= GIC_FIELD_PSI2_X ? L.field2[what - GIC_FIELD_PSI2_X] : L.field[what - GIC_FIELD_DELTA];
    size_t m = L.ncells();
    c.reduce.ensure(m * sizeof(double));
    k_unpad_real<T><<<(unsigned)((m + 255) / 256), 256, 0, s>>>(src.as<T>(), c.reduce.as<double>(), L.n);
    launched();
    GIC_CUDA(cudaMemcpyAsync(host, c.reduce.ptr, m * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  GIC_CUDA(cudaStreamSynchronize(s));
}

template <typename T>
void set_noise_typed(Context &c, Level &L, const double *host) {
  cudaStream_t s = c.stream;
  size_t count = 2 * L.ncomplex();
  L.noise.ensure(count * sizeof(T));
  if (sizeof(T) == 8) {
    GIC_CUDA(cudaMemcpyAsync(L.noise.ptr, host, count * sizeof(double), cudaMemcpyHostToDevice, s));
  } else {
    c.reduce.ensure(count * sizeof(double));
    GIC_CUDA(cudaMemcpyAsync(c.reduce.ptr, host, count * sizeof(double), cudaMemcpyHostToDevice, s));
    k_from_double<T><<<(unsigned)((count + 255) / 256), 256, 0, s>>>(c.reduce.as<double>(), L.noise.as<T>(), count);
    launched();
  }
  GIC_CUDA(cudaStreamSynchronize(s));
  L.have_noise = true;
  L.have_fields = false;
  L.have_lpt2 = false;
}

template <typename T>
double chi2_typed(Context &c, Level &L) {
  const int blocks = 256;
  c.small.ensure(blocks * sizeof(double));
  k_chi2_partial<T><<<blocks, 256, 0, c.stream>>>(L.noise.as<T>(), L.n, c.small.as<double>());
  launched();
  std::vector<double> h(blocks);
  read_small(c, c.small.ptr, blocks * sizeof(double), h.data());
  double s = 0;
  for (double v : h) s += v;
  return s;
}

thread_local std::string g_create_error;

}  // namespace

std::string &host_error() { return g_create_error; }

thread_local MemAccount *t_account = nullptr;
}  // namespace gic

using gic::Error;

#define API_BEGIN(ctxp)                                    \
  if (!(ctxp)) return GIC_ERR_INVALID_ARG;                 \
  gic::Context &C = (ctxp)->impl;                          \
  try {                                                    \
    gic::AccountScope account_scope_(C.account);           \
    gic::use_device(C);
#define API_END                                            \
  }                                                        \
  catch (const Error &e) {                                 \
    C.last_error = e.msg;                                  \
    return e.code;                                         \
  }                                                        \
  catch (const std::bad_alloc &) {                         \
    C.last_error = "host allocation failed";               \
    return GIC_ERR_OOM;                                    \
  }                                                        \
  catch (const std::exception &e) {                        \
    C.last_error = e.what();                               \
    return GIC_ERR_INTERNAL;                               \
  }                                                        \
  if (gic::take_fft_wait_error(C)) return GIC_ERR_TIMEOUT; \
  C.last_error.clear();                                    \
  return GIC_OK;

extern "C" {

int gic_create(gic_ctx **out, const gic_device_opts *opts) {
  if (!out) return GIC_ERR_INVALID_ARG;
  *out = nullptr;
  int precision = opts ? opts->precision : GIC_FP64;
  int device = opts ? opts->device : 0;
  if (precision != GIC_FP64 && precision != GIC_MIXED) {
    gic::g_create_error = "unknown precision form";
    return GIC_ERR_INVALID_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    gic::g_create_error = "no CUDA device available";
    return GIC_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) {
    gic::g_create_error = "device ordinal out of range";
    return GIC_ERR_INVALID_ARG;
  }
  gic_ctx *c = new (std::nothrow) gic_ctx;
  if (!c) return GIC_ERR_OOM;
  c->impl.device = device;
  c->impl.precision = precision;
  c->impl.account.limit = opts ? opts->mem_limit : 0;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->impl.stream, cudaStreamNonBlocking) != cudaSuccess) {
    gic::g_create_error = cudaGetErrorString(cudaGetLastError());
    delete c;
    return GIC_ERR_CUDA;
  }
  // GIC_FFT_TILE selects the FFT passes by hand instead of the tuner: "generic"
  // (runtime-length kernels), "<cols>,<rows>" (fixed-length tile candidates, separate
  // y and z passes) or "<cols>,<rows>,<plane variant>" (x pass, then the plane pass)
  if (const char *t = std::getenv("GIC_FFT_TILE")) {
    int a = -1, b = -1, p = -1;
    const int got = std::sscanf(t, "%d,%d,%d", &a, &b, &p);
    if (std::strcmp(t, "generic") == 0) {
      c->impl.fft.force_cols = -2;
    } else if (got >= 2 && a >= 0 && b >= 0) {
      c->impl.fft.force_cols = a;
      c->impl.fft.force_rows = b;
      c->impl.fft.force_planes = got == 3 && p >= 0 ? p : -1;
    }
  }
  // GIC_FFT_COLTAB=0: the x passes read their per-|k|^2 multipliers from the tables
  // themselves instead of the per-coefficient layouts (the same values)
  if (const char *t = std::getenv("GIC_FFT_COLTAB")) c->impl.fft.col_tables = std::strcmp(t, "0") != 0;
  *out = c;
  return GIC_OK;
}

int gic_launch_count(unsigned long long *count) {
  if (!count) return GIC_ERR_INVALID_ARG;
  *count = gic::g_launches.load();
  return GIC_OK;
}

int gic_set_fft_wait(gic_ctx *ctx, unsigned spin_limit, int unreachable) {
  if (!ctx) return GIC_ERR_INVALID_ARG;
  ctx->impl.fft.plane_spin_limit = spin_limit ? spin_limit : (1u << 22);
  ctx->impl.fft.plane_wait_extra = unreachable ? 1u : 0u;
  return GIC_OK;
}

int gic_fft_choice(gic_ctx *ctx, int n, int *cols, int *rows, int *planes) {
  if (!ctx) return GIC_ERR_INVALID_ARG;
  const gic::FftTables &F = ctx->impl.fft;
  const bool dbl = ctx->impl.dbl();
  if (F.force_cols >= 0 && F.force_rows >= 0) {  // pinned by GIC_FFT_TILE
    if (cols) *cols = F.force_cols;
    if (rows) *rows = F.force_rows;
    if (planes) *planes = F.force_planes >= -1 ? F.force_planes : -1;
    return GIC_OK;
  }
  for (const auto &t : F.tuned)
    if (t.n == n && t.dbl == dbl) {
      if (cols) *cols = F.force_cols >= 0 ? F.force_cols : t.cols;
      if (rows) *rows = F.force_rows >= 0 ? F.force_rows : t.rows;
      if (planes) *planes = F.force_planes >= -1 ? F.force_planes : t.planes;
      return GIC_OK;
    }
  return GIC_ERR_NOT_READY;
}

int gic_memory_use(gic_ctx *ctx, size_t *in_use, size_t *limit) {
  if (!ctx) return GIC_ERR_INVALID_ARG;
  if (in_use) *in_use = ctx->impl.account.used.load();
  if (limit) *limit = ctx->impl.account.limit;
  return GIC_OK;
}

int gic_get_stream(gic_ctx *ctx, void **stream) {
  if (!ctx || !stream) return GIC_ERR_INVALID_ARG;
  *stream = (void *)ctx->impl.stream;
  return GIC_OK;
}

int gic_destroy(gic_ctx *ctx) {
  if (!ctx) return GIC_OK;
  cudaSetDevice(ctx->impl.device);
  cudaStreamSynchronize(ctx->impl.stream);
  cudaStream_t s = ctx->impl.stream, cs = ctx->impl.copy_stream;
  cudaEvent_t ready = ctx->impl.copy_ready;
  cudaEvent_t rec[2] = {ctx->impl.records_read[0], ctx->impl.records_read[1]};
  if (cs) cudaStreamSynchronize(cs);
  delete ctx;  // frees device buffers
  cudaStreamDestroy(s);
  if (cs) cudaStreamDestroy(cs);
  if (ready) cudaEventDestroy(ready);
  for (cudaEvent_t e : rec)
    if (e) cudaEventDestroy(e);
  return GIC_OK;
}

const char *gic_last_error(const gic_ctx *ctx) {
  if (!ctx) return gic::g_create_error.c_str();
  return ctx->impl.last_error.c_str();
}

int gic_level_add(gic_ctx *ctx, double box, int n, double x0, double y0, double z0, int *level_id) {
  API_BEGIN(ctx)
  if (!(box > 0) || n < 2 || n % 2 || n > 2048) gic::fail(GIC_ERR_INVALID_ARG, "level needs box > 0 and an even n <= 2048");
  for (auto &L : C.levels)
    if (L->have_noise) gic::fail(GIC_ERR_NOT_READY, "Trying to initialize a grid after the random field was already drawn");
  auto L = std::make_unique<gic::Level>();
  L->n = n;
  L->box = box;
  L->x0[0] = x0;
  L->x0[1] = y0;
  L->x0[2] = z0;
  L->dx = box / n;
  L->periodic = C.levels.empty() ? box : C.levels[0]->periodic;
  C.levels.push_back(std::move(L));
  C.clear_table_cache();
  if (level_id) *level_id = (int)C.levels.size() - 1;
  API_END
}

int gic_set_cosmology(gic_ctx *ctx, const gic_cosmo *cosmo) {
  API_BEGIN(ctx)
  if (!cosmo) gic::fail(GIC_ERR_INVALID_ARG, "null cosmology");
  C.cosmo.om = cosmo->omega_m;
  C.cosmo.ol = cosmo->omega_lambda;
  C.cosmo.ob = cosmo->omega_b;
  C.cosmo.h = cosmo->hubble;
  C.cosmo.s8 = cosmo->sigma8;
  C.cosmo.ns = cosmo->ns;
  C.cosmo.z = cosmo->redshift;
  C.cosmo.a = 1. / (cosmo->redshift + 1.);
  C.have_cosmo = true;
  C.clear_table_cache();
  API_END
}

int gic_set_transfer(gic_ctx *ctx, const double *table, int nrows, int ncols) {
  API_BEGIN(ctx)
  if (!table) gic::fail(GIC_ERR_INVALID_ARG, "null table");
  gic::transfer_setup(C, table, nrows, ncols);
  API_END
}

int gic_get_normalisation(gic_ctx *ctx, double *amplitude, double *sigma8_unnormalised) {
  API_BEGIN(ctx)
  if (!C.transfer.ready) gic::fail(GIC_ERR_NOT_READY, "no transfer function");
  if (amplitude) *amplitude = C.transfer.amplitude;
  if (sigma8_unnormalised) *sigma8_unnormalised = C.transfer.sigma8_pre;
  API_END
}

int gic_draw_noise(gic_ctx *ctx, unsigned long seed, int mode) {
  API_BEGIN(ctx)
  if (C.levels.empty()) gic::fail(GIC_ERR_NOT_READY, "no grid levels");
  gic::draw_noise_all(C, seed, mode);
  for (auto &L : C.levels) L->have_fields = L->have_lpt2 = false;
  API_END
}

int gic_noise_op(gic_ctx *ctx, int op, double param) {
  API_BEGIN(ctx)
  if (op < GIC_NOISE_REVERSE || op > GIC_NOISE_UNIT_MODULUS) gic::fail(GIC_ERR_INVALID_ARG, "unknown noise operation");
  if (C.levels.empty()) gic::fail(GIC_ERR_NOT_READY, "no grid levels");
  gic::noise_op(C, op, param);
  API_END
}

int gic_gaussian_stream(gic_ctx *ctx, unsigned long seed, size_t n, double *host_dst) {
  API_BEGIN(ctx)
  if (!host_dst && n) gic::fail(GIC_ERR_INVALID_ARG, "null buffer");
  if (n) gic::gaussian_stream(C, seed, n, host_dst);
  API_END
}

int gic_set_noise(gic_ctx *ctx, int level, const double *host_src) {
  API_BEGIN(ctx)
  if (!host_src) gic::fail(GIC_ERR_INVALID_ARG, "null buffer");
  gic::Level &L = gic::level_at(C, level);
  if (C.dbl()) gic::set_noise_typed<double>(C, L, host_src);
  else gic::set_noise_typed<float>(C, L, host_src);
  API_END
}

int gic_zeldovich(gic_ctx *ctx, int order) {
  API_BEGIN(ctx)
  if (order != 1 && order != 2) gic::fail(GIC_ERR_INVALID_ARG, "order must be 1 (Zel'dovich) or 2 (2LPT)");
  if (C.levels.empty()) gic::fail(GIC_ERR_NOT_READY, "no grid levels");
  int nl = (int)C.levels.size();
  for (int l = 0; l < nl; ++l) gic::za_fields(C, l);
  for (int l = 1; l < nl; ++l) gic::zoom_combine(C, l);
  if (order == 2) gic::lpt2_fields(C);
  for (int l = 0; l < nl; ++l) gic::make_particles(C, *C.levels[l], order);
  GIC_CUDA(cudaStreamSynchronize(C.stream));
  API_END
}

int gic_fetch_level(gic_ctx *ctx, int level, int what, double *host_dst) {
  API_BEGIN(ctx)
  if (!host_dst) gic::fail(GIC_ERR_INVALID_ARG, "null buffer");
  if (what < GIC_FIELD_NOISE || what > GIC_FIELD_PSI2_Z) gic::fail(GIC_ERR_INVALID_ARG, "unknown field");
  gic::Level &L = gic::level_at(C, level);
  if (C.dbl()) gic::fetch_typed<double>(C, L, what, host_dst);
  else gic::fetch_typed<float>(C, L, what, host_dst);
  API_END
}

// calls without a context: failures reported through gic_last_error(NULL)
#define HOST_BEGIN try {
#define HOST_END                                           \
  }                                                        \
  catch (const Error &e) {                                 \
    gic::host_error() = e.msg;                             \
    return e.code;                                         \
  }                                                        \
  catch (const std::bad_alloc &) {                         \
    gic::host_error() = "host allocation failed";          \
    return GIC_ERR_OOM;                                    \
  }                                                        \
  catch (const std::exception &e) {                        \
    gic::host_error() = e.what();                          \
    return GIC_ERR_INTERNAL;                               \
  }                                                        \
  gic::host_error().clear();                               \
  return GIC_OK;

int gic_tipsy_count(const gic_particle_map *map, unsigned long long *count) {
  HOST_BEGIN
  if (!count) gic::fail(GIC_ERR_INVALID_ARG, "null count");
  *count = gic::tipsy_count(map);
  HOST_END
}

int gic_tipsy_factors(const gic_particle_map *map, double omega_m, double hubble, double scalefactor, double box,
                      double *pos_factor, double *vel_factor, double *mass_factor) {
  HOST_BEGIN
  gic::tipsy_factors(map, omega_m, hubble, scalefactor, box, pos_factor, vel_factor, mass_factor);
  HOST_END
}

int gic_tipsy_pack_host(const gic_particle_map *map, const double *const *pos, const double *const *vel,
                        unsigned long long first, unsigned long long count, gic_tipsy_dark *out, int threads) {
  HOST_BEGIN
  gic::tipsy_pack_host(map, pos, vel, first, count, out, threads);
  HOST_END
}

int gic_gadget_pack(gic_ctx *ctx, const gic_particle_map *map, const int *level_types, unsigned long long first,
                    unsigned long long count, float *pos_out, float *vel_out, unsigned long long *ids, float *mass_out) {
  API_BEGIN(ctx)
  gic::gadget_pack_device(C, map, level_types, first, count, pos_out, vel_out, ids, mass_out);
  API_END
}

int gic_gadget_pack_host(const gic_particle_map *map, const double *const *pos, const double *const *vel,
                         const int *level_types, unsigned long long first, unsigned long long count, float *pos_out,
                         float *vel_out, unsigned long long *ids, float *mass_out, int threads) {
  HOST_BEGIN
  gic::gadget_pack_host(map, pos, vel, level_types, first, count, pos_out, vel_out, ids, mass_out, threads);
  HOST_END
}

int gic_tipsy_pack(gic_ctx *ctx, const gic_particle_map *map, unsigned long long first, unsigned long long count,
                   gic_tipsy_dark *host_out) {
  API_BEGIN(ctx)
  gic::tipsy_pack_device(C, map, first, count, host_out);
  API_END
}

int gic_grafic_pack(gic_ctx *ctx, const gic_grafic_grid *grid, int z0, int nz, float *vel, float *pos, float *delta,
                    unsigned long long *ids) {
  API_BEGIN(ctx)
  if (!grid) gic::fail(GIC_ERR_INVALID_ARG, "null grid");
  gic::grafic_pack(C, *grid, z0, nz, vel, pos, delta, ids);
  API_END
}

int gic_tipsy_pack_async(gic_ctx *ctx, const gic_particle_map *map, unsigned long long first, unsigned long long count,
                         gic_tipsy_dark *host_out) {
  API_BEGIN(ctx)
  gic::tipsy_pack_device(C, map, first, count, host_out, true);
  API_END
}

int gic_fetch_particles(gic_ctx *ctx, int level, double *pos, double *vel) {
  API_BEGIN(ctx)
  gic::Level &L = gic::level_at(C, level);
  if (!L.pos.ptr) gic::fail(GIC_ERR_NOT_READY, "particles have not been generated");
  size_t m = L.ncells();
  if (pos) GIC_CUDA(cudaMemcpyAsync(pos, L.pos.ptr, 3 * m * sizeof(double), cudaMemcpyDeviceToHost, C.stream));
  if (vel) {
    if (C.dbl()) {
      GIC_CUDA(cudaMemcpyAsync(vel, L.vel.ptr, 3 * m * sizeof(double), cudaMemcpyDeviceToHost, C.stream));
    } else {
      C.reduce.ensure(3 * m * sizeof(double));
      gic::k_to_double<float><<<(unsigned)((3 * m + 255) / 256), 256, 0, C.stream>>>(L.vel.as<float>(),
                                                                                   C.reduce.as<double>(), 3 * m);
      gic::launched();
      GIC_CUDA(cudaMemcpyAsync(vel, C.reduce.ptr, 3 * m * sizeof(double), cudaMemcpyDeviceToHost, C.stream));
    }
  }
  GIC_CUDA(cudaStreamSynchronize(C.stream));
  API_END
}

int gic_fetch_particles_native(gic_ctx *ctx, int level, double *pos, void *vel) {
  API_BEGIN(ctx)
  gic::Level &L = gic::level_at(C, level);
  if (!L.pos.ptr) gic::fail(GIC_ERR_NOT_READY, "particles have not been generated");
  size_t m = L.ncells();
  if (pos) GIC_CUDA(cudaMemcpyAsync(pos, L.pos.ptr, 3 * m * sizeof(double), cudaMemcpyDeviceToHost, C.stream));
  if (vel)
    GIC_CUDA(cudaMemcpyAsync(vel, L.vel.ptr, 3 * m * (C.dbl() ? sizeof(double) : sizeof(float)),
                             cudaMemcpyDeviceToHost, C.stream));
  GIC_CUDA(cudaStreamSynchronize(C.stream));
  API_END
}

int gic_fetch_particles_async(gic_ctx *ctx, int level, double *pos, void *vel) {
  API_BEGIN(ctx)
  gic::fetch_particles_async(C, gic::level_at(C, level), pos, vel);
  API_END
}

int gic_fetch_wait(gic_ctx *ctx) {
  API_BEGIN(ctx)
  gic::finish_fetches(C);
  API_END
}

int gic_fetch_particles_resampled(gic_ctx *ctx, int level, int factor, double *pos, double *vel) {
  API_BEGIN(ctx)
  gic::Level &L = gic::level_at(C, level);
  if (!pos || !vel) gic::fail(GIC_ERR_INVALID_ARG, "null buffer");
  if (factor > -2 && factor < 2) gic::fail(GIC_ERR_INVALID_ARG, "factor must be >= 2 (supersample) or <= -2 (subsample)");
  const int s = factor > 0 ? factor : -factor;
  const long long nv = factor > 0 ? (long long)L.n * s : L.n / s;
  if (factor < 0 && L.n % s) gic::fail(GIC_ERR_INVALID_ARG, "subsampling factor must divide the level's cells per side");
  if (nv < 2 || nv % 2 || nv > 2048) gic::fail(GIC_ERR_INVALID_ARG, "resampled grid needs an even number of cells per side <= 2048");
  gic::resampled_particles(C, L, factor, pos, vel);
  API_END
}

int gic_fetch_particles_matched(gic_ctx *ctx, int level, const unsigned long long *cells, size_t n, double *pos,
                                double *vel) {
  API_BEGIN(ctx)
  gic::level_at(C, level);
  if (level < 1) gic::fail(GIC_ERR_INVALID_ARG, "a resolution-matching grid belongs to a zoom level (level >= 1)");
  if (n && (!cells || !pos || !vel)) gic::fail(GIC_ERR_INVALID_ARG, "null buffer");
  gic::matched_particles(C, level, cells, n, pos, vel);
  API_END
}

int gic_fft(gic_ctx *ctx, int level, int what, int dir) {
  API_BEGIN(ctx)
  gic::Level &L = gic::level_at(C, level);
  if (dir != -1 && dir != 1) gic::fail(GIC_ERR_INVALID_ARG, "dir must be -1 (forward) or +1 (inverse)");
  gic::DevBuf *buf = what == GIC_FIELD_NOISE ? &L.noise : (what >= GIC_FIELD_DELTA && what <= GIC_FIELD_PSI_Z ? &L.field[what - 1] : nullptr);
  if (!buf || !buf->ptr) gic::fail(GIC_ERR_NOT_READY, "field not allocated");
  if (what == GIC_FIELD_DELTA) {
    gic::ensure_delta(C);
    L.have_delta = false;  // transformed in place
  }
  double scale = 1.0 / std::pow((double)L.n, 1.5);
  if (C.dbl()) {
    if (dir < 0) gic::fft_r2c_3d<double>(C, buf->as<double>(), L.n, scale);
    else gic::fft_c2r_3d<double>(C, buf->as<double>(), L.n, scale);
  } else {
    if (dir < 0) gic::fft_r2c_3d<float>(C, buf->as<float>(), L.n, scale);
    else gic::fft_c2r_3d<float>(C, buf->as<float>(), L.n, scale);
  }
  GIC_CUDA(cudaStreamSynchronize(C.stream));
  API_END
}

int gic_fft_box(gic_ctx *ctx, int level, int what, int dir, const int *start, const int *len) {
  API_BEGIN(ctx)
  gic::Level &L = gic::level_at(C, level);
  if (dir != -1 && dir != 1) gic::fail(GIC_ERR_INVALID_ARG, "dir must be -1 (forward) or +1 (inverse)");
  if (!start || !len) gic::fail(GIC_ERR_INVALID_ARG, "null box");
  gic::DevBuf *buf = what == GIC_FIELD_NOISE ? &L.noise : (what >= GIC_FIELD_DELTA && what <= GIC_FIELD_PSI_Z ? &L.field[what - 1] : nullptr);
  if (!buf || !buf->ptr) gic::fail(GIC_ERR_NOT_READY, "field not allocated");
  if (what == GIC_FIELD_DELTA) {
    gic::ensure_delta(C);
    L.have_delta = false;  // transformed in place
  }
  gic::CellBox box;
  for (int a = 0; a < 3; ++a) {
    if (len[a] < 1 || len[a] > L.n) gic::fail(GIC_ERR_INVALID_ARG, "box lengths must be in [1, n]");
    box.set_axis(a, start[a], (long long)start[a] + len[a], 0, L.n);
  }
  double scale = 1.0 / std::pow((double)L.n, 1.5);
  if (C.dbl()) {
    if (dir < 0) gic::fft_r2c_3d<double>(C, buf->as<double>(), L.n, scale, nullptr, &box);
    else gic::fft_c2r_3d<double>(C, buf->as<double>(), L.n, scale, nullptr, &box);
  } else {
    if (dir < 0) gic::fft_r2c_3d<float>(C, buf->as<float>(), L.n, scale, nullptr, &box);
    else gic::fft_c2r_3d<float>(C, buf->as<float>(), L.n, scale, nullptr, &box);
  }
  GIC_CUDA(cudaStreamSynchronize(C.stream));
  API_END
}

int gic_chi2(gic_ctx *ctx, double *chi2) {
  API_BEGIN(ctx)
  if (!chi2) gic::fail(GIC_ERR_INVALID_ARG, "null output");
  if (C.levels.empty()) gic::fail(GIC_ERR_NOT_READY, "no grid levels");
  for (auto &L : C.levels)
    if (!L->have_noise) gic::fail(GIC_ERR_NOT_READY, "white noise has not been drawn");
  if (C.levels.size() == 1)
    *chi2 = C.dbl() ? gic::chi2_typed<double>(C, *C.levels[0]) : gic::chi2_typed<float>(C, *C.levels[0]);
  else
    *chi2 = gic::noise_chi2(C);
  API_END
}

static gic::ModRequest make_request(gic::Context &C, int kind, const unsigned long long *cells, size_t n) {
  if (kind < GIC_MOD_OVERDENSITY || kind > GIC_MOD_LZ) gic::fail(GIC_ERR_INVALID_ARG, "unknown modification");
  if (C.levels.empty()) gic::fail(GIC_ERR_NOT_READY, "no grid levels");
  if (!cells || n == 0)
    gic::fail(GIC_ERR_INVALID_ARG,
              "Linear modifications use exclusively information from the highest resolution grid but no cells have been "
              "flagged on this grid.");
  size_t m = C.levels.back()->ncells();
  for (size_t i = 0; i < n; ++i)
    if (cells[i] >= m) gic::fail(GIC_ERR_INVALID_ARG, "flagged cell outside the finest grid");
  gic::ModRequest r;
  r.kind = kind;
  // genetIC keeps its flagged cells sorted and unique; the covectors follow that order
  r.cells.assign(cells, cells + n);
  std::sort(r.cells.begin(), r.cells.end());
  r.cells.erase(std::unique(r.cells.begin(), r.cells.end()), r.cells.end());
  r.target = 0;
  return r;
}

int gic_calculate(gic_ctx *ctx, int kind, const unsigned long long *cells, size_t n, double *value) {
  API_BEGIN(ctx)
  if (!value) gic::fail(GIC_ERR_INVALID_ARG, "null output");
  gic::ModRequest r = make_request(C, kind, cells, n);
  *value = gic::modification_value(C, r);
  API_END
}

int gic_add_modification(gic_ctx *ctx, int kind, const unsigned long long *cells, size_t n, double target,
                         int relative) {
  API_BEGIN(ctx)
  gic::ModRequest r = make_request(C, kind, cells, n);
  r.target = relative ? target * gic::modification_value(C, r) : target;
  C.mods.push_back(std::move(r));
  API_END
}

int gic_clear_modifications(gic_ctx *ctx) {
  API_BEGIN(ctx)
  C.mods.clear();
  C.quads.clear();
  API_END
}

// checkFilterScale (quadraticmodification.hpp:131-153) and the per-level cell lists
static gic::QuadRequest make_quad_request(gic::Context &C, const unsigned long long *const *cells, const size_t *counts,
                                          double scale) {
  if (C.levels.empty()) gic::fail(GIC_ERR_NOT_READY, "no grid levels");
  if (!cells || !counts) gic::fail(GIC_ERR_INVALID_ARG, "null cell lists");
  if (scale < 0.0)
    gic::fail(GIC_ERR_INVALID_ARG,
              "Trying to calculate filtered variance without initialising variance filtering scale. Use "
              "filtering_scale command to do this.");
  if (scale < C.levels.back()->dx)
    gic::fail(GIC_ERR_INVALID_ARG, "Variance high-pass filtering scale is smaller than the smallest pixel size.");
  gic::QuadRequest q;
  q.scale = scale;
  for (size_t l = 0; l < C.levels.size(); ++l) {
    size_t m = C.levels[l]->ncells();
    if (counts[l] && !cells[l]) gic::fail(GIC_ERR_INVALID_ARG, "null cell list");
    std::vector<unsigned long long> v(cells[l], cells[l] + counts[l]);
    for (size_t i = 0; i < v.size(); ++i) {
      if (v[i] >= m) gic::fail(GIC_ERR_INVALID_ARG, "flagged cell outside its grid");
      if (i && v[i] <= v[i - 1]) gic::fail(GIC_ERR_INVALID_ARG, "flagged cells must be sorted and unique");
    }
    q.cells.push_back(std::move(v));
  }
  if (q.cells.back().empty())
    gic::fail(GIC_ERR_INVALID_ARG, "no cells have been flagged on the finest grid");
  return q;
}

int gic_splice(gic_ctx *ctx, unsigned long new_seed, const unsigned long long *const *cells, const size_t *counts,
               int *iterations) {
  API_BEGIN(ctx)
  if (C.levels.empty()) gic::fail(GIC_ERR_NOT_READY, "no grid levels");
  for (auto &L : C.levels)
    if (!L->have_noise) gic::fail(GIC_ERR_NOT_READY, "white noise has not been drawn");
  if (!C.transfer.ready) gic::fail(GIC_ERR_NOT_READY, "no transfer function");
  if (!cells || !counts) gic::fail(GIC_ERR_INVALID_ARG, "null cell lists");
  std::vector<std::vector<unsigned long long>> lists;
  for (size_t l = 0; l < C.levels.size(); ++l) {
    if (counts[l] && !cells[l]) gic::fail(GIC_ERR_INVALID_ARG, "null cell list");
    std::vector<unsigned long long> v(cells[l], cells[l] + counts[l]);
    for (auto c : v)
      if (c >= C.levels[l]->ncells()) gic::fail(GIC_ERR_INVALID_ARG, "flagged cell outside its grid");
    lists.push_back(std::move(v));
  }
  std::vector<int> its = gic::splice(C, new_seed, lists);
  if (iterations)
    for (size_t l = 0; l < its.size(); ++l) iterations[l] = its[l];
  API_END
}

int gic_calculate_variance(gic_ctx *ctx, const unsigned long long *const *cells, const size_t *counts,
                           double filterscale, double *value) {
  API_BEGIN(ctx)
  if (!value) gic::fail(GIC_ERR_INVALID_ARG, "null output");
  gic::QuadRequest q = make_quad_request(C, cells, counts, filterscale);
  *value = gic::variance_value(C, q);
  API_END
}

int gic_add_variance_modification(gic_ctx *ctx, const unsigned long long *const *cells, const size_t *counts,
                                  double filterscale, double target, int relative, int init_steps, double precision) {
  API_BEGIN(ctx)
  if (init_steps < 2) gic::fail(GIC_ERR_INVALID_ARG, "init_steps must be at least 2");
  if (!(precision > 0)) gic::fail(GIC_ERR_INVALID_ARG, "precision must be positive");
  gic::QuadRequest q = make_quad_request(C, cells, counts, filterscale);
  q.init_steps = init_steps;
  q.precision = precision;
  q.target = relative ? target * gic::variance_value(C, q) : target;
  C.quads.push_back(std::move(q));
  API_END
}

int gic_noise_real(gic_ctx *ctx, int level, void *dev_out) {
  API_BEGIN(ctx)
  if (!dev_out) gic::fail(GIC_ERR_INVALID_ARG, "null output");
  gic::level_at(C, level);
  gic::noise_real(C, level, dev_out);
  API_END
}

static void check_device_arrays(gic::Context &C, const void *const *a, const char *what) {
  if (!a) gic::fail(GIC_ERR_INVALID_ARG, std::string("null ") + what);
  for (size_t l = 0; l < C.levels.size(); ++l)
    if (!a[l]) gic::fail(GIC_ERR_INVALID_ARG, std::string("null ") + what + " array of a level");
}

int gic_field_from_noise(gic_ctx *ctx, int level, int what, const void *const *dev_noise, void *dev_out) {
  API_BEGIN(ctx)
  if (!C.transfer.ready) gic::fail(GIC_ERR_NOT_READY, "no transfer function");
  check_device_arrays(C, dev_noise, "noise");
  if (!dev_out) gic::fail(GIC_ERR_INVALID_ARG, "null output");
  gic::field_from_noise(C, level, what - GIC_FIELD_DELTA, dev_noise, dev_out);
  API_END
}

int gic_field_from_noise_adjoint(gic_ctx *ctx, int level, int what, const void *dev_grad_out,
                                 void *const *dev_grad_noise) {
  API_BEGIN(ctx)
  if (!C.transfer.ready) gic::fail(GIC_ERR_NOT_READY, "no transfer function");
  check_device_arrays(C, dev_grad_noise, "gradient");
  if (!dev_grad_out) gic::fail(GIC_ERR_INVALID_ARG, "null input");
  gic::field_from_noise_adjoint(C, level, what - GIC_FIELD_DELTA, dev_grad_out, dev_grad_noise);
  API_END
}

int gic_variance_gradient(gic_ctx *ctx, const unsigned long long *const *cells, const size_t *counts,
                          double filterscale, const void *const *dev_noise, void *const *dev_grad, int exact,
                          double *value) {
  API_BEGIN(ctx)
  if (!value) gic::fail(GIC_ERR_INVALID_ARG, "null output");
  check_device_arrays(C, dev_noise, "noise");
  check_device_arrays(C, dev_grad, "gradient");
  gic::QuadRequest q = make_quad_request(C, cells, counts, filterscale);
  *value = gic::variance_gradient(C, q, dev_noise, dev_grad, exact != 0);
  API_END
}

int gic_apply_modifications(gic_ctx *ctx, double *chi2_before, double *chi2_after) {
  API_BEGIN(ctx)
  if (C.mods.empty() && C.quads.empty()) gic::fail(GIC_ERR_NOT_READY, "no modifications to apply");
  gic::apply_modifications(C, chi2_before, chi2_after);
  API_END
}

}  // extern "C"
