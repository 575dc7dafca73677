// Batches of independent realisations on one GPU (no genetIC counterpart: the
// reference realises one set of initial conditions per process).
//
// Each context of a batch keeps its own stream and buffers.  One call of
// gic_batch_realise draws every context's white noise and applies its queued
// modifications from a pool of host threads (these steps take host decisions:
// the RNG's segment retries, the Gram-Schmidt scalars), then runs the field maps
// of every context -- Zel'dovich spectra, inverse FFTs, zoom combination and
// particles -- as one CUDA graph: captured once, with a fork from an origin stream
// to each context's stream and a join back, and replayed on later calls.  Small
// realisations then overlap on the GPU instead of queueing behind one another,
// and the ~10^2 kernel launches of each are one graph launch.  The graph holds the
// contexts' device pointers; a signature of those pointers is checked before
// every replay and the graph is captured again when any changed.  Second-order
// (2LPT) fields use pooled scratch and run eagerly from the worker threads.
#include "gic_internal.h"
#include <atomic>
#include <mutex>
#include <thread>

struct gic_batch {
  std::vector<gic_ctx *> ctxs;
  int device = 0;
  cudaStream_t origin = nullptr;
  cudaEvent_t start = nullptr;
  std::vector<cudaEvent_t> done;
  cudaGraphExec_t exec = nullptr;
  std::vector<uintptr_t> signature;
  unsigned long long graph_kernels = 0;
  std::string last_error;
};

namespace gic {
namespace {

void release_graph(gic_batch &b) {
  if (b.exec) cudaGraphExecDestroy(b.exec);
  b.exec = nullptr;
  b.signature.clear();
}

// every device pointer the order-1 field maps of a context touch
void append_signature(const Context &C, std::vector<uintptr_t> &sig) {
  sig.push_back((uintptr_t)C.precision);
  sig.push_back((uintptr_t)C.levels.size());
  for (auto &L : C.levels) {
    for (const DevBuf *d : {&L->noise, &L->field[0], &L->field[1], &L->field[2], &L->field[3], &L->sqrtp,
                            &L->tab_main, &L->tab_lp_src, &L->tab_lp, &L->pos, &L->vel})
      sig.push_back((uintptr_t)d->ptr);
    sig.push_back((uintptr_t)L->n);
  }
  for (int f = 0; f < 4; ++f) sig.push_back((uintptr_t)C.zoom_scratch[f].ptr);
  sig.push_back((uintptr_t)C.geom.ptr);
  for (auto &e : C.fft.entries) {
    sig.push_back((uintptr_t)e->f32.ptr);
    sig.push_back((uintptr_t)e->f64.ptr);
  }
  for (auto &t : C.fft.tuned) sig.push_back((uintptr_t)(t.n * 64 + t.cols * 8 + t.rows) * 16 + (uintptr_t)(t.planes + 1));
  sig.push_back((uintptr_t)C.fft.plane_sync.ptr);
  sig.push_back((uintptr_t)C.fft.wait_flag_dev);
}

void field_maps(Context &C, int order) {
  AccountScope scope(C.account);
  const int nl = (int)C.levels.size();
  for (int l = 0; l < nl; ++l) za_fields(C, l);
  for (int l = 1; l < nl; ++l) zoom_combine(C, l);
  if (order == 2) lpt2_fields(C);
  for (int l = 0; l < nl; ++l) make_particles(C, *C.levels[l], order);
}

void capture(gic_batch &b) {
  release_graph(b);
  cudaEvent_t fork;
  GIC_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  const unsigned long long k0 = launch_count();
  GIC_CUDA(cudaStreamBeginCapture(b.origin, cudaStreamCaptureModeRelaxed));
  try {
    GIC_CUDA(cudaEventRecord(fork, b.origin));
    for (size_t i = 0; i < b.ctxs.size(); ++i) {
      Context &C = b.ctxs[i]->impl;
      GIC_CUDA(cudaStreamWaitEvent(C.stream, fork, 0));
      field_maps(C, 1);
      GIC_CUDA(cudaEventRecord(b.done[i], C.stream));
      GIC_CUDA(cudaStreamWaitEvent(b.origin, b.done[i], 0));
    }
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(b.origin, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    cudaEventDestroy(fork);
    throw;
  }
  cudaGraph_t g = nullptr;
  GIC_CUDA(cudaStreamEndCapture(b.origin, &g));
  cudaError_t e = cudaGraphInstantiate(&b.exec, g, 0);
  cudaGraphDestroy(g);
  cudaEventDestroy(fork);
  GIC_CUDA(e);
  // the launches recorded during capture ran nothing yet
  b.graph_kernels = launch_count() - k0;
  count_launches(0ull - b.graph_kernels);
  for (auto *c : b.ctxs) append_signature(c->impl, b.signature);
}

}  // namespace
}  // namespace gic

extern "C" {

GIC_API int gic_batch_create(gic_batch **out, gic_ctx *const *ctxs, int n) {
  if (!out || !ctxs || n <= 0) return GIC_ERR_INVALID_ARG;
  *out = nullptr;
  auto b = new (std::nothrow) gic_batch;
  if (!b) return GIC_ERR_OOM;
  for (int i = 0; i < n; ++i) {
    if (!ctxs[i] || ctxs[i]->impl.device != ctxs[0]->impl.device) {
      delete b;
      return GIC_ERR_INVALID_ARG;
    }
    for (int j = 0; j < i; ++j)
      if (ctxs[j] == ctxs[i]) {
        delete b;
        return GIC_ERR_INVALID_ARG;
      }
    b->ctxs.push_back(ctxs[i]);
  }
  b->device = ctxs[0]->impl.device;
  b->done.resize(n, nullptr);
  bool ok = cudaSetDevice(b->device) == cudaSuccess &&
            cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->start, cudaEventDisableTiming) == cudaSuccess;
  for (int i = 0; ok && i < n; ++i) ok = cudaEventCreateWithFlags(&b->done[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    for (auto e : b->done)
      if (e) cudaEventDestroy(e);
    if (b->start) cudaEventDestroy(b->start);
    if (b->origin) cudaStreamDestroy(b->origin);
    delete b;
    return GIC_ERR_CUDA;
  }
  *out = b;
  return GIC_OK;
}

GIC_API int gic_batch_destroy(gic_batch *b) {
  if (!b) return GIC_OK;
  cudaSetDevice(b->device);
  gic::release_graph(*b);
  for (auto e : b->done) cudaEventDestroy(e);
  cudaEventDestroy(b->start);
  cudaStreamDestroy(b->origin);
  delete b;
  return GIC_OK;
}

GIC_API const char *gic_batch_last_error(const gic_batch *b) { return b ? b->last_error.c_str() : "null batch"; }

GIC_API int gic_batch_get_stream(gic_batch *b, void **stream) {
  if (!b || !stream) return GIC_ERR_INVALID_ARG;
  *stream = (void *)b->origin;
  return GIC_OK;
}

GIC_API int gic_batch_realise(gic_batch *b, const unsigned long *seeds, const int *modes, int order, int threads) {
  if (!b) return GIC_ERR_INVALID_ARG;
  if (!seeds || (order != 1 && order != 2)) {
    b->last_error = "seeds are required and order must be 1 or 2";
    return GIC_ERR_INVALID_ARG;
  }
  const int n = (int)b->ctxs.size();
  threads = std::max(1, std::min(threads, n));
  std::atomic<int> next{0};
  std::mutex err_mutex;
  int err_code = GIC_OK;
  std::string err_msg;
  try {
    gic::cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
    gic::cuda_check(cudaEventRecord(b->start, b->origin), "cudaEventRecord");
  } catch (const gic::Error &e) {
    b->last_error = e.msg;
    return e.code;
  }
  const bool use_graph = order == 1;
  // noise and modifications, one context at a time per worker, on the context's stream
  auto worker = [&]() {
    for (;;) {
      int i = next.fetch_add(1);
      if (i >= n) return;
      gic::Context &C = b->ctxs[i]->impl;
      try {
        gic::AccountScope scope(C.account);
        gic::cuda_check(cudaSetDevice(C.device), "cudaSetDevice");
        if (C.levels.empty()) gic::fail(GIC_ERR_NOT_READY, "a context of the batch has no grid levels");
        gic::cuda_check(cudaStreamWaitEvent(C.stream, b->start, 0), "cudaStreamWaitEvent");
        gic::draw_noise_all(C, seeds[i], modes ? modes[i] : GIC_SEED_FOURIER_PARALLEL);
        for (auto &L : C.levels) L->have_fields = L->have_lpt2 = false;
        if (!C.mods.empty() || !C.quads.empty()) gic::apply_modifications(C, nullptr, nullptr);
        if (!use_graph) gic::field_maps(C, order);
        gic::cuda_check(cudaEventRecord(b->done[i], C.stream), "cudaEventRecord");
      } catch (const gic::Error &e) {
        std::lock_guard<std::mutex> lock(err_mutex);
        if (err_code == GIC_OK) {
          err_code = e.code;
          err_msg = e.msg;
        }
      } catch (const std::exception &e) {
        std::lock_guard<std::mutex> lock(err_mutex);
        if (err_code == GIC_OK) {
          err_code = GIC_ERR_CUDA;
          err_msg = e.what();
        }
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(worker);
  worker();
  for (auto &t : pool) t.join();
  if (err_code != GIC_OK) {
    for (auto *c : b->ctxs) cudaStreamSynchronize(c->impl.stream);
    b->last_error = err_msg;
    return err_code;
  }
  try {
    for (int i = 0; i < n; ++i) gic::cuda_check(cudaStreamWaitEvent(b->origin, b->done[i], 0), "cudaStreamWaitEvent");
    if (use_graph) {
      std::vector<uintptr_t> sig;
      for (auto *c : b->ctxs) gic::append_signature(c->impl, sig);
      if (!b->exec || sig != b->signature) {
        // the first realisation of a context allocates its buffers and tunes its
        // FFTs: run the maps once outside the graph, then capture
        gic::cuda_check(cudaStreamSynchronize(b->origin), "cudaStreamSynchronize");
        for (auto *c : b->ctxs) {
          gic::field_maps(c->impl, 1);
          gic::cuda_check(cudaStreamSynchronize(c->impl.stream), "cudaStreamSynchronize");
        }
        gic::capture(*b);
      }
      gic::cuda_check(cudaGraphLaunch(b->exec, b->origin), "cudaGraphLaunch");
      gic::count_launches(b->graph_kernels);
      for (int i = 0; i < n; ++i) {
        gic::cuda_check(cudaEventRecord(b->done[i], b->origin), "cudaEventRecord");
        gic::cuda_check(cudaStreamWaitEvent(b->ctxs[i]->impl.stream, b->done[i], 0), "cudaStreamWaitEvent");
      }
    }
    gic::cuda_check(cudaStreamSynchronize(b->origin), "cudaStreamSynchronize");
    for (auto *c : b->ctxs)
      if (gic::take_fft_wait_error(c->impl)) gic::fail(GIC_ERR_TIMEOUT, c->impl.last_error);
    for (auto *c : b->ctxs)
      for (auto &L : c->impl.levels) {
        L->have_fields = true;
        L->have_delta = false;  // delta is made on demand from the new fields
        if (order == 2) L->have_lpt2 = true;
      }
  } catch (const gic::Error &e) {
    b->last_error = e.msg;
    return e.code;
  }
  return GIC_OK;
}

}  // extern "C"
