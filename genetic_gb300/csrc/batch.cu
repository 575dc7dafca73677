// Batches of independent realisations on one GPU (no genetIC counterpart: the
// reference realises one set of initial conditions per process).
//
// Each context of a batch keeps its own stream and buffers.  The whole realisation of
// every context -- white noise, linear modifications, Zel'dovich (or 2LPT) spectra,
// inverse FFTs, zoom combination and particles -- is one CUDA graph, captured on the
// first call (after one eager realisation, which allocates every buffer, tunes the FFTs
// and caches the geometry) with a fork from an origin stream to each context's stream
// and a join back, and replayed on later calls.  Nothing in it goes to the host: the
// Gram-Schmidt of the modifications runs on the device, the noise streams' descriptors
// (which carry the seeds) are copied to the device before each replay, and the RNG's
// underrun flag is read after it (a context whose stream ran short is realised again
// eagerly, with a longer stream).  The graph holds device pointers: a signature of
// them, of the seeding modes, the order, the modifications and of every buffer the
// contexts have freed since is checked before each replay, and the graph is captured
// again when any changed.  Contexts with a quadratic (variance) modification, whose
// iteration count is a host decision, are realised eagerly by host threads beside it.
#include "gic_internal.h"
#include <atomic>
#include <cstring>
#include <mutex>
#include <new>
#include <thread>

struct gic_batch {
  std::vector<gic_ctx *> ctxs;
  int device = 0;
  cudaStream_t origin = nullptr;
  cudaEvent_t start = nullptr;
  std::vector<cudaEvent_t> done;
  cudaGraphExec_t exec = nullptr;
  std::vector<uintptr_t> signature;
  std::vector<int> in_graph;  // the contexts the graph realises
  unsigned long long graph_kernels = 0;
  int replays = 0;         // graph launches since the last capture
  int failed_captures = 0;
  std::string graph_off;   // why the batch stopped capturing (a capture that failed)
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
  // a buffer that existed when the graph was captured, freed since (a regrowth or a
  // release), may be one the graph uses
  sig.push_back((uintptr_t)C.account.frees.load());
  sig.push_back((uintptr_t)C.mods.size());
  for (auto &m : C.mods) {
    uintptr_t bits;
    static_assert(sizeof(bits) >= sizeof(double), "pointer-sized signature entries");
    std::memcpy(&bits, &m.target, sizeof(double));
    sig.push_back(bits);
  }
}

void field_maps(Context &C, int order) {
  AccountScope scope(C.account);
  const int nl = (int)C.levels.size();
  for (int l = 0; l < nl; ++l) za_fields(C, l);
  for (int l = 1; l < nl; ++l) zoom_combine(C, l);
  if (order == 2) lpt2_fields(C);
  for (int l = 0; l < nl; ++l) make_particles(C, *C.levels[l], order);
}

// one realisation: noise, modifications, fields and particles
void realise_one(Context &C, unsigned long long seed, int mode, int order) {
  AccountScope scope(C.account);
  cuda_check(cudaSetDevice(C.device), "cudaSetDevice");
  if (C.levels.empty()) fail(GIC_ERR_NOT_READY, "a context of the batch has no grid levels");
  draw_noise_all(C, seed, mode);
  for (auto &L : C.levels) L->have_fields = L->have_lpt2 = false;
  if (!C.mods.empty() || !C.quads.empty()) apply_modifications(C, nullptr, nullptr);
  field_maps(C, order);
}

// whether a context's realisation can be captured: linear modifications only (their
// coefficients are formed on the device)
bool capturable(const Context &C) { return C.quads.empty() && C.mods.size() <= 16; }

// Captures the realisations of b.in_graph; false (and no graph) when a buffer was freed
// during the capture (a scratch buffer that grew): the graph could hold its pointer.
bool capture(gic_batch &b, const std::vector<int> &modes, int order) {
  release_graph(b);
  std::vector<unsigned long long> frees0;
  for (int i : b.in_graph) {
    MemAccount &a = b.ctxs[i]->impl.account;
    a.graph_serial = ~0ull;  // during the capture every free counts
    frees0.push_back(a.frees.load());
  }
  cudaEvent_t fork;
  GIC_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  const unsigned long long k0 = launch_count();
  GIC_CUDA(cudaStreamBeginCapture(b.origin, cudaStreamCaptureModeRelaxed));
  try {
    GIC_CUDA(cudaEventRecord(fork, b.origin));
    for (int i : b.in_graph) {
      Context &C = b.ctxs[i]->impl;
      GIC_CUDA(cudaStreamWaitEvent(C.stream, fork, 0));
      C.defer_checks = true;
      // the seed does not matter here: the streams' descriptors are copied before each replay
      realise_one(C, 0, modes[i], order);
      C.defer_checks = false;
      GIC_CUDA(cudaEventRecord(b.done[i], C.stream));
      GIC_CUDA(cudaStreamWaitEvent(b.origin, b.done[i], 0));
    }
  } catch (...) {
    for (auto *c : b.ctxs) c->impl.defer_checks = false;
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(b.origin, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    cudaEventDestroy(fork);
    count_launches(0ull - (launch_count() - k0));
    throw;
  }
  cudaGraph_t g = nullptr;
  GIC_CUDA(cudaStreamEndCapture(b.origin, &g));
  bool stable = true;
  for (size_t k = 0; k < b.in_graph.size(); ++k)
    stable = stable && b.ctxs[b.in_graph[k]]->impl.account.frees.load() == frees0[k];
  if (!stable) {
    cudaGraphDestroy(g);
    cudaEventDestroy(fork);
    count_launches(0ull - (launch_count() - k0));
    return false;
  }
  cudaError_t e = cudaGraphInstantiate(&b.exec, g, 0);
  cudaGraphDestroy(g);
  cudaEventDestroy(fork);
  GIC_CUDA(e);
  // from now on only buffers that existed during the capture can invalidate the graph
  for (int i : b.in_graph) {
    MemAccount &a = b.ctxs[i]->impl.account;
    a.graph_serial = a.serial.load();
  }
  // the launches recorded during capture ran nothing yet
  b.graph_kernels = launch_count() - k0;
  count_launches(0ull - b.graph_kernels);
  return true;
}

std::vector<uintptr_t> batch_signature(const gic_batch &b, const std::vector<int> &modes, int order) {
  std::vector<uintptr_t> sig{(uintptr_t)order};
  for (int i : b.in_graph) {
    sig.push_back((uintptr_t)i);
    sig.push_back((uintptr_t)modes[i]);
    append_signature(b.ctxs[i]->impl, sig);
  }
  return sig;
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

GIC_API int gic_batch_graph_info(const gic_batch *b, int *contexts, unsigned long long *kernels, int *replays,
                                 const char **off_reason) {
  if (!b) return GIC_ERR_INVALID_ARG;
  if (contexts) *contexts = b->exec ? (int)b->in_graph.size() : 0;
  if (kernels) *kernels = b->exec ? b->graph_kernels : 0;
  if (replays) *replays = b->replays;
  if (off_reason) *off_reason = b->graph_off.c_str();
  return GIC_OK;
}

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
  std::vector<int> mode(n);
  for (int i = 0; i < n; ++i) {
    mode[i] = modes ? modes[i] : GIC_SEED_FOURIER_PARALLEL;
    if (mode[i] < 0 || mode[i] > 3) {
      b->last_error = "unknown seeding mode";
      return GIC_ERR_INVALID_ARG;
    }
  }
  std::vector<int> in_graph, eager;
  for (int i = 0; i < n; ++i)
    (b->graph_off.empty() && gic::capturable(b->ctxs[i]->impl) ? in_graph : eager).push_back(i);
  std::mutex err_mutex;
  int err_code = GIC_OK;
  std::string err_msg;
  auto record = [&](int code, const std::string &msg) {
    std::lock_guard<std::mutex> lock(err_mutex);
    if (err_code == GIC_OK) {
      err_code = code;
      err_msg = msg;
    }
  };
  // realisations one context at a time per host thread, each on its context's stream
  auto run_eager = [&](const std::vector<int> &which) {
    std::atomic<int> next{0};
    auto worker = [&]() {
      for (;;) {
        const int k = next.fetch_add(1);
        if (k >= (int)which.size()) return;
        const int i = which[k];
        gic::Context &C = b->ctxs[i]->impl;
        try {
          gic::realise_one(C, seeds[i], mode[i], order);
        } catch (const gic::Error &e) {
          record(e.code, e.msg);
        } catch (const std::exception &e) {
          record(GIC_ERR_CUDA, e.what());
        }
      }
    };
    const int nt = std::max(1, std::min(threads, (int)which.size()));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
  };
  try {
    gic::cuda_check(cudaSetDevice(b->device), "cudaSetDevice");
    // asynchronous particle fetches end first: the realisations write the particle buffers
    for (auto *c : b->ctxs) {
      gic::AccountScope scope(c->impl.account);
      gic::finish_fetches(c->impl);
    }
    bool replay = false;
    if (!in_graph.empty()) {
      b->in_graph = in_graph;
      const std::vector<uintptr_t> sig = gic::batch_signature(*b, mode, order);
      replay = b->exec && sig == b->signature;
      if (replay) {
        for (int i : in_graph) {
          gic::Context &C = b->ctxs[i]->impl;
          gic::AccountScope scope(C.account);
          gic::upload_noise_streams(C, seeds[i], mode[i]);
        }
        gic::cuda_check(cudaGraphLaunch(b->exec, b->origin), "cudaGraphLaunch");
        gic::count_launches(b->graph_kernels);
        ++b->replays;
      }
    }
    // contexts outside the graph (and, before the first capture, all of them) eagerly
    run_eager(replay ? eager : [&] {
      std::vector<int> all(n);
      for (int i = 0; i < n; ++i) all[i] = i;
      return all;
    }());
    if (err_code != GIC_OK) {
      for (auto *c : b->ctxs) cudaStreamSynchronize(c->impl.stream);
      cudaStreamSynchronize(b->origin);
      b->last_error = err_msg;
      return err_code;
    }
    gic::cuda_check(cudaStreamSynchronize(b->origin), "cudaStreamSynchronize");
    for (auto *c : b->ctxs) gic::cuda_check(cudaStreamSynchronize(c->impl.stream), "cudaStreamSynchronize");
    if (replay) {
      // a stream that ran short of raw numbers: that realisation again, with a longer stream
      for (int i : in_graph)
        if (gic::noise_underrun(b->ctxs[i]->impl)) gic::realise_one(b->ctxs[i]->impl, seeds[i], mode[i], order);
    } else if (!in_graph.empty()) {
      // every buffer now exists: capture the realisations of the graph's contexts.  The
      // realisations are already complete, so a capture that fails only ends capturing.
      try {
        if (gic::capture(*b, mode, order)) {
          b->signature = gic::batch_signature(*b, mode, order);
          b->replays = 0;
        } else if (++b->failed_captures >= 3) {
          b->graph_off = "scratch buffers were reallocated during three captures";
        }
      } catch (const gic::Error &e) {
        gic::release_graph(*b);
        b->graph_off = e.msg.empty() ? "stream capture failed" : e.msg;
      } catch (const std::exception &e) {
        gic::release_graph(*b);
        b->graph_off = e.what();
      }
    }
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
  } catch (const std::bad_alloc &) {
    b->last_error = "host allocation failed";
    return GIC_ERR_OOM;
  } catch (const std::exception &e) {
    b->last_error = e.what();
    return GIC_ERR_INTERNAL;
  }
  return GIC_OK;
}

}  // extern "C"
