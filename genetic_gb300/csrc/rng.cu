// White-noise drawing on the device, reproducing genetIC's RandomFieldGenerator
// (genetIC/src/simulation/field/randomfieldgenerator.hpp:122-260) bit for bit:
//
//  1. one RANLUX stream per seed (ranlxs2: luxury 794 subtract-with-borrow steps
//     of base 2^24 per block of 24 delivered numbers, Luescher's seeding), split
//     into chunks of kChunkBlocks blocks; each chunk's start state comes from the
//     576-bit LCG jump (bigint576.h), then the thread steps the recurrence in
//     registers;
//  2. the ziggurat consumes 2, 3 or 4 numbers per attempt depending on the data,
//     so gaussian positions in the stream are found with speculative segment
//     walks: every segment of kSegLen numbers is walked from entry offsets
//     0..kSpec-1 in parallel, one thread per stream chains the segments
//     (entry of segment g+1 = exit of segment g), and a final walk writes each
//     gaussian at its index;
//  3. gaussian pairs are placed on Fourier modes in the reference's k-shell
//     order; where two draws hit one stored coefficient (Hermitian folding of
//     kz<0 and of modes with a zero component) the later draw wins, found with
//     an atomicMax over draw indices, then one write per winning draw.
#include "gic_internal.h"
#include <cuda.h>
#include "bigint576.h"
#include "ddlog.h"
#include "zig_tables.h"
#include <algorithm>
#include <cmath>
#include <mutex>

namespace gic {
namespace {

constexpr int kLux = 794;          // 24-bit steps per delivered block
constexpr int kChunkBlocks = 16;   // blocks per generator thread
constexpr int kSegLen = 1024;      // stream numbers per ziggurat segment
constexpr int kSpec = 8;           // speculative entry offsets per segment
constexpr int kSpecThreads = 128;  // segments per CTA of the speculative walk
constexpr int kBlockSegs = 64;     // segments per block of the two-level chain
constexpr uint32_t kUnderrun = 0xFFFFFFFFu;

// Ziggurat tables: doubles for the values, floats (the doubles rounded to nearest)
// for the slow-path decision.  Kernels that walk many segments copy them into shared
// memory; the occasional walk of step_segment reads them here.
struct ZigTab {
  unsigned int K[128];
  float Wf[128], Yf[129];
  double W[128], Y[129];
};
__device__ const ZigTab gZig = {GIC_ZIG_K_INIT, GIC_ZIG_WF_INIT, GIC_ZIG_YF_INIT, GIC_ZIG_W_INIT, GIC_ZIG_Y_INIT};

__device__ __forceinline__ void load_zig(ZigTab &t) {
  for (int i = threadIdx.x; i < 128; i += blockDim.x) {
    t.K[i] = gZig.K[i];
    t.W[i] = gZig.W[i];
    t.Y[i] = gZig.Y[i];
    t.Wf[i] = gZig.Wf[i];
    t.Yf[i] = gZig.Yf[i];
  }
  if (threadIdx.x == 0) {
    t.Y[128] = 0.0;
    t.Yf[128] = 0.0f;
  }
}

struct Stream {
  unsigned long long seed;
  unsigned long long raw_off, raw_count;      // numbers generated for this stream
  unsigned long long gauss_off, gauss_count;  // gaussians required
  unsigned long long seg_off;                 // first global segment
  unsigned long long chunk_off;               // first global generator chunk
  unsigned long long blk_off;                 // first global chain block
  unsigned int nseg, nchunk, nblk;
  U576 y0;
};

// ---- stream generation ------------------------------------------------------

__global__ void k_seed(Stream *st, int nstreams) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nstreams) return;
  uint32_t y[24];
  ranlux_seed_state(y, st[s].seed);
  u576_from_state(st[s].y0, y, 0);
}

// chunk multipliers a^(794 * kChunkBlocks * t) mod m, from the table of
// a^(794 * kChunkBlocks * 2^i)
__global__ void k_chunk_multipliers(U576 *out, int count, const U576 *pow2, int npow2) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  U576 acc;
  u576_zero(acc);
  acc.w[0] = 1;
  for (int i = 0; i < npow2; ++i)
    if ((t >> i) & 1) u576_mulmod(acc, acc, pow2[i]);
  out[t] = acc;
}

__device__ __forceinline__ int find_stream_by_chunk(const Stream *st, int nstreams, unsigned long long c) {
  int lo = 0, hi = nstreams - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (st[mid].chunk_off <= c) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int find_stream_by_block(const Stream *st, int nstreams, unsigned long long b) {
  int lo = 0, hi = nstreams - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (st[mid].blk_off <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int find_stream_by_segment(const Stream *st, int nstreams, unsigned long long g) {
  int lo = 0, hi = nstreams - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (st[mid].seg_off <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <int K>
__device__ __forceinline__ void swb_group(uint32_t (&y)[24], uint32_t &c) {
  // one step replacing slot K (the oldest word) by y_{n-10} - y_{n-24} - c
  int32_t d = (int32_t)y[(K + 14) % 24] - (int32_t)y[K] - (int32_t)c;
  c = (uint32_t)d >> 31;
  y[K] = (uint32_t)d & 0xFFFFFFu;
}

__device__ __forceinline__ void swb_24(uint32_t (&y)[24], uint32_t &c) {
  swb_group<0>(y, c);  swb_group<1>(y, c);  swb_group<2>(y, c);  swb_group<3>(y, c);
  swb_group<4>(y, c);  swb_group<5>(y, c);  swb_group<6>(y, c);  swb_group<7>(y, c);
  swb_group<8>(y, c);  swb_group<9>(y, c);  swb_group<10>(y, c); swb_group<11>(y, c);
  swb_group<12>(y, c); swb_group<13>(y, c); swb_group<14>(y, c); swb_group<15>(y, c);
  swb_group<16>(y, c); swb_group<17>(y, c); swb_group<18>(y, c); swb_group<19>(y, c);
  swb_group<20>(y, c); swb_group<21>(y, c); swb_group<22>(y, c); swb_group<23>(y, c);
}

__global__ void __launch_bounds__(128) k_generate(const Stream *st, int nstreams, unsigned long long nchunks,
                                                  const U576 *chunkmul, uint32_t *raw) {
  unsigned long long gc = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gc >= nchunks) return;
  int s = find_stream_by_chunk(st, nstreams, gc);
  unsigned long long t = gc - st[s].chunk_off;
  if (t >= st[s].nchunk) return;
  U576 Y;
  u576_mulmod(Y, st[s].y0, chunkmul[t]);
  uint32_t y[24];
  u576_to_state(y, Y);
  uint32_t c = 0;
  unsigned long long first = t * (unsigned long long)kChunkBlocks * 24ull;
  unsigned long long count = st[s].raw_count;
  uint32_t *dst = raw + st[s].raw_off;
  for (int b = 0; b < kChunkBlocks; ++b) {
    unsigned long long base = first + (unsigned long long)b * 24ull;
    if (base >= count) break;
#pragma unroll 1
    for (int g = 0; g < kLux / 24; ++g) swb_24(y, c);
    swb_group<0>(y, c);
    swb_group<1>(y, c);
    // oldest word now in slot 2: rotate so that slot 0 is the oldest again
    uint32_t t0 = y[0], t1 = y[1];
#pragma unroll
    for (int k = 0; k < 22; ++k) y[k] = y[k + 2];
    y[22] = t0;
    y[23] = t1;
    if (base + 24 <= count) {
      // a block of 24 numbers starts 96 bytes into its stream (raw_off and base are
      // multiples of 24), so it is six aligned 16-byte stores
      uint4 *v = reinterpret_cast<uint4 *>(dst + base);
#pragma unroll
      for (int k = 0; k < 6; ++k) v[k] = make_uint4(y[4 * k], y[4 * k + 1], y[4 * k + 2], y[4 * k + 3]);
    } else {
#pragma unroll
      for (int k = 0; k < 24; ++k)
        if (base + k < count) dst[base + k] = y[k];
    }
  }
}

// ---- ziggurat ---------------------------------------------------------------
//
// A gaussian starting at stream position p consumes 2 numbers when the first
// attempt is accepted on the integer test j < ktab[i] (97.2% of attempts);
// otherwise 3 (layer < 127) or 4 (base strip) numbers plus, if rejected,
// further attempts.  Consumption is found with integer work alone on the fast
// path; doubles are only used on the slow path and for the final values.

// j * w rounded to the nearest double (ties to even), for 0 < j < 2^24 and w a positive
// normal double whose product stays normal: the ziggurat's x = j W[i].  Exactly the
// value of __dmul_rn((double)j, w), formed on the integer pipe: the 77-bit product of
// j and w's 53-bit significand, rounded to 53 bits, with the exponent adjusted.
__device__ __forceinline__ double mul_u24_rn(uint32_t j, double w) {
  const unsigned long long wb = (unsigned long long)__double_as_longlong(w);
  const int ew = (int)((wb >> 52) & 0x7FF);
  const unsigned long long mw = (wb & ((1ull << 52) - 1)) | (1ull << 52);
  const unsigned long long lo = (unsigned long long)j * mw, hi = __umul64hi((unsigned long long)j, mw);
  const int nbits = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)lo);
  const int sh = nbits - 53;  // 0..24
  unsigned long long m, rem = 0, half = 0;
  if (sh == 0) {
    m = lo;
  } else {
    m = (lo >> sh) | (hi << (64 - sh));
    rem = lo & ((1ull << sh) - 1);
    half = 1ull << (sh - 1);
  }
  int e = sh + ew;
  if (rem > half || (rem == half && half && (m & 1))) {
    ++m;
    if (m == (1ull << 53)) {
      m >>= 1;
      ++e;
    }
  }
  return __longlong_as_double((long long)(((unsigned long long)e << 52) | (m & ((1ull << 52) - 1))));
}

// Stream numbers by absolute position: the walks of neighbouring threads read
// disjoint segments, and the eight entry walks of one segment read the same lines
// again, so they come through L1.
struct Reader {
  const uint32_t *g;
  __device__ __forceinline__ uint32_t operator()(unsigned long long p) const { return __ldg(g + p); }
};

// Advance p past one gaussian of the stream ending at `end`; optionally return
// its value.  Returns false when the stream runs out.
//
// The accept/reject test of a slow-path attempt is first made in single
// precision with a relative margin of 1e-4: the float evaluation of y and
// exp(-x^2/2) is within a few 1e-6 of the double one (x <= 8.3, tables rounded
// once), so a decision outside the margin is the double-precision decision.
// Only attempts inside the margin are evaluated in double.  Values are always
// computed in double.
// Accepted base-strip tail samples need x = R - log(1 - kk/2^24) / R in double, a
// correctly rounded double-double log and a division: about a thousand FP64
// instructions, run by one lane of a warp at a time, and on GB300 each of them holds the
// narrow FP64 pipe for the whole warp.  With `defer` set the value is left to
// k_tail_values (a dense pass over the queued samples): the sample's kk and sign go to
// tail_kk / tail_neg (tail_kk > 0) and g is not set.
template <bool VALUE>
__device__ __forceinline__ bool zig_gaussian(const ZigTab &T, const Reader &rd, unsigned long long end,
                                             unsigned long long &p, double &g, bool defer = false,
                                             uint32_t *tail_kk = nullptr, unsigned long long *tail_neg = nullptr) {
  const double R = GIC_ZIG_PARAM_R;
  const float Rf = (float)GIC_ZIG_PARAM_R;
  for (int guard = 0; guard < 1 << 20; ++guard) {
    if (p + 2 > end) return false;
    uint32_t k1 = rd(p), k2 = rd(p + 1);
    unsigned i = k1 & 0xFFu;
    uint32_t j = k2 & 0xFFFFFFu;
    unsigned il = i & 0x7Fu;
    unsigned long long neg = (i & 0x80u) ? 0ull : 0x8000000000000000ull;
    if (j < T.K[il]) {
      if (VALUE) g = j ? __longlong_as_double(__double_as_longlong(mul_u24_rn(j, T.W[il])) ^ neg)
                       : __longlong_as_double((long long)neg);
      p += 2;
      return true;
    }
    int accept;
    float xf = (float)j * T.Wf[il];
    if (il < 127) {
      if (p + 3 > end) return false;
      uint32_t r2 = rd(p + 2);
      float yf = T.Yf[il + 1] + (T.Yf[il] - T.Yf[il + 1]) * ((float)r2 * (1.0f / 16777216.0f));
      float ef = expf(-0.5f * xf * xf);
      accept = yf < ef * (1.0f - 1e-4f) ? 1 : (yf > ef * (1.0f + 1e-4f) ? 0 : -1);
      if (accept < 0) {
        double x = __dmul_rn((double)j, T.W[il]);
        double u1 = __dmul_rn((double)r2, 1.0 / 16777216.0);
        double y = __dadd_rn(T.Y[il + 1], __dmul_rn(__dsub_rn(T.Y[il], T.Y[il + 1]), u1));
        accept = y < exp(__dmul_rn(__dmul_rn(-0.5, x), x)) ? 1 : 0;
      }
      p += 3;
      if (accept) {
        if (VALUE) g = j ? __longlong_as_double(__double_as_longlong(mul_u24_rn(j, T.W[il])) ^ neg)
                         : __longlong_as_double((long long)neg);
        return true;
      }
    } else {
      if (p + 4 > end) return false;
      uint32_t kk = rd(p + 2), r3 = rd(p + 3);
      float u1f = (float)(16777216u - kk) * (1.0f / 16777216.0f);
      float u2f = (float)r3 * (1.0f / 16777216.0f);
      float xt = Rf - logf(u1f) / Rf;
      float yf = expf(-Rf * (xt - 0.5f * Rf)) * u2f;
      float ef = expf(-0.5f * xt * xt);
      accept = yf < ef * (1.0f - 1e-4f) ? 1 : (yf > ef * (1.0f + 1e-4f) ? 0 : -1);
      double x = 0;
      if (VALUE && accept > 0 && defer) {
        p += 4;
        *tail_kk = 16777216u - kk;
        *tail_neg = neg;
        return true;
      }
      if (accept < 0 || (VALUE && accept > 0)) {
        double lg = gic_log_k24(16777216u - kk);  // log(1 - kk/2^24), correctly rounded
        x = __dsub_rn(R, __ddiv_rn(lg, R));
      }
      if (accept < 0) {
        double u2 = __dmul_rn((double)r3, 1.0 / 16777216.0);
        double y = __dmul_rn(exp(__dmul_rn(-R, __dsub_rn(x, __dmul_rn(0.5, R)))), u2);
        accept = y < exp(__dmul_rn(__dmul_rn(-0.5, x), x)) ? 1 : 0;
      }
      p += 4;
      if (accept) {
        if (VALUE) g = __longlong_as_double(__double_as_longlong(x) ^ neg);
        return true;
      }
    }
  }
  return false;
}

// Walk [seg_start, seg_end) from seg_start + entry, counting gaussians that
// start in the segment; exit = position after the last one minus seg_end.
// tail samples whose values k_tail_values computes: where the value goes, its argument
// 2^24 - kk and its sign bit
struct TailSample {
  double *at;
  uint32_t arg;
  uint32_t neg;  // 1: negative
};
struct TailQueue {
  TailSample *items = nullptr;  // null: values computed in place
  unsigned *count = nullptr;
  unsigned cap = 0;
};

template <bool VALUE>
__device__ void walk_segment(const ZigTab &T, const Reader &rd, unsigned long long stream_end, unsigned long long seg_start,
                             unsigned long long seg_end, unsigned entry, uint32_t &count, uint32_t &exit_off,
                             double *out, unsigned long long out_limit, TailQueue q = TailQueue{}) {
  unsigned long long p = seg_start + entry;
  uint32_t cnt = 0;
  while (p < seg_end) {
    if (VALUE && cnt >= out_limit) break;
    double g = 0;
    uint32_t tail_kk = 0;
    unsigned long long tail_neg = 0;
    const unsigned long long p_before = p;
    if (!zig_gaussian<VALUE>(T, rd, stream_end, p, g, VALUE && q.items != nullptr, &tail_kk, &tail_neg)) {
      count = cnt;
      exit_off = kUnderrun;
      return;
    }
    if (VALUE) {
      if (tail_kk) {
        const unsigned slot = atomicAdd(q.count, 1u);
        if (slot < q.cap) {
          q.items[slot] = TailSample{out + cnt, tail_kk, tail_neg ? 1u : 0u};
        } else {
          // queue full: this sample's value in place
          unsigned long long p2 = p_before;
          zig_gaussian<VALUE>(T, rd, stream_end, p2, g);
          out[cnt] = g;
        }
      } else {
        out[cnt] = g;
      }
    }
    ++cnt;
  }
  count = cnt;
  exit_off = p >= seg_end ? (uint32_t)(p - seg_end) : 0u;
}

// packed (count, exit): count in the low 16 bits, exit in the high 16, 0xFFFF = underrun/overflow
__device__ __forceinline__ uint32_t pack_ce(uint32_t cnt, uint32_t ex) {
  return (cnt & 0xFFFFu) | ((ex == kUnderrun || ex >= 0xFFFFu ? 0xFFFFu : ex) << 16);
}

__device__ __forceinline__ void segment_bounds(const Stream &s, unsigned long long lseg, unsigned long long &a,
                                               unsigned long long &b) {
  a = s.raw_off + lseg * kSegLen;
  b = a + kSegLen;
  unsigned long long e = s.raw_off + s.raw_count;
  if (b > e) b = e;
}

// One thread per segment tabulates (count, exit) for the entry offsets 0..kSpec-1.
// The walk from entry 0 marks the start of each of its gaussians in a bitmap of
// the segment (a column of shared memory per thread, conflict-free).  The walk
// from entry e > 0 then runs only until it stands on a marked position: from
// there on both are the same walk, so its count is the gaussians it found before
// plus entry 0's from that position on, and its exit (or underrun) is entry 0's.
// Fast-path gaussians take 2 numbers, so even entries meet entry 0 at once and odd
// ones after the first 3-number attempt of either walk: the kSpec tables cost
// about 1.3 walks of the segment instead of kSpec.
__global__ void __launch_bounds__(kSpecThreads) k_walk_speculative(const Stream *st, int nstreams,
                                                                    unsigned long long nseg_total,
                                                                    const uint32_t *raw, uint32_t *tab) {
  __shared__ ZigTab zt;
  __shared__ uint32_t marks[kSegLen / 32][kSpecThreads];
  load_zig(zt);
  const int t = threadIdx.x;
  for (int w = 0; w < kSegLen / 32; ++w) marks[w][t] = 0u;
  __syncthreads();
  unsigned long long gseg = (unsigned long long)blockIdx.x * kSpecThreads + t;
  if (gseg >= nseg_total) return;
  int s = find_stream_by_segment(st, nstreams, gseg);
  const Stream &S = st[s];
  unsigned long long a, b;
  segment_bounds(S, gseg - S.seg_off, a, b);
  const unsigned long long end = S.raw_off + S.raw_count;
  const Reader rd{raw};
  double g;
  unsigned long long p = a;
  uint32_t total0 = 0, ex0;
  bool under = false;
  while (p < b) {
    uint32_t r = (uint32_t)(p - a);
    marks[r >> 5][t] |= 1u << (r & 31);
    if (!zig_gaussian<false>(zt, rd, end, p, g)) {
      under = true;
      break;
    }
    ++total0;
  }
  ex0 = under ? kUnderrun : (uint32_t)(p - b);
  uint32_t *out = tab + gseg * kSpec;
  out[0] = pack_ce(total0, ex0);
  for (unsigned e = 1; e < (unsigned)kSpec; ++e) {
    unsigned long long q = a + e;
    uint32_t cnt = 0, ex = 0;
    bool met = false;
    while (q < b) {
      uint32_t r = (uint32_t)(q - a);
      uint32_t word = marks[r >> 5][t];
      if ((word >> (r & 31)) & 1u) {
        uint32_t before = __popc(word & ((1u << (r & 31)) - 1u));  // entry 0's gaussians before r
        for (uint32_t w = 0; w < (r >> 5); ++w) before += __popc(marks[w][t]);
        cnt += total0 - before;
        ex = ex0;
        met = true;
        break;
      }
      if (!zig_gaussian<false>(zt, rd, end, q, g)) {
        ex = kUnderrun;
        met = true;
        break;
      }
      ++cnt;
    }
    if (!met) ex = (uint32_t)(q - b);
    out[e] = pack_ce(cnt, ex);
  }
}

// Follow segment g from entry e: table lookup, or a real walk when the entry
// is beyond the speculated offsets.
__device__ __forceinline__ void step_segment(const Stream &s, const uint32_t *raw, const uint32_t *tab,
                                             unsigned long long gseg, unsigned e, uint32_t &cnt, uint32_t &ex) {
  if (e < (unsigned)kSpec) {
    uint32_t v = tab[gseg * kSpec + e];
    cnt = v & 0xFFFFu;
    ex = v >> 16;
    if (ex != 0xFFFFu) return;
  }
  unsigned long long a, b;
  segment_bounds(s, gseg - s.seg_off, a, b);
  const Reader rd{raw};
  walk_segment<false>(gZig, rd, s.raw_off + s.raw_count, a, b, e, cnt, ex, nullptr, 0);
}

// Level 1: map of each block of kBlockSegs segments for every entry offset.
__global__ void k_block_maps(const Stream *st, int nstreams, unsigned long long nblk_total, const uint32_t *raw,
                             const uint32_t *tab, uint2 *bmap) {
  unsigned long long id = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nblk_total * kSpec) return;
  unsigned long long blk = id / kSpec;
  unsigned e = (unsigned)(id % kSpec);
  int s = find_stream_by_block(st, nstreams, blk);
  const Stream &S = st[s];
  unsigned long long lblk = blk - S.blk_off;
  unsigned long long g = S.seg_off + lblk * kBlockSegs;
  unsigned long long gend = min(S.seg_off + (unsigned long long)S.nseg, g + kBlockSegs);
  uint32_t total = 0;
  for (; g < gend; ++g) {
    uint32_t cnt, ex;
    step_segment(S, raw, tab, g, e, cnt, ex);
    total += cnt;
    if (ex == kUnderrun || ex == 0xFFFFu) { e = 0xFFFFu; break; }
    e = ex;
  }
  bmap[id] = make_uint2(total, e);
}

// Level 2: one thread per stream chains its blocks.  flags[0] set on underrun.
__global__ void k_chain_blocks(const Stream *st, int nstreams, const uint32_t *raw, const uint32_t *tab,
                               const uint2 *bmap, uint32_t *blk_entry, unsigned long long *blk_base, int *flags) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nstreams) return;
  const Stream &S = st[s];
  unsigned long long need = S.gauss_count, base = 0;
  unsigned e = 0;
  for (unsigned b = 0; b < S.nblk; ++b) {
    unsigned long long blk = S.blk_off + b;
    blk_entry[blk] = e;
    blk_base[blk] = base;
    if (base >= need) continue;
    uint32_t total, ex;
    if (e < (unsigned)kSpec) {
      uint2 v = bmap[blk * kSpec + e];
      total = v.x;
      ex = v.y;
    } else {
      // entry beyond the speculated offsets: chain the block's segments here
      total = 0;
      ex = e;
      unsigned long long g = S.seg_off + (unsigned long long)b * kBlockSegs;
      unsigned long long gend = min(S.seg_off + (unsigned long long)S.nseg, g + kBlockSegs);
      for (; g < gend; ++g) {
        uint32_t cnt, x2;
        step_segment(S, raw, tab, g, ex, cnt, x2);
        total += cnt;
        if (x2 == kUnderrun || x2 == 0xFFFFu) { ex = 0xFFFFu; break; }
        ex = x2;
      }
    }
    base += total;
    if (ex == 0xFFFFu) {
      if (base < need) atomicExch(flags, 1);
      e = 0;
      continue;
    }
    e = ex;
  }
  if (base < need) atomicExch(flags, 1);
}

// Level 3: one thread per block writes each segment's entry and gaussian base.
__global__ void k_chain_segments(const Stream *st, int nstreams, unsigned long long nblk_total, const uint32_t *raw,
                                 const uint32_t *tab, const uint32_t *blk_entry, const unsigned long long *blk_base,
                                 uint32_t *seg_entry, unsigned long long *seg_base) {
  unsigned long long blk = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (blk >= nblk_total) return;
  int s = find_stream_by_block(st, nstreams, blk);
  const Stream &S = st[s];
  unsigned long long g = S.seg_off + (blk - S.blk_off) * kBlockSegs;
  unsigned long long gend = min(S.seg_off + (unsigned long long)S.nseg, g + kBlockSegs);
  unsigned e = blk_entry[blk];
  unsigned long long base = blk_base[blk];
  for (; g < gend; ++g) {
    seg_entry[g] = e;
    seg_base[g] = base;
    if (base >= S.gauss_count) { e = 0; continue; }
    uint32_t cnt, ex;
    step_segment(S, raw, tab, g, e, cnt, ex);
    base += cnt;
    e = (ex == kUnderrun || ex == 0xFFFFu) ? 0 : ex;
  }
}

__global__ void k_walk_final(const Stream *st, int nstreams, unsigned long long nseg_total, const uint32_t *raw,
                             const uint32_t *seg_entry, const unsigned long long *seg_base, double *gauss,
                             int *flags, TailQueue q) {
  __shared__ ZigTab zt;
  load_zig(zt);
  __syncthreads();
  unsigned long long gseg = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gseg >= nseg_total) return;
  int s = find_stream_by_segment(st, nstreams, gseg);
  const Stream &S = st[s];
  unsigned long long base = seg_base[gseg];
  unsigned long long need = S.gauss_count;
  if (base >= need) return;
  unsigned long long a, b;
  segment_bounds(S, gseg - S.seg_off, a, b);
  const Reader rd{raw};
  uint32_t cnt, ex;
  walk_segment<true>(zt, rd, S.raw_off + S.raw_count, a, b, seg_entry[gseg], cnt, ex, gauss + S.gauss_off + base,
                     need - base, q);
  if (ex == kUnderrun && base + cnt < need) atomicExch(flags, 1);
}

// The deferred tail values: x = R - log(1 - kk/2^24) / R, correctly rounded log, one
// sample per thread
__global__ void k_tail_values(TailQueue q) {
  const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned n = min(*q.count, q.cap);
  if (i >= n) return;
  const TailSample t = q.items[i];
  const double R = GIC_ZIG_PARAM_R;
  const double lg = gic_log_k24(t.arg);
  const double x = __dsub_rn(R, __ddiv_rn(lg, R));
  *t.at = __longlong_as_double(__double_as_longlong(x) ^ (t.neg ? 0x8000000000000000ull : 0ull));
}

// ---- placement ----------------------------------------------------------------

// modes drawn before shell ks: sum_{j<ks} 3 (2j)^2
__host__ __device__ __forceinline__ unsigned long long shell_offset(long long ks) {
  return ks <= 1 ? 0ull : (unsigned long long)(2 * (ks - 1) * ks * (2 * ks - 1));
}

// Draw index Q -> mode.  shell_offset(ks) ~ 4 ks^3, so ks starts from the cube root of
// Q / 4 and is corrected exactly by at most a step or two; the rest fits 32 bits
// (Q < 2^31: draw_noise_all checks the grid size).
__device__ __forceinline__ void decode_mode(unsigned long long Q, int half, int &k1, int &k2, int &k3) {
  int ks = (int)cbrtf((float)Q * 0.25f);
  ks = max(1, min(ks, half - 1));
  while (ks < half - 1 && shell_offset(ks + 1) <= Q) ++ks;
  while (ks > 1 && shell_offset(ks) > Q) --ks;
  const unsigned q = (unsigned)(Q - shell_offset(ks));
  const unsigned t = q / 3u;
  const int which = (int)(q - 3u * t);
  const unsigned side = 2u * (unsigned)ks;
  const unsigned ta = t / side;
  const int a = (int)ta - ks;
  const int b = (int)(t - ta * side) - ks;
  if (which == 0) { k1 = ks; k2 = a; k3 = b; }
  else if (which == 1) { k1 = a; k2 = ks; k3 = b; }
  else { k1 = a; k2 = b; k3 = ks; }
}

// storage index of mode (kx,ky,kz) of a real field's half spectrum; conj = folded
__device__ __forceinline__ size_t coeff_index(int n, int kx, int ky, int kz, bool &conj) {
  conj = false;
  if (kz < 0) { kx = -kx; ky = -ky; kz = -kz; conj = true; }
  if (ky < 0) ky += n;
  if (kx < 0) kx += n;
  return (size_t)kz + (size_t)(n / 2 + 1) * ((size_t)ky + (size_t)n * (size_t)kx);
}

__device__ __forceinline__ bool needs_partner(int n, int k1, int k2, int k3) {
  int nyq = n / 2;
  return k1 == 0 || k1 == nyq || k2 == 0 || k2 == nyq || k3 == 0 || k3 == nyq;
}

__global__ void k_place_owner(int n, unsigned long long nmodes, int *owner) {
  unsigned long long Q = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (Q >= nmodes) return;
  int k1, k2, k3;
  decode_mode(Q, n / 2, k1, k2, k3);
  bool cj;
  atomicMax(owner + coeff_index(n, k1, k2, k3, cj), (int)Q);
  if (needs_partner(n, k1, k2, k3)) atomicMax(owner + coeff_index(n, -k1, -k2, -k3, cj), (int)Q);
}

template <typename T>
__global__ void k_place_write(int n, unsigned long long nmodes, const int *owner, const double *gauss, T norm,
                              int reverse, T *out /* interleaved complex */) {
  unsigned long long Q = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (Q >= nmodes) return;
  int k1, k2, k3;
  decode_mode(Q, n / 2, k1, k2, k3);
  // FloatType a = norm * gaussian  (double gaussian, promoted product, rounded to T)
  T a = (T)((double)norm * gauss[2 * Q]);
  T b = (T)((double)norm * gauss[2 * Q + 1]);
  T re = reverse ? b : a, im = reverse ? a : b;
  bool cj;
  size_t c1 = coeff_index(n, k1, k2, k3, cj);
  if (owner[c1] == (int)Q) {
    out[2 * c1] = re;
    out[2 * c1 + 1] = cj ? -im : im;
  }
  if (needs_partner(n, k1, k2, k3)) {
    size_t c2 = coeff_index(n, -k1, -k2, -k3, cj);
    if (owner[c2] == (int)Q) {
      out[2 * c2] = re;
      out[2 * c2 + 1] = cj ? im : -im;
    }
  }
}

template <typename T>
__global__ void k_place_real(int n, const double *gauss, T *out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t m = (size_t)n * n * n;
  if (i >= m) return;
  size_t row = i / n, z = i % n;
  out[row * (size_t)(2 * (n / 2 + 1)) + z] = (T)gauss[i];
}

template <typename T>
__global__ void k_zero_first(T *out) {
  out[0] = (T)0;
}

unsigned long long raw_needed(unsigned long long g) {
  // mean 2.0534 numbers per gaussian, generous margin
  double m = 2.0534 * (double)g + 12.0 * std::sqrt((double)g + 1.0) + 512.0;
  return (unsigned long long)m;
}

}  // namespace

struct StreamTotals {
  unsigned long long raw = 0, seg = 0, chunk = 0, max_chunks = 0, blk = 0;
};

// raw-number, segment, chunk and block ranges of every stream (a function of the
// gaussian counts and the margin only, not of the seeds)
static StreamTotals layout_streams(std::vector<Stream> &streams, double margin) {
  StreamTotals t;
  unsigned long long &raw_total = t.raw, &seg_total = t.seg, &chunk_total = t.chunk, &max_chunks = t.max_chunks,
                     &blk_total = t.blk;
  for (auto &s : streams) {
    s.raw_off = raw_total;
    s.raw_count = (unsigned long long)(raw_needed(s.gauss_count) * margin);
    s.raw_count = (s.raw_count + 23) / 24 * 24;
    raw_total += s.raw_count;
    s.nseg = (unsigned int)((s.raw_count + kSegLen - 1) / kSegLen);
    s.seg_off = seg_total;
    seg_total += s.nseg;
    s.nblk = (s.nseg + kBlockSegs - 1) / kBlockSegs;
    s.blk_off = blk_total;
    blk_total += s.nblk;
    unsigned long long blocks = s.raw_count / 24;
    s.nchunk = (unsigned int)((blocks + kChunkBlocks - 1) / kChunkBlocks);
    s.chunk_off = chunk_total;
    chunk_total += s.nchunk;
    max_chunks = std::max<unsigned long long>(max_chunks, s.nchunk);
  }
  return t;
}

// Generate `streams` gaussians into ctx.rng.gauss (layout given by gauss_off).  With
// ctx.defer_checks the descriptors are not uploaded (upload_noise_streams did) and the
// underrun flag is left on the device (noise_underrun reads it).
static void generate_gaussians(Context &ctx, std::vector<Stream> &streams, unsigned long long total_gauss,
                               double margin) {
  cudaStream_t cs = ctx.stream;
  int ns = (int)streams.size();
  const StreamTotals tot = layout_streams(streams, margin);
  const unsigned long long raw_total = tot.raw, seg_total = tot.seg, chunk_total = tot.chunk,
                           max_chunks = tot.max_chunks, blk_total = tot.blk;
  RngScratch &R = ctx.rng;
  R.raw.ensure(raw_total * sizeof(uint32_t));
  R.gauss.ensure(total_gauss * sizeof(double));
  R.segtab.ensure(seg_total * kSpec * sizeof(uint32_t));
  R.segentry.ensure(seg_total * sizeof(uint32_t));
  R.segbase.ensure(seg_total * sizeof(unsigned long long));
  R.blkmap.ensure(blk_total * kSpec * sizeof(uint2));
  R.blkentry.ensure(blk_total * sizeof(uint32_t));
  R.blkbase.ensure(blk_total * sizeof(unsigned long long));
  R.streams.ensure(streams.size() * sizeof(Stream));
  R.flags.ensure(sizeof(int) * 4);

  // chunk multipliers (seed independent; computed once for the largest stream)
  if ((unsigned long long)R.chunkmul_count < max_chunks) {
    int count = (int)std::max<unsigned long long>(max_chunks, 1024);
    std::vector<U576> pow2;
    U576 a, step;
    u576_ranlux_multiplier(a);
    u576_powmod(step, a, (uint64_t)kLux * kChunkBlocks);
    int npow = 0;
    while ((1 << npow) < count) ++npow;
    pow2.resize(std::max(npow, 1));
    pow2[0] = step;
    for (int i = 1; i < npow; ++i) u576_mulmod(pow2[i], pow2[i - 1], pow2[i - 1]);
    DevBuf dpow;
    dpow.ensure(pow2.size() * sizeof(U576));
    GIC_CUDA(cudaMemcpyAsync(dpow.ptr, pow2.data(), pow2.size() * sizeof(U576), cudaMemcpyHostToDevice, cs));
    R.chunkmul.ensure((size_t)count * sizeof(U576));
    k_chunk_multipliers<<<(count + 127) / 128, 128, 0, cs>>>(R.chunkmul.as<U576>(), count, dpow.as<U576>(), npow);
    launched();
    GIC_CUDA(cudaStreamSynchronize(cs));
    R.chunkmul_count = count;
  }

  Stream *dst = R.streams.as<Stream>();
  if (!ctx.defer_checks)
    GIC_CUDA(cudaMemcpyAsync(dst, streams.data(), streams.size() * sizeof(Stream), cudaMemcpyHostToDevice, cs));
  GIC_CUDA(cudaMemsetAsync(R.flags.ptr, 0, sizeof(int) * 4, cs));
  k_seed<<<(ns + 127) / 128, 128, 0, cs>>>(dst, ns);
  launched();
  k_generate<<<(unsigned)((chunk_total + 127) / 128), 128, 0, cs>>>(dst, ns, chunk_total, R.chunkmul.as<U576>(),
                                                                   R.raw.as<uint32_t>());
  launched();
  k_walk_speculative<<<(unsigned)((seg_total + kSpecThreads - 1) / kSpecThreads), kSpecThreads, 0, cs>>>(
      dst, ns, seg_total, R.raw.as<uint32_t>(), R.segtab.as<uint32_t>());
  launched();
  unsigned long long nbm = blk_total * kSpec;
  k_block_maps<<<(unsigned)((nbm + 127) / 128), 128, 0, cs>>>(dst, ns, blk_total, R.raw.as<uint32_t>(),
                                                             R.segtab.as<uint32_t>(), R.blkmap.as<uint2>());
  launched();
  k_chain_blocks<<<(ns + 63) / 64, 64, 0, cs>>>(dst, ns, R.raw.as<uint32_t>(), R.segtab.as<uint32_t>(),
                                               R.blkmap.as<uint2>(), R.blkentry.as<uint32_t>(),
                                               R.blkbase.as<unsigned long long>(), R.flags.as<int>());
  launched();
  k_chain_segments<<<(unsigned)((blk_total + 127) / 128), 128, 0, cs>>>(
      dst, ns, blk_total, R.raw.as<uint32_t>(), R.segtab.as<uint32_t>(), R.blkentry.as<uint32_t>(),
      R.blkbase.as<unsigned long long>(), R.segentry.as<uint32_t>(), R.segbase.as<unsigned long long>());
  launched();
  // tail samples, about 6e-4 of the gaussians: a queue of 1/512 of them (overflow is
  // computed in place), its count in the flags word 3
  const unsigned tail_cap = (unsigned)std::min<unsigned long long>(total_gauss / 512 + 4096, 1ull << 30);
  R.tailq.ensure((size_t)tail_cap * sizeof(TailSample));
  TailQueue q{R.tailq.as<TailSample>(), reinterpret_cast<unsigned *>(R.flags.as<int>() + 3), tail_cap};
  k_walk_final<<<(unsigned)((seg_total + 127) / 128), 128, 0, cs>>>(
      dst, ns, seg_total, R.raw.as<uint32_t>(), R.segentry.as<uint32_t>(), R.segbase.as<unsigned long long>(),
      R.gauss.as<double>(), R.flags.as<int>(), q);
  k_tail_values<<<(tail_cap + 255) / 256, 256, 0, cs>>>(q);
  launched(2);
  if (ctx.defer_checks) return;
  int flag = 0;
  read_small(ctx, R.flags.ptr, sizeof(int), &flag);
  if (flag) {
    if (margin > 4.0) fail(GIC_ERR_INTERNAL, "random stream shorter than the gaussians it must supply");
    generate_gaussians(ctx, streams, total_gauss, margin * 1.5);
  }
}

// Place this level's gaussians (device pointer) on its half spectrum.
template <typename T>
static void place_level(Context &ctx, Level &L, const double *gauss, int mode) {
  cudaStream_t cs = ctx.stream;
  int n = L.n;
  size_t nc = L.ncomplex();
  L.noise.ensure(nc * 2 * sizeof(T));
  T *out = L.noise.as<T>();
  GIC_CUDA(cudaMemsetAsync(out, 0, nc * 2 * sizeof(T), cs));
  if (mode == GIC_SEED_REAL_SPACE) {
    unsigned long long m = L.ncells();
    k_place_real<T><<<(unsigned)((m + 255) / 256), 256, 0, cs>>>(n, gauss, out);
    launched();
    fft_r2c_3d<T>(ctx, out, n, 1.0 / std::pow((double)n, 1.5));
    k_zero_first<T><<<1, 1, 0, cs>>>(out);
    launched();
  } else {
    unsigned long long nmodes = shell_offset(n / 2);
    if (nmodes > 0) {
      ctx.rng.owner.ensure(nc * sizeof(int));
      GIC_CUDA(cudaMemsetAsync(ctx.rng.owner.ptr, 0xFF, nc * sizeof(int), cs));
      unsigned blocks = (unsigned)((nmodes + 255) / 256);
      k_place_owner<<<blocks, 256, 0, cs>>>(n, nmodes, ctx.rng.owner.as<int>());
      launched();
      T norm = (T)(1.0 / std::sqrt(2.0));
      k_place_write<T><<<blocks, 256, 0, cs>>>(n, nmodes, ctx.rng.owner.as<int>(), gauss, norm,
                                               mode == GIC_SEED_FOURIER_REVERSE ? 1 : 0, out);
      launched();
    }
  }
  L.have_noise = true;
}

// genetIC draws level after level (randomfieldgenerator.hpp:122-139): the
// serial and real-space modes keep consuming one stream across levels, the
// parallel mode reseeds every shell with seed + ks on every level, so all
// levels share the shell streams of the largest one.
// The streams genetIC draws the levels' noise from: per shell seed + ks in the parallel
// mode (every level reseeds each shell), one stream of `seed` across the levels otherwise.
// offset: each level's first gaussian; total: the gaussians drawn.
static std::vector<Stream> noise_streams(const Context &ctx, unsigned long long seed, int mode,
                                         std::vector<unsigned long long> &offset, unsigned long long &total) {
  std::vector<Stream> streams;
  offset.assign(ctx.levels.size(), 0);
  total = 0;
  if (mode == GIC_SEED_FOURIER_PARALLEL) {
    int half = 0;
    for (auto &L : ctx.levels) half = std::max(half, L->n / 2);
    for (int ks = 1; ks < half; ++ks) {
      Stream s{};
      s.seed = seed + (unsigned long long)ks;
      s.gauss_off = 2 * shell_offset(ks);
      s.gauss_count = 2 * (shell_offset(ks + 1) - shell_offset(ks));
      streams.push_back(s);
    }
    if (!streams.empty()) total = 2 * shell_offset(half);
  } else {
    for (size_t l = 0; l < ctx.levels.size(); ++l) {
      offset[l] = total;
      const Level &L = *ctx.levels[l];
      total += mode == GIC_SEED_REAL_SPACE ? (unsigned long long)L.ncells() : 2 * shell_offset(L.n / 2);
    }
    Stream s{};
    s.seed = seed;
    s.gauss_off = 0;
    s.gauss_count = total;
    if (total > 0) streams.push_back(s);
  }
  return streams;
}

template <typename T>
static void draw_all_typed(Context &ctx, unsigned long long seed, int mode) {
  std::vector<unsigned long long> offset;
  unsigned long long total = 0;
  std::vector<Stream> streams = noise_streams(ctx, seed, mode, offset, total);
  if (!streams.empty()) generate_gaussians(ctx, streams, total, 1.0);
  for (size_t l = 0; l < ctx.levels.size(); ++l) {
    Level &L = *ctx.levels[l];
    if (mode == GIC_SEED_FOURIER_PARALLEL) {
      // same shell streams: a level of the same size as an earlier one draws the same noise
      size_t same = l;
      for (size_t m = 0; m < l; ++m)
        if (ctx.levels[m]->n == L.n) { same = m; break; }
      if (same != l) {
        size_t bytes = L.ncomplex() * 2 * sizeof(T);
        L.noise.ensure(bytes);
        GIC_CUDA(cudaMemcpyAsync(L.noise.ptr, ctx.levels[same]->noise.ptr, bytes, cudaMemcpyDeviceToDevice,
                                 ctx.stream));
        L.have_noise = true;
        continue;
      }
    }
    place_level<T>(ctx, L, ctx.rng.gauss.as<double>() + offset[l], mode);
  }
  if (!ctx.defer_checks) GIC_CUDA(cudaStreamSynchronize(ctx.stream));
}

void upload_noise_streams(Context &ctx, unsigned long long seed, int mode) {
  std::vector<unsigned long long> offset;
  unsigned long long total = 0;
  std::vector<Stream> streams = noise_streams(ctx, seed, mode, offset, total);
  if (streams.empty()) return;
  layout_streams(streams, 1.0);
  if (ctx.rng.streams.bytes < streams.size() * sizeof(Stream))
    fail(GIC_ERR_INTERNAL, "the noise streams were not laid out by an earlier draw");
  GIC_CUDA(cudaMemcpyAsync(ctx.rng.streams.ptr, streams.data(), streams.size() * sizeof(Stream), cudaMemcpyHostToDevice,
                           ctx.stream));
  GIC_CUDA(cudaStreamSynchronize(ctx.stream));  // the host vector goes out of scope
}

bool noise_underrun(Context &ctx) {
  if (!ctx.rng.flags.ptr) return false;
  int flag = 0;
  read_small(ctx, ctx.rng.flags.ptr, sizeof(int), &flag);
  return flag != 0;
}

void gaussian_stream(Context &ctx, unsigned long long seed, size_t n, double *host) {
  std::vector<Stream> streams(1);
  streams[0] = Stream{};
  streams[0].seed = seed;
  streams[0].gauss_count = n;
  generate_gaussians(ctx, streams, n, 1.0);
  GIC_CUDA(cudaMemcpyAsync(host, ctx.rng.gauss.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, ctx.stream));
  GIC_CUDA(cudaStreamSynchronize(ctx.stream));
}

void draw_noise_all(Context &ctx, unsigned long long seed, int mode) {
  if (mode < 0 || mode > 3) fail(GIC_ERR_INVALID_ARG, "unknown seeding mode");
  for (auto &L : ctx.levels)
    if ((long long)L->n * L->n * (L->n / 2 + 1) >= (1ll << 31))
      fail(GIC_ERR_INVALID_ARG, "grid too large for 32-bit mode indices");
  if (ctx.dbl())
    draw_all_typed<double>(ctx, seed, mode);
  else
    draw_all_typed<float>(ctx, seed, mode);
}


// ---- allocation-free gaussian stream ------------------------------------------------
//
// For callers that cannot allocate device memory themselves -- code running
// inside another runtime's memory pool or budget, where a cudaMalloc of its
// own is not permitted -- this variant of the gaussian-stream pipeline keeps
// all its scratch (the raw RANLUX numbers, the chunk jump multipliers, the
// segment walk tables, the stream descriptor and the underrun flag) in one
// file-scope device array.  The array is NoallocScratchBytes bytes on every
// device that loads the library, for the lifetime of the process, and every
// call shares it: calls that overlap on the GPU (different streams or host
// threads) race on it and must be serialised by the caller.  Every region a
// call reads is written by that same call first (the flag is cleared), so no
// state carries over from an earlier call.  A call reads the underrun flag
// back and synchronises the caller's stream before it returns.

constexpr unsigned long long kNoallocMaxGauss = GIC_NOALLOC_MAX_GAUSSIANS;
constexpr size_t NoallocScratchBytes = 24ull << 20;
static __device__ __align__(256) unsigned char gNoallocScratch[NoallocScratchBytes];

namespace {

__global__ void k_set_stream(Stream *dst, Stream s) { *dst = s; }

// pow2[i] = a^(794 kChunkBlocks 2^i) mod m, one thread
__global__ void k_pow2_multipliers(U576 *pow2, int npow) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  U576 a;
  u576_ranlux_multiplier(a);
  u576_powmod(pow2[0], a, (uint64_t)kLux * kChunkBlocks);
  for (int i = 1; i < npow; ++i) u576_mulmod(pow2[i], pow2[i - 1], pow2[i - 1]);
}

struct NoallocLayout {
  size_t raw, pow2, chunkmul, segtab, segentry, segbase, blkmap, blkentry, blkbase, stream, flags, end;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// byte offsets of every scratch region for a stream of raw_count numbers
NoallocLayout noalloc_layout(unsigned long long raw_count, unsigned long long nchunk, unsigned long long nseg,
                             unsigned long long nblk, int npow) {
  NoallocLayout L;
  size_t o = 0;
  L.raw = o;
  o = align256(o + raw_count * sizeof(uint32_t));
  L.pow2 = o;
  o = align256(o + (size_t)npow * sizeof(U576));
  L.chunkmul = o;
  o = align256(o + nchunk * sizeof(U576));
  L.segtab = o;
  o = align256(o + nseg * kSpec * sizeof(uint32_t));
  L.segentry = o;
  o = align256(o + nseg * sizeof(uint32_t));
  L.segbase = o;
  o = align256(o + nseg * sizeof(unsigned long long));
  L.blkmap = o;
  o = align256(o + nblk * kSpec * sizeof(uint2));
  L.blkentry = o;
  o = align256(o + nblk * sizeof(uint32_t));
  L.blkbase = o;
  o = align256(o + nblk * sizeof(unsigned long long));
  L.stream = o;
  o = align256(o + sizeof(Stream));
  L.flags = o;
  o = align256(o + 4 * sizeof(int));
  L.end = o;
  return L;
}

// Device address of the scratch array, looked up once per device and CUDA
// context: a context made after cudaDeviceReset loads the module again, so the
// address is looked up again when the current context's id changes.
std::mutex g_noalloc_mutex;
struct NoallocSlot {
  unsigned long long ctx_id;
  void *base;
};
NoallocSlot g_noalloc_slot[64];

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

// id of the current CUDA context (0 when it cannot be read); the driver calls
// are reached through the runtime, so the library does not link libcuda
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
    cudaGetLastError();
    looked_up = true;
  }
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&c) == CUDA_SUCCESS && c && get_id(c, &id) == CUDA_SUCCESS) return id;
  return 0;
}

}  // namespace

static int noalloc_scratch(void **base) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return GIC_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  const unsigned long long id = current_context_id();
  NoallocSlot &slot = g_noalloc_slot[dev];
  if (!slot.base || id == 0 || slot.ctx_id != id) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, gNoallocScratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return GIC_ERR_CUDA;
    }
    slot.base = p;
    slot.ctx_id = current_context_id();  // the lookup makes the device's context current
  }
  *base = slot.base;
  return GIC_OK;
}

static int noalloc_run(unsigned long long seed, unsigned long long n, double *out, cudaStream_t cs, double margin,
                       bool *underrun) {
  void *base = nullptr;
  int st = noalloc_scratch(&base);
  if (st != GIC_OK) return st;
  // an error left by the caller's own earlier launches is not this call's
  cudaGetLastError();
  Stream s{};
  s.seed = seed;
  s.raw_off = 0;
  s.raw_count = ((unsigned long long)(raw_needed(n) * margin) + 23) / 24 * 24;
  s.gauss_off = 0;
  s.gauss_count = n;
  s.nseg = (unsigned int)((s.raw_count + kSegLen - 1) / kSegLen);
  s.seg_off = 0;
  s.nblk = (s.nseg + kBlockSegs - 1) / kBlockSegs;
  s.blk_off = 0;
  s.nchunk = (unsigned int)((s.raw_count / 24 + kChunkBlocks - 1) / kChunkBlocks);
  s.chunk_off = 0;
  int npow = 1;
  while ((1ull << npow) < s.nchunk) ++npow;
  NoallocLayout L = noalloc_layout(s.raw_count, s.nchunk, s.nseg, s.nblk, npow);
  if (L.end > NoallocScratchBytes) return GIC_ERR_NOT_READY;
  unsigned char *b = static_cast<unsigned char *>(base);
  uint32_t *raw = reinterpret_cast<uint32_t *>(b + L.raw);
  U576 *pow2 = reinterpret_cast<U576 *>(b + L.pow2);
  U576 *chunkmul = reinterpret_cast<U576 *>(b + L.chunkmul);
  uint32_t *segtab = reinterpret_cast<uint32_t *>(b + L.segtab);
  uint32_t *segentry = reinterpret_cast<uint32_t *>(b + L.segentry);
  unsigned long long *segbase = reinterpret_cast<unsigned long long *>(b + L.segbase);
  uint2 *blkmap = reinterpret_cast<uint2 *>(b + L.blkmap);
  uint32_t *blkentry = reinterpret_cast<uint32_t *>(b + L.blkentry);
  unsigned long long *blkbase = reinterpret_cast<unsigned long long *>(b + L.blkbase);
  Stream *dst = reinterpret_cast<Stream *>(b + L.stream);
  int *flags = reinterpret_cast<int *>(b + L.flags);
  cudaError_t e = cudaSuccess;
  auto ok = [&]() { e = cudaGetLastError(); return e == cudaSuccess; };
  if (cudaMemsetAsync(flags, 0, 4 * sizeof(int), cs) != cudaSuccess) return GIC_ERR_CUDA;
  k_set_stream<<<1, 1, 0, cs>>>(dst, s);
  k_pow2_multipliers<<<1, 1, 0, cs>>>(pow2, npow);
  k_chunk_multipliers<<<(s.nchunk + 127) / 128, 128, 0, cs>>>(chunkmul, (int)s.nchunk, pow2, npow);
  k_seed<<<1, 1, 0, cs>>>(dst, 1);
  k_generate<<<(s.nchunk + 127) / 128, 128, 0, cs>>>(dst, 1, s.nchunk, chunkmul, raw);
  if (!ok()) return GIC_ERR_CUDA;
  k_walk_speculative<<<(s.nseg + kSpecThreads - 1) / kSpecThreads, kSpecThreads, 0, cs>>>(dst, 1, s.nseg, raw, segtab);
  k_block_maps<<<(s.nblk * kSpec + 127) / 128, 128, 0, cs>>>(dst, 1, s.nblk, raw, segtab, blkmap);
  k_chain_blocks<<<1, 64, 0, cs>>>(dst, 1, raw, segtab, blkmap, blkentry, blkbase, flags);
  k_chain_segments<<<(s.nblk + 127) / 128, 128, 0, cs>>>(dst, 1, s.nblk, raw, segtab, blkentry, blkbase, segentry,
                                                         segbase);
  k_walk_final<<<(s.nseg + 127) / 128, 128, 0, cs>>>(dst, 1, s.nseg, raw, segentry, segbase, out, flags, TailQueue{});
  if (!ok()) return GIC_ERR_CUDA;
  int flag = 0;
  if (cudaMemcpyAsync(&flag, flags, sizeof(int), cudaMemcpyDeviceToHost, cs) != cudaSuccess ||
      cudaStreamSynchronize(cs) != cudaSuccess) {
    cudaGetLastError();
    return GIC_ERR_CUDA;
  }
  *underrun = flag != 0;
  return GIC_OK;
}

}  // namespace gic

extern "C" GIC_API int gic_gaussian_stream_noalloc(unsigned long seed, size_t n, double *device_out, void *stream) {
  if (n == 0) return GIC_OK;
  if (!device_out || n > gic::kNoallocMaxGauss) return GIC_ERR_INVALID_ARG;
  cudaStream_t cs = static_cast<cudaStream_t>(stream);
  // The stream is drawn with a margin of raw numbers over the expected count;
  // on the (rare) underrun the margin grows by 1.5, through the same margins
  // as gic_gaussian_stream's (1, 1.5, 2.25, 3.375, 5.0625), for as long as the
  // longer stream still fits the scratch array.
  bool underrun = true;
  int st = GIC_OK;
  for (double margin = 1.0; underrun && margin < 6.0; margin *= 1.5) {
    st = gic::noalloc_run(seed, n, device_out, cs, margin, &underrun);
    if (st == GIC_ERR_NOT_READY) return GIC_ERR_INTERNAL;  // the longer stream does not fit
    if (st != GIC_OK) return st;
  }
  return underrun ? GIC_ERR_INTERNAL : GIC_OK;
}
