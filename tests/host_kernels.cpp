// Host build of the decode kernel (csrc/grand_decode.cuh with grand_triage.cuh
// and grand_search.cuh) on emulated warps, for the CPU parity tests
// (tests/test_host_kernels.py).
//
// The kernel runs as one thread block: one host thread per lane, the lanes of a
// warp meeting at a barrier in every warp collective (ballot, shuffles,
// reductions, votes, __syncwarp), the block's __shared__ arrays as static
// storage, device atomics as host atomics, a nap as a yield.  The kernel's code
// keeps its lanes converged at every collective, so it runs here as on the GPU,
// the order of the warps' work aside (which never changes a result: every
// search result is an exact minimum).  The block's warps classify, triage and
// search as the GPU's do, waiting for one another's published work.  Code
// tables are built as the library builds them.  GRAND_EMU_FAST=0 sends every
// shot through the per-shot path.
//
// Usage: host_kernels DIR   reads DIR/params.txt, DIR/H.bin, DIR/rec.bin (int32
// records) and, for a CSS code, DIR/Hother.bin (the other check matrix) or, for
// a DEM, DIR/L.bin (m x n_logicos) and DIR/log.bin (true logical flips), plus
// DIR/llr.txt for ML; writes DIR/res.bin (72-byte results), DIR/dec.bin (decoded
// errors, a byte per column and shot) and, for a DEM, DIR/declog.bin (decoded
// logical flips) and DIR/cost.bin (ML costs, FP32).  With DIR/mixed.txt it runs
// one batch that mixes several codes instead (see main).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

// ---- thread and warp emulation ------------------------------------------------
struct Idx3 {
  unsigned x, y, z;
};
static thread_local Idx3 threadIdx;
static Idx3 blockIdx = {0, 0, 0}, blockDim = {0, 1, 1}, gridDim = {1, 1, 1};

// a warp's meeting point: the last lane to arrive opens the next generation;
// the others spin briefly, then yield (lanes far outnumber host cores)
struct LaneBarrier {
  std::atomic<int> count{0}, gen{0};
  void arrive_and_wait() {
    const int g = gen.load(std::memory_order_acquire);
    if (count.fetch_add(1, std::memory_order_acq_rel) == 31) {
      count.store(0, std::memory_order_relaxed);
      gen.fetch_add(1, std::memory_order_release);
      return;
    }
    for (int spin = 0; gen.load(std::memory_order_acquire) == g; ++spin)
      if (spin > 64) std::this_thread::yield();
  }
};
struct WarpState {
  LaneBarrier bar;
  unsigned long long v[32];
};
static thread_local WarpState *tl_warp = nullptr;

template <class F>
static auto collective(unsigned long long mine, F f) {
  const unsigned lane = threadIdx.x & 31;
  tl_warp->v[lane] = mine;
  tl_warp->bar.arrive_and_wait();
  auto r = f(tl_warp->v, lane);
  tl_warp->bar.arrive_and_wait();
  return r;
}
static inline void __syncwarp(unsigned = 0xffffffffu) { tl_warp->bar.arrive_and_wait(); }
static inline unsigned __ballot_sync(unsigned, int p) {
  return collective((unsigned long long)(p != 0), [](const unsigned long long *v, unsigned) {
    unsigned m = 0;
    for (int i = 0; i < 32; ++i) m |= (unsigned)(v[i] & 1ull) << i;
    return m;
  });
}
static inline int __any_sync(unsigned m, int p) { return __ballot_sync(m, p) != 0u; }
static inline int __all_sync(unsigned m, int p) { return __ballot_sync(m, p) == 0xffffffffu; }
template <class T>
static inline T __shfl_sync(unsigned, T x, int src) {
  unsigned long long u = 0;
  memcpy(&u, &x, sizeof(T));
  return collective(u, [src](const unsigned long long *v, unsigned) {
    T r;
    memcpy(&r, &v[src & 31], sizeof(T));
    return r;
  });
}
template <class T>
static inline T __shfl_xor_sync(unsigned, T x, int m) {
  unsigned long long u = 0;
  memcpy(&u, &x, sizeof(T));
  return collective(u, [m](const unsigned long long *v, unsigned lane) {
    T r;
    memcpy(&r, &v[(lane ^ (unsigned)m) & 31], sizeof(T));
    return r;
  });
}
template <class T>
static inline T __shfl_up_sync(unsigned, T x, unsigned d) {
  unsigned long long u = 0;
  memcpy(&u, &x, sizeof(T));
  return collective(u, [d](const unsigned long long *v, unsigned lane) {
    T r;
    memcpy(&r, &v[lane >= d ? lane - d : lane], sizeof(T));
    return r;
  });
}
static inline unsigned __reduce_min_sync(unsigned, unsigned x) {
  return collective(x, [](const unsigned long long *v, unsigned) {
    unsigned r = 0xffffffffu;
    for (int i = 0; i < 32; ++i) r = std::min(r, (unsigned)v[i]);
    return r;
  });
}
static inline unsigned __reduce_max_sync(unsigned, unsigned x) {
  return collective(x, [](const unsigned long long *v, unsigned) {
    unsigned r = 0u;
    for (int i = 0; i < 32; ++i) r = std::max(r, (unsigned)v[i]);
    return r;
  });
}
template <class T>
static inline T __shfl_down_sync(unsigned, T x, unsigned d) {
  unsigned long long u = 0;
  memcpy(&u, &x, sizeof(T));
  return collective(u, [d](const unsigned long long *v, unsigned lane) {
    T r;
    memcpy(&r, &v[lane + d < 32 ? lane + d : lane], sizeof(T));
    return r;
  });
}
static inline unsigned __funnelshift_r(unsigned lo, unsigned hi, unsigned sh) {
  const unsigned long long v = ((unsigned long long)hi << 32) | lo;
  return (unsigned)(v >> (sh & 31));
}
static inline void grand_host_nap(int) { std::this_thread::yield(); }
static inline int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
static inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline unsigned __float_as_uint(float f) {
  unsigned u;
  memcpy(&u, &f, 4);
  return u;
}
static inline float __uint_as_float(unsigned u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
static inline long long __double_as_longlong(double d) {
  long long u;
  memcpy(&u, &d, 8);
  return u;
}
static inline unsigned __vimin3_u32(unsigned a, unsigned b, unsigned c) {
  return std::min(a, std::min(b, c));
}
template <class T>
static inline T __ldg(const T *p) {
  T r;
  memcpy(&r, p, sizeof(T));
  return r;
}
template <class T>
static inline T __ldcg(const T *p) {
  T r;
  memcpy(&r, p, sizeof(T));
  return r;
}
static inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline void __threadfence() { __atomic_thread_fence(__ATOMIC_SEQ_CST); }
static inline unsigned long long atomicAdd(unsigned long long *a, unsigned long long v) {
  return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST);
}
static inline unsigned atomicAdd(unsigned *a, unsigned v) {
  return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST);
}
static inline unsigned atomicOr(unsigned *a, unsigned v) {
  return __atomic_fetch_or(a, v, __ATOMIC_SEQ_CST);
}
static inline unsigned long long atomicMin(unsigned long long *a, unsigned long long v) {
  unsigned long long cur = __atomic_load_n(a, __ATOMIC_SEQ_CST);
  while (v < cur &&
         !__atomic_compare_exchange_n(a, &cur, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
  }
  return cur;
}
static inline unsigned long long atomicMax(unsigned long long *a, unsigned long long v) {
  unsigned long long cur = __atomic_load_n(a, __ATOMIC_SEQ_CST);
  while (v > cur &&
         !__atomic_compare_exchange_n(a, &cur, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
  }
  return cur;
}
static inline unsigned atomicCAS(unsigned *a, unsigned cmp, unsigned v) {
  __atomic_compare_exchange_n(a, &cmp, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return cmp;
}
static inline unsigned long long atomicCAS(unsigned long long *a, unsigned long long cmp,
                                           unsigned long long v) {
  __atomic_compare_exchange_n(a, &cmp, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return cmp;
}
static std::mutex g_cas_mu;
static inline void grand_host_cas128(unsigned long long *slot, unsigned long long c0,
                                     unsigned long long c1, unsigned long long n0,
                                     unsigned long long n1, unsigned long long *g0,
                                     unsigned long long *g1) {
  std::lock_guard<std::mutex> lk(g_cas_mu);
  *g0 = slot[0];
  *g1 = slot[1];
  if (*g0 == c0 && *g1 == c1) {
    slot[0] = n0;
    slot[1] = n1;
  }
}

// a block's __shared__ arrays: static storage shared by the block's host threads
#undef __shared__
#define __shared__ static
#ifndef __launch_bounds__
#define __launch_bounds__(...)
#endif
#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif

#define GRAND_HOST_EMULATION 1
#include "grand_decode.cuh"
#include "grand_solo.h"

using namespace grand;

// run body on blockDim.x host threads, one emulated warp per 32 lanes
static void run_block(int threads, const std::function<void()> &body) {
  blockDim.x = (unsigned)threads;
  std::vector<WarpState> warps(threads / 32);
  std::vector<std::thread> th;
  for (int t = 0; t < threads; ++t)
    th.emplace_back([&, t] {
      threadIdx.x = (unsigned)t;
      tl_warp = &warps[t / 32];
      body();
    });
  for (auto &x : th) x.join();
}

static std::vector<int> read_ints(const std::string &path, size_t n) {
  std::vector<int> v(n);
  FILE *f = fopen(path.c_str(), "rb");
  if (!f || fread(v.data(), 4, n, f) != n) {
    fprintf(stderr, "cannot read %s\n", path.c_str());
    exit(2);
  }
  fclose(f);
  return v;
}

static unsigned long long C(int n, int k) {
  if (k < 0 || n < k) return 0;
  unsigned long long r = 1;
  for (int i = 1; i <= k; ++i) r = r * (unsigned long long)(n - k + i) / (unsigned long long)i;
  return r;
}

// One code: its parameters (DIR/params.txt), its matrices and, for ML, its LLRs,
// with the code tables built as the library builds them.
struct Code {
  int family = 0, variant = 0, input_kind = 0, n = 0, m = 0, N = 0, W = 0, nl = 0, packed = 0;
  int light = 12, tile_k = 4, rec_len = 0, log_len = 0;
  std::vector<uint32_t> cols, hcol, rows, lcols;
  std::vector<int> colw, pivrow;
  SoloTable solo;
  std::vector<float> llr;
  DevCode d;
};

static bool load_code(const std::string &dir, Code &k) {
  FILE *pf = fopen((dir + "/params.txt").c_str(), "r");
  if (!pf) return false;
  int mode, thr, cap, num_phases, n_masks;
  if (fscanf(pf, "%d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d", &k.family, &k.variant,
             &k.input_kind, &k.n, &k.m, &k.N, &k.W, &mode, &thr, &cap, &num_phases, &n_masks,
             &k.light, &k.tile_k, &k.nl, &k.packed) != 16)
    return false;
  DevCode &d = k.d;
  memset(&d, 0, sizeof(d));
  for (int q = 0; q < n_masks; ++q)
    if (fscanf(pf, "%d %d %d %d", &d.mask_tam_upper[q], &d.mask_order[q][0], &d.mask_order[q][1],
               &d.mask_order[q][2]) != 4)
      return false;
  fclose(pf);
  const int n = k.n, m = k.m, nl = k.nl;
  const bool dem = k.family == kDem;
  const std::vector<int> H = read_ints(dir + "/H.bin", (size_t)n * m);
  const std::vector<int> Ho = dem ? std::vector<int>() : read_ints(dir + "/Hother.bin", (size_t)n * m);
  const std::vector<int> L = dem ? read_ints(dir + "/L.bin", (size_t)m * nl) : std::vector<int>();
  // records: one int32 per entry, or LSB-first uint32 words when packed
  const int entries = k.input_kind == kInErrors ? m : n;
  k.rec_len = k.packed ? (entries + 31) / 32 : entries;
  k.log_len = k.packed ? (nl + 31) / 32 : nl;
  k.llr.assign(m, 0.0f);
  if (k.variant == kMl) {  // the library's reader: fscanf("%f") per column
    FILE *lf = fopen((dir + "/llr.txt").c_str(), "r");
    if (!lf) return false;
    for (int i = 0; i < m; ++i)
      if (fscanf(lf, "%f", &k.llr[i]) != 1) return false;
    fclose(lf);
  }
  const int nw = (n + 31) / 32;
  const int nwp = nw <= 2 ? nw : (nw <= 4 ? 4 : (nw <= 8 ? 8 : (nw + 3) & ~3));
  const int mw = (m + 31) / 32;
  k.cols.assign((size_t)m * nwp, 0u);
  k.hcol.assign(m, 0u);
  k.colw.assign(m, 0);
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < m; ++c)
      if (H[(size_t)r * m + c] != 0) {
        ++k.colw[c];
        k.cols[(size_t)c * nwp + (r >> 5)] |= 1u << (r & 31);
        k.hcol[c] ^= row_hash(r);
      }
  // the solo-column table, as the library builds it
  k.solo = build_solo_table(k.cols, nwp, nw, m, k.hcol);
  int binary = 1;
  for (size_t i = 0; i < H.size(); ++i)
    if (H[i] != 0 && H[i] != 1) binary = 0;
  int max_soma = 0, regular = 1;
  for (int c = 0; c < m; ++c) max_soma = std::max(max_soma, k.colw[c]);
  for (int c = 1; c < m; ++c)
    if (k.colw[c] != k.colw[0]) regular = 0;
  k.rows.assign(dem ? 0 : (size_t)n * mw, 0u);
  for (int r = 0; r < n && !dem; ++r)
    for (int c = 0; c < m; ++c)
      if (Ho[(size_t)r * m + c] & 1) k.rows[(size_t)r * mw + (c >> 5)] |= 1u << (c & 31);
  k.pivrow.assign(m, -1);
  int rank = 0;
  for (int c = 0; c < m && rank < n && !dem; ++c) {  // reduced row echelon form over GF(2)
    const int q = c >> 5;
    const uint32_t bit = 1u << (c & 31);
    int p = -1;
    for (int i = rank; i < n; ++i)
      if (k.rows[(size_t)i * mw + q] & bit) {
        p = i;
        break;
      }
    if (p < 0) continue;
    for (int j = 0; j < mw; ++j) std::swap(k.rows[(size_t)rank * mw + j], k.rows[(size_t)p * mw + j]);
    for (int i = 0; i < n; ++i)
      if (i != rank && (k.rows[(size_t)i * mw + q] & bit))
        for (int j = 0; j < mw; ++j) k.rows[(size_t)i * mw + j] ^= k.rows[(size_t)rank * mw + j];
    k.pivrow[c] = rank++;
  }
  const int nlw = (nl + 31) / 32;
  k.lcols.assign((size_t)m * std::max(nlw, 1), 0u);
  for (int c = 0; c < m && dem; ++c)
    for (int j = 0; j < nl; ++j)
      if (L[(size_t)c * nl + j] != 0) k.lcols[(size_t)c * nlw + (j >> 5)] |= 1u << (j & 31);
  d.R = n;
  d.m = m;
  d.nw = nw;
  d.nwp = nwp;
  d.mw = mw;
  d.max_soma = max_soma;
  d.regular = regular;
  d.family = dem ? kDem : kCss;
  d.n_logicos = nl;
  d.nlw = nlw;
  d.lcols = k.lcols.data();
  d.llr = k.llr.data();
  d.variant = k.variant;
  d.input_kind = k.input_kind;
  d.W = k.W;
  d.Wc = std::min(k.W, (int)kMaxW);
  d.mode = mode;
  d.thr = thr;
  d.cap = cap;
  d.num_phases = num_phases;
  d.n_masks = n_masks;
  d.rank = rank;
  d.rec_len = k.rec_len;
  d.packed = k.packed;
  d.cols = k.cols.data();
  d.colw = k.colw.data();
  d.rref = k.rows.data();
  d.pivrow = k.pivrow.data();
  d.hcol = k.hcol.data();
  d.binary = binary;
  d.solo_keys = k.solo.keys.data();
  d.solo_cols = k.solo.cols.data();
  d.solo_mask = k.solo.mask;
  return true;
}

static void write_bytes(const std::string &path, const void *p, size_t n) {
  FILE *f = fopen(path.c_str(), "wb");
  fwrite(p, 1, n, f);
  fclose(f);
}

// Both kernels over a batch, as the library launches them (counters zeroed).
static unsigned run_batch(DevBatch &b, int N) {
  static std::vector<unsigned long long> ncr;
  if (ncr.empty()) {
    ncr.resize((size_t)(kMaxTam + 1) * (kMaxW + 1));
    for (int a = 0; a <= kMaxTam; ++a)
      for (int k = 0; k <= kMaxW; ++k) ncr[(size_t)a * (kMaxW + 1) + k] = C(a, k);
  }
  const int max_jobs = std::max(N, 1);
  static std::vector<Job> jobs;
  jobs.assign(max_jobs, Job());
  alignas(128) static unsigned long long small[kCtlAllocBytes / 8];
  memset(small, 0, sizeof(small));
  const unsigned long long scratch_words = 8ull << 20;
  static std::vector<uint32_t> scratch;
  scratch.assign(scratch_words, 0u);
  static std::vector<int> deferred;
  static std::vector<unsigned long long> queue;
  static std::vector<uint32_t> rec_cache;
  deferred.assign(N, 0);
  queue.assign(std::max(N, 1), 0ull);
  rec_cache.assign((size_t)std::max(N, 1) * kRecCacheWords, 0xa5a5a5a5u);
  b.num_shots = N;
  b.ncr = ncr.data();
  b.jobs = jobs.data();
  b.max_jobs = max_jobs;
  b.counters = small;
  b.status = reinterpret_cast<unsigned *>(reinterpret_cast<char *>(small) + kStatusByteOffset);
  b.scratch = scratch.data();
  b.scratch_words = scratch_words;
  b.deferred = deferred.data();
  b.queue = queue.data();
  // GRAND_EMU_CACHE=0: the per-shot path reads every record again instead
  const char *fc = getenv("GRAND_EMU_CACHE");
  b.rec_cache = (fc && *fc == '0') ? nullptr : rec_cache.data();
  b.epoch = reinterpret_cast<unsigned *>(reinterpret_cast<char *>(small) + kCtlBytes);
  const char *fe = getenv("GRAND_EMU_FAST");
  b.fast = (fe && *fe == '0') ? 0 : 1;
  run_block(kDecodeWarps * 32, [&] {
    if (b.has_ml) decode_kernel<true>(b);
    else decode_kernel<false>(b);
  });
  for (int i = 0; i < N; ++i)
    if (deferred[i]) {
      fprintf(stderr, "shot %d deferred (status %u)\n", i, *b.status);
      exit(3);
    }
  printf("ok %d shots, %llu jobs, %llu slow, status %u\n", N,
         *ctr_ptr(small, kCtrJobs) >> 40, *ctr_ptr(small, kCtrSlowDone), *b.status);
  return *b.status;
}

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  const std::string dir = argv[1];
  DevBatch b;
  memset(&b, 0, sizeof(b));

  // a mixed batch: DIR/mixed.txt = "K N light tile_k", codes in DIR/code<k>/, the
  // shots' records back to back in DIR/rec.bin with DIR/off.bin (int64 start of
  // each record) and DIR/code.bin (int32 code of each shot); results only
  if (FILE *mf = fopen((dir + "/mixed.txt").c_str(), "r")) {
    int K, N, light, tile_k;
    if (fscanf(mf, "%d %d %d %d", &K, &N, &light, &tile_k) != 4) return 2;
    fclose(mf);
    std::vector<Code> codes(K);
    std::vector<DevCode> dcs(K);
    for (int k = 0; k < K; ++k) {
      if (!load_code(dir + "/code" + std::to_string(k), codes[k])) return 2;
      dcs[k] = codes[k].d;
      b.has_ml |= codes[k].variant == kMl;
    }
    FILE *rf = fopen((dir + "/rec.bin").c_str(), "rb");
    if (!rf) return 2;
    fseek(rf, 0, SEEK_END);
    const size_t total = (size_t)ftell(rf) / 4;
    fclose(rf);
    const std::vector<int> rec = read_ints(dir + "/rec.bin", total);
    std::vector<long long> off(N);
    FILE *of = fopen((dir + "/off.bin").c_str(), "rb");
    if (!of || fread(off.data(), 8, N, of) != (size_t)N) return 2;
    fclose(of);
    const std::vector<int> shot_code = read_ints(dir + "/code.bin", N);
    std::vector<GrandDecoderResult> res(N);
    b.num_codes = K;
    b.codes = dcs.data();
    b.in = rec.data();
    b.in_off = off.data();
    b.shot_code = shot_code.data();
    b.results = res.data();
    b.light_max_log2 = light;
    b.tile_k = tile_k;
    run_batch(b, N);
    write_bytes(dir + "/res.bin", res.data(), sizeof(GrandDecoderResult) * N);
    return 0;
  }

  Code k;
  if (!load_code(dir, k)) return 2;
  const int N = k.N, m = k.m, nl = k.nl;
  const bool dem = k.family == kDem;
  const std::vector<int> rec = read_ints(dir + "/rec.bin", (size_t)N * k.rec_len);
  const std::vector<int> logicals =
      dem ? read_ints(dir + "/log.bin", (size_t)N * std::max(k.log_len, 1)) : std::vector<int>();
  std::vector<GrandDecoderResult> res(N);
  std::vector<unsigned char> dec((size_t)N * m, 0), declog((size_t)N * std::max(nl, 1), 0);
  std::vector<float> cost(N, 0.0f);
  b.num_codes = 1;
  b.codes = &k.d;
  b.in = rec.data();
  b.results = res.data();
  b.dec_err = dec.data();
  if (dem) {
    b.in_log = logicals.data();
    b.dec_log = declog.data();
    b.ml_cost = k.variant == kMl ? cost.data() : nullptr;
  }
  b.light_max_log2 = k.light;
  b.tile_k = k.tile_k;
  b.has_ml = k.variant == kMl;
  run_batch(b, N);
  write_bytes(dir + "/res.bin", res.data(), sizeof(GrandDecoderResult) * N);
  write_bytes(dir + "/dec.bin", dec.data(), dec.size());
  if (dem) {
    write_bytes(dir + "/declog.bin", declog.data(), (size_t)N * nl);
    write_bytes(dir + "/cost.bin", cost.data(), sizeof(float) * N);
  }
  return 0;
}
