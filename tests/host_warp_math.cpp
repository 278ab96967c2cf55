// Host build of the search's warp-level device code (csrc/grand_device.cuh,
// csrc/grand_lookup.cuh)
// on an emulated warp: 32 host threads, one per lane, whose warp collectives
// (ballot, shuffles, reductions, votes, __syncwarp) meet at a barrier, so code
// that keeps its lanes converged at every collective runs as on the GPU.
// Checked against plain combinatorics and brute force: the 32-way warp search,
// the warp-parallel lexicographic unranking of the result writer, the warp
// minima, whole masked colex tiles (weights 1-6) first-hit and ML, the lookup
// tables (csrc/grand_lookup.cuh) and whole lookup tiles (weights 1-6) first-hit
// and ML.
// Prints "ok" or the first mismatch (exit 1).
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
#include <random>
#include <thread>
#include <vector>

struct LaneIndex {
  unsigned x, y, z;
};
static thread_local LaneIndex threadIdx;

// ---- the emulated warp ------------------------------------------------------
// the warp's meeting point: the last lane to arrive opens the next generation;
// the others spin briefly, then yield (lanes outnumber host cores)
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
static WarpState *g_warp = nullptr;

// every lane publishes one value; all lanes read all of them; a second barrier
// keeps the next collective from overwriting values still being read
template <class F>
static auto collective(unsigned long long mine, F f) {
  const unsigned lane = threadIdx.x & 31;
  g_warp->v[lane] = mine;
  g_warp->bar.arrive_and_wait();
  auto r = f(g_warp->v, lane);
  g_warp->bar.arrive_and_wait();
  return r;
}
static inline void __syncwarp(unsigned = 0xffffffffu) { g_warp->bar.arrive_and_wait(); }
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
static inline unsigned __vimin3_u32(unsigned a, unsigned b, unsigned c) {
  return std::min(a, std::min(b, c));
}
template <class T>
static inline T __ldg(const T *p) {
  return *p;
}
static inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }
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
static inline unsigned atomicOr(unsigned *a, unsigned v) {
  return __atomic_fetch_or(a, v, __ATOMIC_SEQ_CST);
}
static inline unsigned atomicAdd(unsigned *a, unsigned v) {
  return __atomic_fetch_add(a, v, __ATOMIC_SEQ_CST);
}
// the host build of the device headers (global timer, shared-memory loads and
// the 128-bit CAS swapped for host equivalents)
#define GRAND_HOST_EMULATION 1
static inline void grand_host_cas128(unsigned long long *slot, unsigned long long c0,
                                     unsigned long long c1, unsigned long long n0,
                                     unsigned long long n1, unsigned long long *g0,
                                     unsigned long long *g1) {
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  *g0 = slot[0];
  *g1 = slot[1];
  if (slot[0] == c0 && slot[1] == c1) {
    slot[0] = n0;
    slot[1] = n1;
  }
}
#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif

#include "grand_device.cuh"
#include "grand_lookup.cuh"

using namespace grand;

// run body(lane) on 32 lane threads; returns false if any lane reported failure
static bool run_warp(const std::function<bool(unsigned)> &body) {
  WarpState w;
  g_warp = &w;
  bool ok[32];
  std::vector<std::thread> th;
  for (unsigned l = 0; l < 32; ++l)
    th.emplace_back([&, l] {
      threadIdx.x = l;
      ok[l] = body(l);
    });
  for (auto &t : th) t.join();
  g_warp = nullptr;
  for (bool b : ok)
    if (!b) return false;
  return true;
}

static unsigned long long C(int n, int k) {
  if (k < 0 || n < k) return 0;
  unsigned long long r = 1;
  for (int i = 1; i <= k; ++i) r = r * (unsigned long long)(n - k + i) / (unsigned long long)i;
  return r;
}

#define FAIL(...)                 \
  do {                            \
    fprintf(stderr, __VA_ARGS__); \
    fprintf(stderr, "\n");        \
    return 1;                     \
  } while (0)

int main() {
  std::vector<unsigned long long> t((size_t)(kMaxTam + 1) * (kMaxW + 1));
  for (int n = 0; n <= kMaxTam; ++n)
    for (int k = 0; k <= kMaxW; ++k) t[(size_t)n * (kMaxW + 1) + k] = C(n, k);
  std::mt19937_64 rng(97);

  // warp minima
  for (int trial = 0; trial < 50; ++trial) {
    unsigned long long vals[32];
    uint32_t os[32];
    unsigned long long rs[32];
    for (int l = 0; l < 32; ++l) {
      vals[l] = rng() % 50;
      os[l] = (uint32_t)(rng() % 4);
      rs[l] = rng() % 8;
    }
    unsigned long long want = *std::min_element(vals, vals + 32);
    uint32_t wo = 0xffffffffu;
    unsigned long long wr = ~0ull;
    for (int l = 0; l < 32; ++l)
      if (os[l] < wo || (os[l] == wo && rs[l] < wr)) {
        wo = os[l];
        wr = rs[l];
      }
    const bool ok = run_warp([&](unsigned l) {
      const unsigned long long m = warp_min_u64(vals[l]);
      uint32_t o = os[l];
      unsigned long long r = rs[l];
      warp_min_key(o, r);
      return m == want && o == wo && r == wr;
    });
    if (!ok) FAIL("warp minima, trial %d", trial);
  }

  // lexicographic unranking by the warp: every lane gets the tuple of the rank
  for (int trial = 0; trial < 150; ++trial) {
    const int n = 1 + (int)(rng() % 300);
    const int w = 1 + (int)(rng() % std::min(n, kMaxW));
    const unsigned long long total = C(n, w);
    const unsigned long long rank = rng() % total;
    // brute force for small cases, else check the rank round trip
    int want[kMaxW] = {0, 0, 0, 0, 0, 0};
    bool brute = total <= 200000ull;
    if (brute) {
      std::vector<int> x(w);
      for (int i = 0; i < w; ++i) x[i] = i;
      for (unsigned long long r = 0; r < rank; ++r) {
        int i = w - 1;
        while (x[i] == n - w + i) --i;
        ++x[i];
        for (int j = i + 1; j < w; ++j) x[j] = x[j - 1] + 1;
      }
      for (int i = 0; i < w; ++i) want[i] = x[i];
    }
    const bool ok = run_warp([&](unsigned) {
      int c[kMaxW];
      lex_unrank_warp(rank, n, w, c);
      for (int i = 0; i < w; ++i) {
        if (c[i] < 0 || c[i] >= n || (i > 0 && c[i] <= c[i - 1])) return false;
        if (brute && c[i] != want[i]) return false;
      }
      if (w >= 2) {
        int p[5] = {0, 0, 0, 0, 0};
        for (int i = 0; i < w - 1 && i < 5; ++i) p[i] = c[i];
        if (w <= 6 && lex_rank(t.data(), n, w, p, w - 1, c[w - 1]) != rank) return false;
      } else if ((unsigned long long)c[0] != rank) {
        return false;
      }
      return true;
    });
    if (!ok) FAIL("lex_unrank_warp n=%d w=%d rank=%llu", n, w, rank);
  }

  // masked colex tiles (the weight blocks a warp scans without run tiles)
  int cases = 0, matched = 0;
  for (int trial = 0; trial < 70; ++trial) {
    const int tam = 2 + (int)(rng() % 30);
    const int w = 1 + (int)(rng() % 6);
    if (w > tam || C(tam, w) > 400000ull) continue;
    const int K = 1 + (int)(rng() % 6);
    const int R = 6 + (int)(rng() % 58), nw = (R + 31) / 32, nwp = nw == 1 ? 1 : 2;
    std::vector<uint32_t> cols((size_t)tam * nwp, 0u), hc(tam), sw(32, 0u);
    for (int c = 0; c < tam; ++c)
      for (int r = 0; r < R; ++r)
        if (rng() & 1) cols[(size_t)c * nwp + r / 32] |= 1u << (r % 32);
    if (rng() % 3 == 0) {
      const int a = (int)(rng() % tam), b = (int)(rng() % tam);
      for (int i = 0; i < nwp; ++i) cols[(size_t)a * nwp + i] = cols[(size_t)b * nwp + i];
    }
    if (rng() % 4) {
      std::vector<int> pick(tam);
      for (int i = 0; i < tam; ++i) pick[i] = i;
      std::shuffle(pick.begin(), pick.end(), rng);
      for (int e = 0; e < w; ++e)
        for (int i = 0; i < nw; ++i) sw[i] ^= cols[(size_t)pick[e] * nwp + i];
    } else {
      for (int i = 0; i < nw; ++i) sw[i] = (uint32_t)rng();
      if (R % 32) sw[nw - 1] &= (1u << (R % 32)) - 1u;
    }
    auto sketch = [&](const uint32_t *v) {
      uint32_t h = 0;
      for (int r = 0; r < R; ++r)
        if ((v[r / 32] >> (r % 32)) & 1u) h ^= row_hash(r);
      return h;
    };
    for (int c = 0; c < tam; ++c) hc[c] = sketch(&cols[(size_t)c * nwp]);
    std::vector<float> llr(tam);
    for (auto &v : llr) v = (float)(1 + rng() % 6) * 0.25f;
    const SegView sv{hc.data(), cols.data(), llr.data(), sketch(sw.data()), tam, w, K,
                     nwp, nw, w >= 2 ? C(tam - 1, w - 1) : 1ull, 500ull};
    const unsigned long long ntiles = (sv.nprefix + 32ull * K - 1) / (32ull * K);
    // brute force in lexicographic order
    unsigned long long bg = kNone, br = kNone;
    uint32_t bo = 0xffffffffu;
    {
      std::vector<int> x(w);
      for (int i = 0; i < w; ++i) x[i] = i;
      for (unsigned long long r = 0;; ++r) {
        bool eq = true;
        for (int i = 0; i < nw && eq; ++i) {
          uint32_t z = sw[i];
          for (int e = 0; e < w; ++e) z ^= cols[(size_t)x[e] * nwp + i];
          eq = z == 0u;
        }
        if (eq) {
          if (bg == kNone) bg = sv.base + r;
          float cst = 0.0f;
          for (int e = 0; e < w; ++e) cst = cst + llr[x[e]];
          const uint32_t k2 = cost_key(cst);
          if (k2 < bo || (k2 == bo && r < br)) {
            bo = k2;
            br = r;
          }
        }
        int i = w - 1;
        while (i >= 0 && x[i] == tam - w + i) --i;
        if (i < 0) break;
        ++x[i];
        for (int j = i + 1; j < w; ++j) x[j] = x[j - 1] + 1;
      }
    }
    for (int ml = 0; ml < 2; ++ml) {
      unsigned long long got_g = kNone, got_r = kNone;
      uint32_t got_o = 0xffffffffu;
      const bool ok = run_warp([&](unsigned) {
        LaneBest lb;
        lb.reset();
        for (unsigned long long tile = 0; tile < ntiles; ++tile) {
          if (ml) eval_tile<true>(sv, t.data(), sw.data(), tile, lb);
          else eval_tile<false>(sv, t.data(), sw.data(), tile, lb);
        }
        const unsigned long long g = warp_min_u64(lb.g);
        uint32_t o = lb.o;
        unsigned long long r = lb.r;
        warp_min_key(o, r);
        if ((threadIdx.x & 31) == 0) {
          got_g = g;
          got_o = o;
          got_r = r;
        }
        return true;
      });
      if (!ok) FAIL("colex tile run failed");
      if (!ml && got_g != bg) FAIL("colex tiles first-hit tam=%d w=%d K=%d: %llu vs %llu", tam, w, K, got_g, bg);
      if (ml && (got_o != bo || got_r != br)) FAIL("colex tiles ML tam=%d w=%d K=%d", tam, w, K);
      ++cases;
      matched += (!ml && bg != kNone);
    }
  }
  if (cases < 60 || matched < 15) FAIL("too few colex-tile cases: %d (%d matched)", cases, matched);
  printf("ok %d colex-tile cases\n", cases);

  // lookup tables: every column is found through the filter and its bucket, the
  // buckets partition the columns by their sketch's top bits, and a sketch that
  // is no column passes the filter about as rarely as the layout promises
  std::vector<uint32_t> stage(4096);
  for (int tam : {1, 2, 5, 17, 31, 64, 126, 300, 700, 1500, 2048}) {
    std::vector<uint32_t> hc(tam);
    for (auto &v : hc) v = (uint32_t)rng();
    if (tam > 3) hc[tam - 1] = hc[1];  // two columns with one sketch
    const LookLayout L = look_layout(tam, 2720);
    std::vector<uint32_t> blk((size_t)L.words + 4, 0xdeadbeefu);
    for (int i = 0; i < tam; ++i) blk[i] = hc[i];
    if (!run_warp([&](unsigned) {
          build_lookup(blk.data(), tam, L);
          return true;
        }))
      FAIL("build_lookup failed");
    const LookView lk = look_view(blk.data(), L);
    const int nb = 1 << L.B;
    if (lk.bst[0] != 0u || lk.bst[nb] != (uint32_t)tam) FAIL("bucket bounds tam=%d", tam);
    for (int b = 0; b < nb; ++b) {
      if (lk.bst[b] > lk.bst[b + 1]) FAIL("bucket bounds not monotone tam=%d", tam);
      for (uint32_t e = lk.bst[b]; e < lk.bst[b + 1]; ++e)
        if ((lk.key[e] >> lk.shift) != (uint32_t)b || hc[lk.pos[e]] != lk.key[e])
          FAIL("bucket entry tam=%d b=%d", tam, b);
    }
    for (int i = 0; i < tam; ++i) {
      const uint32_t m = bloom_bits(hc[i], L.F);
      if ((lk.filt[hc[i] & lk.wmask] & m) != m) FAIL("filter misses column %d tam=%d", i, tam);
      const uint32_t b = hc[i] >> lk.shift;
      bool seen = false;
      for (uint32_t e = lk.bst[b]; e < lk.bst[b + 1]; ++e) seen = seen || (lk.pos[e] == i);
      if (!seen) FAIL("bucket misses column %d tam=%d", i, tam);
    }
    int pass = 0;
    const int probes = 200000;
    for (int q = 0; q < probes; ++q) {
      const uint32_t h = (uint32_t)rng();
      const uint32_t m = bloom_bits(h, L.F);
      pass += (lk.filt[h & lk.wmask] & m) == m;
    }
    // each word holds Poisson(tam / 2^(F-5)) columns' three bits: E[(3b/32)^3] bounds
    // the pass rate of a random sketch from above (bits can coincide)
    const double lam = (double)tam / (double)(1 << (L.F - 5));
    const double bound = 27.0 / 32768.0 * (lam * lam * lam + 3 * lam * lam + lam);
    if ((double)pass / probes > 2.0 * bound + 1e-4) FAIL("filter pass rate %g > %g tam=%d", (double)pass / probes, bound, tam);
  }
  printf("ok lookup tables\n");

  // lookup tiles (the Jobs' search) against brute force, first-hit and ML
  int lcases = 0, lmatched = 0;
  for (int trial = 0; trial < 90; ++trial) {
    const int tam = 1 + (int)(rng() % 140);
    const int w = 1 + (int)(rng() % 6);
    if (w > tam || C(tam, w) > 3000000ull) continue;
    const int R = 6 + (int)(rng() % 90), nw = (R + 31) / 32, nwp = nw == 1 ? 1 : (nw == 2 ? 2 : 4);
    std::vector<uint32_t> cols((size_t)tam * nwp, 0u), hc(tam), sw(32, 0u);
    for (int c = 0; c < tam; ++c)
      for (int r = 0; r < R; ++r)
        if (rng() % 4 == 0) cols[(size_t)c * nwp + r / 32] |= 1u << (r % 32);
    if (rng() % 3 == 0) {
      const int a = (int)(rng() % tam), b = (int)(rng() % tam);
      for (int i = 0; i < nwp; ++i) cols[(size_t)a * nwp + i] = cols[(size_t)b * nwp + i];
    }
    if (rng() % 4) {
      std::vector<int> pick(tam);
      for (int i = 0; i < tam; ++i) pick[i] = i;
      std::shuffle(pick.begin(), pick.end(), rng);
      for (int e = 0; e < w; ++e)
        for (int i = 0; i < nw; ++i) sw[i] ^= cols[(size_t)pick[e] * nwp + i];
    } else {
      for (int i = 0; i < nw; ++i) sw[i] = (uint32_t)rng();
      if (R % 32) sw[nw - 1] &= (1u << (R % 32)) - 1u;
    }
    auto sketch = [&](const uint32_t *v) {
      uint32_t h = 0;
      for (int r = 0; r < R; ++r)
        if ((v[r / 32] >> (r % 32)) & 1u) h ^= row_hash(r);
      return h;
    };
    for (int c = 0; c < tam; ++c) hc[c] = sketch(&cols[(size_t)c * nwp]);
    std::vector<float> llr(tam);
    for (auto &v : llr) v = (float)(1 + rng() % 6) * 0.25f;
    const LookLayout L = look_layout(tam, 2720);
    std::vector<uint32_t> blk((size_t)L.words + 8, 0u);
    for (int i = 0; i < tam; ++i) blk[i] = hc[i];
    if (!run_warp([&](unsigned) {
          build_lookup(blk.data(), tam, L);
          return true;
        }))
      FAIL("build_lookup failed");
    const LookView lk = look_view(blk.data(), L);
    const SegView sv{blk.data(), cols.data(), llr.data(), sketch(sw.data()), tam, w, kLookK,
                     nwp, nw, C(tam - 1, w - 1), 700ull};
    const unsigned long long ntiles = lookup_tiles(sv.nprefix);
    unsigned long long bg = kNone, br = kNone;
    uint32_t bo = 0xffffffffu;
    {
      std::vector<int> x(w);
      for (int i = 0; i < w; ++i) x[i] = i;
      for (unsigned long long r = 0;; ++r) {
        bool eq = true;
        for (int i = 0; i < nw && eq; ++i) {
          uint32_t z = sw[i];
          for (int e = 0; e < w; ++e) z ^= cols[(size_t)x[e] * nwp + i];
          eq = z == 0u;
        }
        if (eq) {
          if (bg == kNone) bg = sv.base + r;
          float cst = 0.0f;
          for (int e = 0; e < w; ++e) cst = cst + llr[x[e]];
          const uint32_t k2 = cost_key(cst);
          if (k2 < bo || (k2 == bo && r < br)) {
            bo = k2;
            br = r;
          }
        }
        int i = w - 1;
        while (i >= 0 && x[i] == tam - w + i) --i;
        if (i < 0) break;
        ++x[i];
        for (int j = i + 1; j < w; ++j) x[j] = x[j - 1] + 1;
      }
    }
    for (int ml = 0; ml < 2; ++ml) {
      unsigned long long got_g = kNone, got_r = kNone;
      uint32_t got_o = 0xffffffffu;
      const bool ok = run_warp([&](unsigned) {
        LaneBest acc;
        acc.reset();
        for (unsigned long long tile = 0; tile < ntiles; ++tile) {
          const LaneBest lb = ml ? eval_lookup_tile<kLookK, true, true>(sv, lk, t.data(), sw.data(), tile)
                                 : eval_lookup_tile<kLookK, false, true>(sv, lk, t.data(), sw.data(), tile);
          if (lb.g < acc.g) acc.g = lb.g;
          if (lb.o < acc.o || (lb.o == acc.o && lb.r < acc.r)) {
            acc.o = lb.o;
            acc.r = lb.r;
          }
        }
        const unsigned long long g = warp_min_u64(acc.g);
        uint32_t o = acc.o;
        unsigned long long r = acc.r;
        warp_min_key(o, r);
        if ((threadIdx.x & 31) == 0) {
          got_g = g;
          got_o = o;
          got_r = r;
        }
        return true;
      });
      if (!ok) FAIL("lookup tile run failed");
      if (!ml && got_g != bg) FAIL("lookup tiles first-hit tam=%d w=%d: %llu vs %llu", tam, w, got_g, bg);
      if (ml && (got_o != bo || got_r != br)) FAIL("lookup tiles ML tam=%d w=%d", tam, w);
    }
    ++lcases;
    lmatched += bg != kNone;
  }
  if (lcases < 50 || lmatched < 25) FAIL("too few lookup-tile cases: %d (%d matched)", lcases, lmatched);
  printf("ok %d lookup-tile cases\n", lcases);
  return 0;
}
