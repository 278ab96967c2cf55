// grand_device.cuh -- device building blocks of the GRAND search (sm_103a).
//
// Enumeration.  Upstream enumerates the weight-w subsets of the active positions
// in lexicographic order of ascending index tuples (grand_decoder.cu:83-100,
// 264-280) and its CPU mode returns the lowest-ranked match.  Here a weight-w
// candidate is split into a (w-1)-prefix and a last index j > prefix max.  The
// prefixes are dealt out in colex order, one prefix per lane, so the 32 lanes of
// a warp usually share the same prefix maximum; the warp then walks j in
// lockstep and every lane reads the same staged column (a shared-memory
// broadcast).  Per candidate a lane does one XOR of 32-bit column sketches
// against the sketch of s ^ (the prefix columns) and half a 3-way min: the
// prefix sketch is updated incrementally when the prefix advances, never
// recomputed per candidate, and a zero sketch is confirmed word by word.
// Matches are mapped back to their lexicographic rank, so the reduction is an
// exact minimum over the rank upstream would have reached first, whatever order
// the tiles run in.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "grand_common.h"

namespace grand {

constexpr unsigned kFull = 0xffffffffu;
constexpr unsigned long long kNone = ~0ull;

// Nanoseconds of the GPU's global timer (the per-shot timing fields).
__device__ __forceinline__ unsigned long long global_ns() {
#ifdef GRAND_HOST_EMULATION  // the host build of the kernels used by the CPU tests
  return 0ull;
#else
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
#endif
}

__device__ __forceinline__ unsigned long long ncr(const unsigned long long *t, int n, int k) {
  if (n < 0 || k < 0 || n > kMaxTam || k > kMaxW) return 0ull;
  return __ldg(t + n * (kMaxW + 1) + k);
}

// C(n, k) for k <= 6 by upstream's multiplicative formula (grand_decoder.cu:42-52)
// with constant divisors: each step r * (n - i + 1) / i is exact and stays below
// 2^64 for n <= 2048.  No table load, so a chain of them costs no memory latency.
__device__ __forceinline__ unsigned long long binom(int n, int k) {
  if (k < 0 || n < k) return 0ull;
  const unsigned long long m = (unsigned long long)n;
  unsigned long long r = 1ull;
  if (k >= 1) r = m;
  if (k >= 2) r = r * (m - 1ull) / 2ull;
  if (k >= 3) r = r * (m - 2ull) / 3ull;
  if (k >= 4) r = r * (m - 3ull) / 4ull;
  if (k >= 5) r = r * (m - 4ull) / 5ull;
  if (k >= 6) r = r * (m - 5ull) / 6ull;
  return r;
}

// Largest v in [lo, hi] with C(v, k) <= q (C(v, k) is non-decreasing in v there).
__device__ __forceinline__ int ncr_floor(const unsigned long long *t, unsigned long long q, int k,
                                         int lo, int hi) {
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (ncr(t, mid, k) <= q) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Colex unranking of a k-subset of [0, hi + 1): ascending x[0..k-1].
__device__ __forceinline__ void colex_unrank(const unsigned long long *t, unsigned long long q,
                                             int k, int hi, int (&x)[5]) {
#pragma unroll
  for (int i = 4; i >= 0; --i) {
    if (i < k) {
      int v = ncr_floor(t, q, i + 1, i, hi);
      q -= ncr(t, v, i + 1);
      x[i] = v;
      hi = v - 1;
    }
  }
}

// Largest i in [lo, hi] with key(i) <= x, for key non-decreasing and
// key(lo) <= x.  Each step the 32 lanes probe 32 points of the range, so n
// entries take ceil(log32 n) dependent loads instead of log2 n.
template <class Key>
__device__ __forceinline__ int warp_search_le(int lo, int hi, unsigned long long x, Key key) {
  const int lane = threadIdx.x & 31;
  while (lo < hi) {
    const long long span = (long long)hi - lo + 1;
    const unsigned m = __ballot_sync(kFull, key(lo + (int)((lane * span) >> 5)) <= x);
    const int l = 31 - __clz(m);  // lane 0 probes lo, so m != 0
    const int nlo = lo + (int)((l * span) >> 5);
    hi = (l == 31) ? hi : lo + (int)(((l + 1) * span) >> 5) - 1;
    lo = nlo;
  }
  return lo;
}

// Lexicographic unranking (upstream order): rank -> ascending c[0..w-1] of
// [0, n), through the colex rank of the reflected subset {n-1-c}, by the whole
// warp: each element's binomial search probes 32 points per step
// (warp_search_le) and computes the binomials instead of loading them, so a
// result writer's unranking is a few rounds of ballots with no dependent memory
// loads.  Every lane gets c.
__device__ __forceinline__ void lex_unrank_warp(unsigned long long rank, int n, int w,
                                                int (&c)[kMaxW]) {
  unsigned long long q = binom(n, w) - 1ull - rank;
  int hi = n - 1;
#pragma unroll
  for (int i = kMaxW; i >= 1; --i) {
    if (i <= w) {
      const int v = warp_search_le(i - 1, hi, q, [&](int x) { return binom(x, i); });
      q -= binom(v, i);
#pragma unroll
      for (int e = 0; e < kMaxW; ++e)  // c[w - i], with constant indices
        if (e == w - i) c[e] = n - 1 - v;
      hi = v - 1;
    }
  }
}

// Lexicographic rank of prefix x[0..k-1] followed by last index j (k = w - 1).
__device__ __forceinline__ unsigned long long lex_rank(const unsigned long long *t, int n, int w,
                                                       const int (&x)[5], int k, int j) {
  unsigned long long r = ncr(t, n, w) - 1ull;
#pragma unroll
  for (int i = 0; i < 5; ++i)
    if (i < k) r -= ncr(t, n - 1 - x[i], w - i);
  r -= (unsigned long long)(n - 1 - j);
  return r;
}

// FP32 cost -> unsigned key with the same order (costs are never -0.0: the sum
// starts from +0.0f, as upstream's does, grand_decoder.cu:641).
__device__ __forceinline__ uint32_t cost_key(float c) {
  uint32_t u = __float_as_uint(c);
  if (c == 0.0f) u = 0u;
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_cost(uint32_t k) {
  uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  return __uint_as_float(u);
}

// What one tile evaluation needs to know about its weight block.
struct SegView {
  const uint32_t *hcols;  // tam column sketches of the active columns (staged)
  const uint32_t *cols;   // tam x nwp active columns (exact test of sketch hits)
  const float *llr;       // tam LLRs in the same order (ML)
  uint32_t hs;            // sketch of the syndrome
  int tam, w, K, nwp, nw;
  unsigned long long nprefix;
  unsigned long long base;  // global index of rank 0 (first-hit)
};

struct LaneBest {
  unsigned long long g;     // first-hit: lowest global index
  uint32_t o;               // ML: lowest cost key
  unsigned long long r;     // ML: its lexicographic rank
  __device__ __forceinline__ void reset() { g = kNone; o = 0xffffffffu; r = kNone; }
};

// Exact test of a sketch hit: the syndrome XOR the columns of prefix x[0..k-1]
// and of j is zero in every word.
__device__ __forceinline__ bool exact_match(const SegView &sv, const uint32_t *sw,
                                            const int (&x)[5], int k, int j) {
  for (int i = 0; i < sv.nw; ++i) {
    uint32_t z = sw[i] ^ sv.cols[(size_t)j * sv.nwp + i];
#pragma unroll
    for (int e = 0; e < 5; ++e)
      if (e < k) z ^= sv.cols[(size_t)x[e] * sv.nwp + i];
    if (z != 0u) return false;
  }
  return true;
}

// A verified match: its global index (first-hit) or {cost key, rank} (ML) into
// the lane's best.  ML costs add the LLRs in ascending position order.
template <bool ML>
__device__ __forceinline__ void record_match(const SegView &sv, const unsigned long long *t,
                                             const int (&x)[5], int k, int j, LaneBest &lb) {
  const unsigned long long r = lex_rank(t, sv.tam, sv.w, x, k, j);
  if constexpr (!ML) {
    const unsigned long long g = sv.base + r;
    if (g < lb.g) lb.g = g;
  } else {
    float c = 0.0f;
#pragma unroll
    for (int e = 0; e < 5; ++e)
      if (e < k) c = __fadd_rn(c, sv.llr[x[e]]);
    c = __fadd_rn(c, sv.llr[j]);
    const uint32_t o = cost_key(c);
    if (o < lb.o || (o == lb.o && r < lb.r)) {
      lb.o = o;
      lb.r = r;
    }
  }
}

// ---------------------------------------------------------------------------
// Sketch filter.
//
// A candidate matches when s ^ col(p_1) ^ ... ^ col(p_w) = 0 over all ceil(R/32)
// words.  The scans below test a 32-bit linear sketch of that vector instead:
// h(s) ^ h(col p_1) ^ ... ^ h(col p_w), which is 0 for every match (h is linear
// and h(0) = 0) and, for a non-match, 0 only when the residual vector happens to
// lie in the kernel of h.  A zero sketch is then tested word by word
// (exact_match), so the result is exactly the word-by-word search's; the filter
// only decides how much work a non-match costs: one XOR and half a 3-way minimum
// per candidate, whatever the number of check rows.
// ---------------------------------------------------------------------------

// Evaluate one colex tile: lane l takes the K colex prefixes tile*32K + l*K + [0, K).
template <bool ML>
__device__ __forceinline__ void eval_tile(const SegView &sv, const unsigned long long *t,
                                          const uint32_t *sw, unsigned long long tile,
                                          LaneBest &lb) {
  const int lane = threadIdx.x & 31;
  const int k = sv.w - 1;
  const int tam = sv.tam;
  const uint32_t *hc = sv.hcols;

  unsigned long long q = tile * (32ull * (unsigned long long)sv.K) + (unsigned long long)lane * sv.K;
  bool valid = q < sv.nprefix;
  int x[5] = {0, 0, 0, 0, 0};
  uint32_t h = sv.hs;
  int clast = -1;
  if (valid && k > 0) {
    if (k == 1) x[0] = (int)q;  // a 1-subset's colex rank is its element
    else colex_unrank(t, q, k, tam - 2, x);
#pragma unroll
    for (int i = 0; i < 5; ++i)
      if (i < k) {
        h ^= hc[x[i]];
        clast = x[i];
      }
  }

  for (int step = 0; step < sv.K; ++step) {
    const bool v = valid && (q + step < sv.nprefix);
    const int cl = v ? clast : tam;
    const int lo = (int)__reduce_min_sync(kFull, (unsigned)(cl + 1));
    const int hi = (int)__reduce_max_sync(kFull, v ? (unsigned)(cl + 1) : 0u) - 1;
    uint32_t acc = 0xffffffffu;
    int j = lo;
    const int ahi = hi < tam - 1 ? hi : tam - 1;
    for (; j <= ahi; ++j) {
      const uint32_t z = h ^ hc[j];
      if (j > cl) acc = min(acc, z);
    }
    if (j < hi + 1) j = hi + 1;
#pragma unroll 4
    for (; j < tam; ++j) acc = min(acc, h ^ hc[j]);

    if (v && acc == 0u) {
      // A zero sketch for this prefix: test those candidates word by word (rare).
      for (int jj = cl + 1; jj < tam; ++jj) {
        if ((h ^ hc[jj]) != 0u || !exact_match(sv, sw, x, k, jj)) continue;
        record_match<ML>(sv, t, x, k, jj, lb);
        if constexpr (!ML) break;  // ranks grow with the last index
      }
    }

    if (step + 1 < sv.K && v && k > 0) {
      // Colex successor: raise the lowest element that has room, reset those below.
      int adv = -1;
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        if (i < k && adv < 0) {
          int lim = tam - 1;
          if (i + 1 < 5 && i + 1 < k) lim = x[(i + 1) < 5 ? i + 1 : 4];
          if (x[i] + 1 < lim) adv = i;
        }
      }
      if (adv < 0) {
        valid = false;
      } else {
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          if (i < k && i <= adv) {
            const int old = x[i];
            const int nv = (i == adv) ? old + 1 : i;
            if (nv != old) {
              h ^= hc[old] ^ hc[nv];
              x[i] = nv;
            }
          }
        }
#pragma unroll
        for (int i = 0; i < 5; ++i)
          if (i < k) clast = x[i];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Register-blocked run tiles for weights >= 3.
//
// The (w-1)-prefixes whose largest element is c form one contiguous colex run
// of C(c, w-2) prefixes (their other w-2 elements are any subset of [0, c)).  A
// run tile gives each lane KK consecutive prefixes of one run, so every prefix
// in the warp has the same largest element: the warp walks j = c+1 .. tam-1 in
// lockstep with no masking, loads sketch j once (shared-memory broadcast) and
// XORs it into the KK prefix sketches each lane keeps in registers.
// ---------------------------------------------------------------------------

// Colex successor of an ascending kk-subset y of [0, c); returns the highest
// changed position (elements 0..adv changed), -1 when exhausted.
__device__ __forceinline__ int colex_next(int (&y)[5], int kk, int c) {
  int adv = -1;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    if (i < kk && adv < 0) {
      int lim = c;
      if (i + 1 < 5 && i + 1 < kk) lim = y[(i + 1) < 5 ? i + 1 : 4];
      if (y[i] + 1 < lim) adv = i;
    }
  }
  if (adv >= 0) {
#pragma unroll
    for (int i = 0; i < 5; ++i)
      if (i < kk && i <= adv) y[i] = (i == adv) ? y[i] + 1 : i;
  }
  return adv;
}

// Colex unranking of a 2-subset: y1 = largest v with C(v, 2) <= r (from the
// float square root, then corrected), y0 = the rest.
__device__ __forceinline__ void unrank2(unsigned long long r, int &y0, int &y1) {
  int v = (int)((1.0f + sqrtf(1.0f + 8.0f * (float)r)) * 0.5f);
  if (v < 1) v = 1;
  while ((unsigned long long)v * (v - 1) / 2 > r) --v;
  while ((unsigned long long)(v + 1) * v / 2 <= r) ++v;
  y1 = v;
  y0 = (int)(r - (unsigned long long)v * (v - 1) / 2);
}

// Largest v in [lo, hi] with C(v, k) <= q, from the estimate C(v, k) ~
// (v - (k - 1) / 2)^k / k! corrected with computed binomials (no table loads).
__device__ __forceinline__ int binom_floor(unsigned long long q, int k, int lo, int hi) {
  const float fact = k == 4 ? 24.0f : (k == 5 ? 120.0f : (k == 3 ? 6.0f : (k == 2 ? 2.0f : 1.0f)));
  int v = (int)(powf(fact * (float)q, 1.0f / (float)k) + 0.5f * (float)(k - 1));
  v = v < lo ? lo : (v > hi ? hi : v);
  while (v > lo && binom(v, k) > q) --v;
  while (v < hi && binom(v + 1, k) <= q) ++v;
  return v;
}

// Colex unranking of a kk-subset of [0, c): closed forms for kk <= 3 (weights 3
// to 5, the common case), estimated and corrected binomial searches otherwise.
__device__ __forceinline__ void sub_unrank(const unsigned long long *t, unsigned long long r,
                                           int kk, int c, int (&y)[5]) {
  if (kk == 1) {
    y[0] = (int)r;
  } else if (kk == 2) {
    unrank2(r, y[0], y[1]);
  } else if (kk == 3) {
    // largest v with C(v, 3) <= r, from the float cube root, then corrected
    int v = (int)cbrtf(6.0f * (float)r) + 1;
    if (v < 2) v = 2;
    auto c3 = [](int x) { return (unsigned long long)x * (x - 1) * (x - 2) / 6; };
    while (v > 2 && c3(v) > r) --v;
    while (c3(v + 1) <= r) ++v;
    y[2] = v;
    unrank2(r - c3(v), y[0], y[1]);
  } else {
    int hi = c - 1;
#pragma unroll
    for (int i = 4; i >= 0; --i) {
      if (i < kk) {
        const int v = binom_floor(r, i + 1, i, hi);
        r -= binom(v, i + 1);
        y[i] = v;
        hi = v - 1;
      }
    }
  }
}

// Colex successor inside a run (the caller only asks for existing successors).
__device__ __forceinline__ int sub_next(int (&y)[5], int kk, int c) {
  if (kk == 1) {
    ++y[0];
    return 0;
  }
  if (kk == 2) {
    if (y[0] + 1 < y[1]) {
      ++y[0];
      return 0;
    }
    ++y[1];
    y[0] = 0;
    return 1;
  }
  return colex_next(y, kk, c);
}

// One run tile: run c, lane l takes prefixes r0 + l*KK + [0, KK) of the run.
template <int KK, bool ML>
__device__ __forceinline__ void eval_run_tile(const SegView &sv, const unsigned long long *t,
                                              const uint32_t *sw, int c, unsigned long long r0,
                                              LaneBest &lb) {
  const int lane = threadIdx.x & 31;
  const int k = sv.w - 1;   // prefix length (>= 2)
  const int kk = k - 1;     // elements below c (>= 1)
  const int tam = sv.tam;
  const uint32_t *hc = sv.hcols;
  const unsigned long long run = ncr(t, c, kk);
  const unsigned long long r = r0 + (unsigned long long)lane * KK;
  const int v = r >= run ? 0 : (int)((run - r) < (unsigned long long)KK ? (run - r) : KK);

  const uint32_t hb = sv.hs ^ hc[c];
  uint32_t H[KK];  // sketches of s ^ (the lane's prefixes); lanes past the run repeat one
  if (kk == 1) {
    // weight 3: prefixes {y, c}, y = r, r+1, ...
    const int y0 = v > 0 ? (int)r : 0;
#pragma unroll
    for (int s = 0; s < KK; ++s) H[s] = hb ^ hc[s < v ? y0 + s : y0];
  } else if (kk == 2) {
    // weight 4: prefixes {y0, y1, c} in colex order, y0 < y1 < c
    int y[5] = {0, 1, 2, 3, 4};
    if (v > 0) sub_unrank(t, r, 2, c, y);
    int y0 = y[0], y1 = y[1];
    uint32_t h1 = hb ^ hc[y1];
#pragma unroll
    for (int s = 0; s < KK; ++s) {
      H[s] = h1 ^ hc[y0];
      if (s + 1 < v) {
        if (++y0 == y1) {
          y0 = 0;
          h1 = hb ^ hc[++y1];
        }
      }
    }
  } else if (kk == 3) {
    // weight 5: prefixes {y0, y1, y2, c} in colex order
    int y[5] = {0, 1, 2, 3, 4};
    if (v > 0) sub_unrank(t, r, 3, c, y);
    int y0 = y[0], y1 = y[1], y2 = y[2];
    uint32_t h2 = hb ^ hc[y2];
    uint32_t h1 = h2 ^ hc[y1];
#pragma unroll
    for (int s = 0; s < KK; ++s) {
      H[s] = h1 ^ hc[y0];
      if (s + 1 < v) {
        if (++y0 == y1) {
          y0 = 0;
          if (++y1 == y2) {
            y1 = 1;
            h2 = hb ^ hc[++y2];
          }
          h1 = h2 ^ hc[y1];
        }
      }
    }
  } else {
    int y[5] = {0, 1, 2, 3, 4};
    if (v > 0) sub_unrank(t, r, kk, c, y);
    H[0] = hb;
#pragma unroll
    for (int e = 0; e < 5; ++e)
      if (e < kk) H[0] ^= hc[y[e]];
#pragma unroll
    for (int s = 1; s < KK; ++s) {
      H[s] = H[s - 1];
      if (s < v) {
        int old[5];
#pragma unroll
        for (int e = 0; e < 5; ++e) old[e] = y[e];
        const int adv = sub_next(y, kk, c);
#pragma unroll
        for (int e = 0; e < 5; ++e)
          if (e < kk && e <= adv && old[e] != y[e]) H[s] ^= hc[old[e]] ^ hc[y[e]];
      }
    }
  }

  uint32_t acc = 0xffffffffu;
#pragma unroll 4
  for (int j = c + 1; j < tam; ++j) {
    const uint32_t hj = hc[j];
    if constexpr (KK % 2 == 0) {
#pragma unroll
      for (int s = 0; s < KK; s += 2) acc = __vimin3_u32(acc, H[s] ^ hj, H[s + 1] ^ hj);
    } else {
#pragma unroll
      for (int s = 0; s < KK; ++s) acc = min(acc, H[s] ^ hj);
    }
  }

  if (v > 0 && acc == 0u) {
    // A zero sketch among this lane's prefixes (rare): rescan, and test each
    // (prefix, j) whose sketch is zero word by word.  Lanes without valid
    // prefixes only repeat prefix 0's sketch and never get here.
    for (int j = c + 1; j < tam; ++j) {
      const uint32_t hj = hc[j];
#pragma unroll
      for (int s = 0; s < KK; ++s) {
        if (s < v && (H[s] ^ hj) == 0u) {
          int yy[5] = {0, 1, 2, 3, 4};
          sub_unrank(t, r + (unsigned long long)s, kk, c, yy);
          int x[5];
#pragma unroll
          for (int e = 0; e < 5; ++e) x[e] = (e < kk) ? yy[e] : (e == kk ? c : 0);
          if (exact_match(sv, sw, x, k, j)) record_match<ML>(sv, t, x, k, j, lb);
        }
      }
    }
  }
}

// Number of run tiles of run c for weight w (KK prefixes per lane).
__device__ __forceinline__ unsigned long long run_tiles(const unsigned long long *t, int c, int w,
                                                        int KK) {
  const unsigned long long n = binom(c, w - 2);
  const unsigned long long per = 32ull * (unsigned long long)KK;
  return (n + per - 1ull) / per;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long u = __shfl_xor_sync(kFull, v, o);
    v = u < v ? u : v;
  }
  return v;
}

__device__ __forceinline__ void warp_min_key(uint32_t &o, unsigned long long &r) {
#pragma unroll
  for (int s = 16; s > 0; s >>= 1) {
    uint32_t o2 = __shfl_xor_sync(kFull, o, s);
    unsigned long long r2 = __shfl_xor_sync(kFull, r, s);
    if (o2 < o || (o2 == o && r2 < r)) {
      o = o2;
      r = r2;
    }
  }
}

// 128-bit compare-and-swap minimum of {cost key, rank} (lexicographic).
__device__ __forceinline__ bool atomic_min_key(unsigned long long *slot, uint32_t o,
                                               unsigned long long r) {
  unsigned long long cur0 = *reinterpret_cast<volatile unsigned long long *>(slot);
  unsigned long long cur1 = *reinterpret_cast<volatile unsigned long long *>(slot + 1);
  for (int guard = 0; guard < (1 << 20); ++guard) {
    if ((unsigned long long)o > cur0 || ((unsigned long long)o == cur0 && r >= cur1)) return true;
    unsigned long long got0, got1;
#ifdef GRAND_HOST_EMULATION  // the host build supplies the 128-bit CAS
    grand_host_cas128(slot, cur0, cur1, (unsigned long long)o, r, &got0, &got1);
#else
    asm volatile(
        "{\n\t.reg .b128 d, c, n;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 n, {%4, %5};\n\t"
        "atom.global.cas.b128 d, [%6], c, n;\n\t"
        "mov.b128 {%0, %1}, d;\n\t}"
        : "=l"(got0), "=l"(got1)
        : "l"(cur0), "l"(cur1), "l"((unsigned long long)o), "l"(r), "l"(slot)
        : "memory");
#endif
    if (got0 == cur0 && got1 == cur1) return true;
    cur0 = got0;
    cur1 = got1;
  }
  return false;
}

}  // namespace grand
