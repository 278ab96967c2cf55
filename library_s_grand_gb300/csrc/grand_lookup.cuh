// grand_lookup.cuh -- the prefix-lookup search of a Job's weight blocks (sm_103a).
//
// A weight-w candidate is a (w-1)-prefix P (ascending positions of the active
// list) followed by a last index j > max(P).  It matches when
//   s ^ col(P) ^ col(j) = 0,
// and its 32-bit sketch (grand_device.cuh) is then h(s) ^ h(P) ^ hcol[j] = 0,
// that is hcol[j] = h(s) ^ h(P).  So instead of testing every j against every
// prefix, the iteration's column sketches go into a small hash set, and each
// prefix asks it once for the positions j whose sketch equals h(s) ^ h(P).  Each
// position returned with j > max(P) is confirmed word by word (exact_match) and
// recorded under its lexicographic rank exactly as a scan records it, so the
// answer -- the lowest-rank match, or for ML every match's cost -- is the scan's.
// A prefix costs O(1) whatever the number of its candidates (tam - 1 - max(P)).
//
// Per heavy iteration the Job's scratch holds one contiguous lookup block, built
// once by the publishing warp and copied into a search warp's shared-memory
// stage when the warp starts on that iteration:
//   hc     tam column sketches (in active-list order)
//   filt   a 2^F-bit filter: bit (hc & (2^F - 1)) set for every column
//   bst    2^B + 1 bucket starts (u16): the entries of bucket b (top B bits of the
//          sketch) are key/pos[bst[b] .. bst[b+1])
//   key    the tam sketches grouped by bucket
//   pos    their active-list indices (u16)
// A probe reads one filter word; only when its bit is set (about tam / 2^F of
// prefixes that match nothing) does it walk the bucket.  Filter and buckets use
// disjoint bits of the sketch (F + B <= 26).
#pragma once

#include "grand_device.cuh"

namespace grand {

constexpr int kLookK = 16;        // prefixes per lane in a lookup tile
constexpr int kLookMaxF = 15;     // largest filter (2^15 bits = 4 KB)
constexpr int kLookMinF = 10;

struct LookLayout {
  int F, B;                       // filter bits, bucket bits (log2)
  int o_filt, o_bst, o_key, o_pos;  // word offsets inside the block (hc at 0)
  int words;                      // block size in words (a multiple of 4)
};

GRAND_HD inline int ceil_log2i(int x) {
  int b = 0;
  while ((1 << b) < x) ++b;
  return b;
}

// Layout of the lookup block of an active set of tam positions.  The filter is
// as large as the stage (cap_words) allows, up to 2^15 bits and down to 2^10; a
// block that still does not fit is read from the Job's scratch instead of the
// stage (the same tables, slower loads).
GRAND_HD inline LookLayout look_layout(int tam, int cap_words) {
  LookLayout L;
  const int t4 = (tam + 3) & ~3;
  L.B = ceil_log2i(tam);
  if (L.B < 1) L.B = 1;
  const int nb = 1 << L.B;
  const int bst_words = ((nb + 2) / 2 + 3) & ~3;
  const int pos_words = ((tam + 1) / 2 + 3) & ~3;
  int F = ceil_log2i(tam) + 7;
  if (F > kLookMaxF) F = kLookMaxF;
  if (F < kLookMinF) F = kLookMinF;
  for (;;) {
    const int fw = 1 << (F - 5);
    const int words = t4 + fw + bst_words + t4 + pos_words;
    if (words <= cap_words || F == kLookMinF) {
      L.F = F;
      L.o_filt = t4;
      L.o_bst = t4 + fw;
      L.o_key = L.o_bst + bst_words;
      L.o_pos = L.o_key + t4;
      L.words = words;
      return L;
    }
    --F;
  }
}

// Build the tables of a block whose first tam words already hold the column
// sketches (one warp; T is shared scratch of at least max(2^(F-5), 2^(B-1) + 1)
// words).  Entries of one bucket land in any order: a probe checks them all.
__device__ __forceinline__ void build_lookup(uint32_t *blk, int tam, const LookLayout &L,
                                             uint32_t *T) {
  const int lane = threadIdx.x & 31;
  uint32_t *filt = blk + L.o_filt;
  uint16_t *bst = reinterpret_cast<uint16_t *>(blk + L.o_bst);
  uint32_t *key = blk + L.o_key;
  uint16_t *pos = reinterpret_cast<uint16_t *>(blk + L.o_pos);
  const int fw = 1 << (L.F - 5);
  const uint32_t fmask = (1u << L.F) - 1u;
  const int shift = 32 - L.B;
  const int nb = 1 << L.B;

  // filter
  for (int i = lane; i < fw; i += 32) T[i] = 0u;
  __syncwarp();
  for (int i = lane; i < tam; i += 32) {
    const uint32_t f = blk[i] & fmask;
    atomicOr(&T[f >> 5], 1u << (f & 31u));
  }
  __syncwarp();
  for (int i = lane; i < fw; i += 32) filt[i] = T[i];
  __syncwarp();

  // bucket sizes, 16 bits each (two buckets per word; sizes and starts stay
  // below 2^16 because tam <= 2048)
  const int nbw = (nb + 1) >> 1;
  for (int i = lane; i <= nbw; i += 32) T[i] = 0u;
  __syncwarp();
  for (int i = lane; i < tam; i += 32) {
    const uint32_t bk = blk[i] >> shift;
    atomicAdd(&T[bk >> 1], 1u << ((bk & 1u) * 16u));
  }
  __syncwarp();
  // exclusive scan in bucket order: each lane an even-sized run of buckets (so
  // no two lanes touch one word), then the lanes' totals across the warp
  const int per = nb / 32 > 2 ? nb / 32 : 2;
  const int b0 = lane * per;
  int mine = 0;
  for (int bk = b0; bk < b0 + per && bk < nb; ++bk) mine += (T[bk >> 1] >> ((bk & 1) * 16)) & 0xffffu;
  int incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += u;
  }
  int run = incl - mine;
  for (int bk = b0; bk < b0 + per && bk < nb; ++bk) {
    const unsigned sh = (unsigned)(bk & 1) * 16u;
    const int cnt = (int)((T[bk >> 1] >> sh) & 0xffffu);
    bst[bk] = (uint16_t)run;
    T[bk >> 1] = (T[bk >> 1] & ~(0xffffu << sh)) | ((uint32_t)run << sh);  // the bucket's cursor
    run += cnt;
  }
  if (lane == 0) bst[nb] = (uint16_t)tam;
  __syncwarp();
  // scatter
  for (int i = lane; i < tam; i += 32) {
    const uint32_t h = blk[i];
    const uint32_t bk = h >> shift;
    const unsigned sh = (bk & 1u) * 16u;
    const uint32_t old = atomicAdd(&T[bk >> 1], 1u << sh);
    const int slot = (int)((old >> sh) & 0xffffu);
    key[slot] = h;
    pos[slot] = (uint16_t)i;
  }
  __syncwarp();
}

// Where a warp reads an iteration's lookup tables (its stage or the scratch).
struct LookView {
  const uint32_t *filt;
  const uint16_t *bst;
  const uint32_t *key;
  const uint16_t *pos;
  uint32_t fmask;
  int shift;
};

__device__ __forceinline__ LookView look_view(const uint32_t *blk, const LookLayout &L) {
  LookView v;
  v.filt = blk + L.o_filt;
  v.bst = reinterpret_cast<const uint16_t *>(blk + L.o_bst);
  v.key = blk + L.o_key;
  v.pos = reinterpret_cast<const uint16_t *>(blk + L.o_pos);
  v.fmask = (1u << L.F) - 1u;
  v.shift = 32 - L.B;
  return v;
}

// The candidates of prefix x[0..k-1] (largest element cl, sketch h = h(s) ^ h(P)):
// every j > cl whose column sketch equals h, confirmed word by word.
template <bool ML>
__device__ __forceinline__ void probe_prefix(const SegView &sv, const LookView &lk,
                                             const unsigned long long *t, const uint32_t *sw,
                                             uint32_t h, const int (&x)[5], int k, int cl,
                                             LaneBest &lb) {
  const uint32_t f = h & lk.fmask;
  if (!((lk.filt[f >> 5] >> (f & 31u)) & 1u)) return;
  const uint32_t bk = h >> lk.shift;
  const int e1 = lk.bst[bk + 1];
  for (int e = lk.bst[bk]; e < e1; ++e) {
    if (lk.key[e] != h) continue;
    const int j = lk.pos[e];
    if (j > cl && exact_match(sv, sw, x, k, j)) record_match<ML>(sv, t, x, k, j, lb);
  }
}

// One lookup tile: lane l takes the K colex-consecutive prefixes
// tile * 32K + l * K + [0, K) of the block's C(tam - 1, w - 1) prefixes (ascending
// (w-1)-subsets of [0, tam - 1), so each has at least one j above it).  The
// prefix sketch is updated incrementally: a colex step changes the lowest
// element (one staged sketch load) and, rarely, the ones above it.
template <int K, bool ML>
__device__ __forceinline__ void eval_lookup_tile(const SegView &sv, const LookView &lk,
                                                 const unsigned long long *t, const uint32_t *sw,
                                                 unsigned long long tile, LaneBest &lb) {
  const int lane = threadIdx.x & 31;
  const int k = sv.w - 1;
  const int tam = sv.tam;
  const uint32_t *hc = sv.hcols;
  const uint32_t hs = sv.hs;
  const unsigned long long q = tile * (32ull * K) + (unsigned long long)lane * K;
  if (q >= sv.nprefix) return;
  const int v = (sv.nprefix - q) < (unsigned long long)K ? (int)(sv.nprefix - q) : K;
  int x[5] = {0, 1, 2, 3, 4};
  if (k == 0) {  // weight 1: the empty prefix, every j
    probe_prefix<ML>(sv, lk, t, sw, hs, x, 0, -1, lb);
    return;
  }
  sub_unrank(t, q, k, tam - 1, x);
  if (k == 1) {
    for (int s = 0; s < v; ++s) {
      probe_prefix<ML>(sv, lk, t, sw, hs ^ hc[x[0]], x, 1, x[0], lb);
      ++x[0];
    }
  } else if (k == 2) {
    uint32_t h1 = hs ^ hc[x[1]];
    for (int s = 0; s < v; ++s) {
      probe_prefix<ML>(sv, lk, t, sw, h1 ^ hc[x[0]], x, 2, x[1], lb);
      if (++x[0] == x[1]) {
        x[0] = 0;
        h1 = hs ^ hc[++x[1]];
      }
    }
  } else if (k == 3) {
    uint32_t h2 = hs ^ hc[x[2]];
    uint32_t h1 = h2 ^ hc[x[1]];
    for (int s = 0; s < v; ++s) {
      probe_prefix<ML>(sv, lk, t, sw, h1 ^ hc[x[0]], x, 3, x[2], lb);
      if (++x[0] == x[1]) {
        x[0] = 0;
        if (++x[1] == x[2]) {
          x[1] = 1;
          h2 = hs ^ hc[++x[2]];
        }
        h1 = h2 ^ hc[x[1]];
      }
    }
  } else {
    uint32_t h = hs;
#pragma unroll
    for (int e = 0; e < 5; ++e)
      if (e < k) h ^= hc[x[e]];
    for (int s = 0; s < v; ++s) {
      int cl = x[0];
#pragma unroll
      for (int e = 0; e < 5; ++e)
        if (e < k) cl = x[e];
      probe_prefix<ML>(sv, lk, t, sw, h, x, k, cl, lb);
      if (s + 1 < v) {
        int old[5];
#pragma unroll
        for (int e = 0; e < 5; ++e) old[e] = x[e];
        const int adv = colex_next(x, k, tam - 1);
#pragma unroll
        for (int e = 0; e < 5; ++e)
          if (e < k && e <= adv && old[e] != x[e]) h ^= hc[old[e]] ^ hc[x[e]];
      }
    }
  }
}

// Lookup tiles of a weight block with nprefix prefixes.
GRAND_HD inline unsigned long long lookup_tiles(unsigned long long nprefix) {
  const unsigned long long per = 32ull * (unsigned long long)kLookK;
  return (nprefix + per - 1ull) / per;
}

}  // namespace grand
