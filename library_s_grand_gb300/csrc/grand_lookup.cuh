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
// A search warp that starts on an iteration copies the column sketches from the
// Job's scratch into its shared-memory stage and builds the tables there, so the
// lookup block of an iteration is (an active set too large for the stage has
// its block built once, in the scratch, by the publishing warp):
//   hc     tam column sketches (in active-list order)
//   filt   a 2^F-bit blocked Bloom filter: each column sets three bits of one
//          32-bit word (word = low F-5 bits of its sketch, bit positions = the
//          next three 5-bit fields)
//   bst    2^B + 1 bucket bounds (u32): the entries of bucket b (top B bits of
//          the sketch) are key/pos[bst[b] .. bst[b+1])
//   key    the tam sketches grouped by bucket
//   pos    their active-list indices (u16)
// A probe reads one filter word; only when all three of its bits are set does it
// walk the bucket.  A word holds the bits of Poisson(tam / 2^(F-5)) columns, so a
// prefix that matches nothing passes with probability about
// E[(3b/32)^3], b ~ Poisson(tam / 2^(F-5)): one in ~7000 at tam = 126 (F = 15).
#pragma once

#include "grand_device.cuh"

namespace grand {

constexpr int kLookK = 32;        // prefixes per lane in a lookup tile
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
  const int bst_words = (nb + 2 + 3) & ~3;
  const int pos_words = ((tam + 1) / 2 + 3) & ~3;
  int F = ceil_log2i(tam) + 8;
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

// The three filter bits of sketch h (in the word h & (2^(F-5) - 1)).
GRAND_HD inline uint32_t bloom_bits(uint32_t h, int F) {
  return (1u << ((h >> (F - 5)) & 31u)) | (1u << ((h >> F) & 31u)) | (1u << ((h >> (F + 5)) & 31u));
}

// Build the tables of a block whose first tam words already hold the column
// sketches (one warp; the block in shared memory, or in the scratch for an
// active set too large for the stage).  The bucket bounds double as counters:
// bst[b + 1] counts bucket b, becomes its start after the scan and its end (the
// next bucket's start) after the scatter, with bst[0] = 0 throughout.  Entries
// of one bucket land in any order: a probe checks them all.
__device__ __forceinline__ void build_lookup(uint32_t *blk, int tam, const LookLayout &L) {
  const int lane = threadIdx.x & 31;
  uint32_t *filt = blk + L.o_filt;
  uint32_t *bst = blk + L.o_bst;
  uint32_t *key = blk + L.o_key;
  uint16_t *pos = reinterpret_cast<uint16_t *>(blk + L.o_pos);
  const int fw = 1 << (L.F - 5);
  const int shift = 32 - L.B;
  const int nb = 1 << L.B;
  for (int i = lane; i < fw; i += 32) filt[i] = 0u;
  for (int i = lane; i < nb + 2; i += 32) bst[i] = 0u;
  __syncwarp();
  for (int i = lane; i < tam; i += 32) {
    const uint32_t h = blk[i];
    atomicOr(&filt[h & (uint32_t)(fw - 1)], bloom_bits(h, L.F));
    atomicAdd(&bst[(h >> shift) + 1u], 1u);
  }
  __syncwarp();
  // exclusive scan of the counts in place: each lane a run of buckets, then the
  // lanes' totals across the warp
  const int per = nb >= 32 ? nb / 32 : 1;
  const int b0 = 1 + lane * per;
  const int b1 = (b0 + per < nb + 1) ? b0 + per : nb + 1;
  uint32_t mine = 0u;
  for (int i = b0; i < b1; ++i) mine += bst[i];
  uint32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += u;
  }
  uint32_t run = incl - mine;
  for (int i = b0; i < b1; ++i) {
    const uint32_t c = bst[i];
    bst[i] = run;
    run += c;
  }
  __syncwarp();
  for (int i = lane; i < tam; i += 32) {
    const uint32_t h = blk[i];
    const uint32_t slot = atomicAdd(&bst[(h >> shift) + 1u], 1u);
    key[slot] = h;
    pos[slot] = (uint16_t)i;
  }
  __syncwarp();
}

// Where a warp reads an iteration's lookup tables (its stage or the scratch).
struct LookView {
  const uint32_t *filt;
  const uint32_t *bst;
  const uint32_t *key;
  const uint16_t *pos;
  uint32_t wmask;  // filter word index mask, 2^(F-5) - 1
  int F;
  int shift;
};

__device__ __forceinline__ LookView look_view(const uint32_t *blk, const LookLayout &L) {
  LookView v;
  v.filt = blk + L.o_filt;
  v.bst = blk + L.o_bst;
  v.key = blk + L.o_key;
  v.pos = reinterpret_cast<const uint16_t *>(blk + L.o_pos);
  v.wmask = (1u << (L.F - 5)) - 1u;
  v.F = L.F;
  v.shift = 32 - L.B;
  return v;
}

// Word i of a staged table at shared-memory address a (SH), or of p.
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
#ifdef GRAND_HOST_EMULATION
  (void)p;
  return 0u;
#else
  return (uint32_t)__cvta_generic_to_shared(p);
#endif
}
// (Not volatile: the tables do not change while a tile is evaluated, so the
// compiler may schedule and combine these loads freely inside the tile
// function, which is never inlined into code that rewrites the stage.)
template <bool SH>
__device__ __forceinline__ uint32_t tab_word(const uint32_t *p, uint32_t a, uint32_t i) {
#ifndef GRAND_HOST_EMULATION
  if constexpr (SH) {
    uint32_t v;
    asm("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a + 4u * i));
    return v;
  }
#endif
  (void)a;
  return p[i];
}

// The candidates of prefix x[0..k-1] (largest element cl, sketch h = h(s) ^ h(P))
// that passed the filter: every j > cl whose column sketch equals h, confirmed
// word by word.
template <bool ML>
__device__ __forceinline__ void probe_bucket(const SegView &sv, const LookView &lk,
                                             const unsigned long long *t, const uint32_t *sw,
                                             uint32_t h, const int (&x)[5], int k, int cl,
                                             LaneBest &lb) {
  const uint32_t bk = h >> lk.shift;
  const int e1 = (int)lk.bst[bk + 1];
  for (int e = (int)lk.bst[bk]; e < e1; ++e) {
    if (lk.key[e] != h) continue;
    const int j = lk.pos[e];
    if (j > cl && exact_match(sv, sw, x, k, j)) record_match<ML>(sv, t, x, k, j, lb);
  }
}

// Colex walk over the prefixes of one lane, for prefixes of KP elements
// (KP = 0: the runtime k, any length): x0 (the lowest element) rises under the
// upper elements x[1..k-1], whose sketch XOR h(s) is hu; when x0 meets x1 the
// upper elements take their colex successor.  For KP = 1..4 the carry is a few
// increments with the partial sketches kept (hp[e] = h(s) ^ hc[x_e] ^ .. ^
// hc[x_{k-1}]), so a lane that carries (while the others wait) costs little.
template <int KP>
struct PrefixWalk {
  int x[5];
  uint32_t hp[5];
  int k, tam;
  uint32_t hs;
  __device__ __forceinline__ int kk() const { return KP ? KP : k; }
  template <bool SH>
  __device__ __forceinline__ void start(const unsigned long long *t, unsigned long long q, int k_,
                                        int tam_, uint32_t hs_, const uint32_t *hc, uint32_t hca) {
    k = k_;
    tam = tam_;
    hs = hs_;
#pragma unroll
    for (int e = 0; e < 5; ++e) x[e] = e;
    sub_unrank(t, q, kk(), tam - 1, x);
    sketches<SH>(4, hc, hca);
  }
  // hp[e] for the upper elements from position e0 down to 1
  template <bool SH>
  __device__ __forceinline__ void sketches(int e0, const uint32_t *hc, uint32_t hca) {
    uint32_t h = hs;
#pragma unroll
    for (int e = 4; e >= 1; --e) {
      if (e < kk()) {
        if (e <= e0) hp[e] = (e + 1 < kk() ? hp[e < 4 ? e + 1 : 4] : hs) ^
                             tab_word<SH>(hc, hca, (uint32_t)x[e]);
        h = hp[e];
      }
    }
    hp[0] = kk() >= 2 ? h : hs;
  }
  __device__ __forceinline__ uint32_t hu() const { return hp[0]; }
  __device__ __forceinline__ int top() const {
    int t0 = x[0];
#pragma unroll
    for (int e = 1; e < 5; ++e)
      if (e < kk()) t0 = x[e];
    return t0;
  }
  template <bool SH>
  __device__ __forceinline__ void next(const uint32_t *hc, uint32_t hca) {
    const int k1 = kk();
    if (k1 == 1) {
      ++x[0];
      return;
    }
    if (x[0] + 1 < x[1]) {
      ++x[0];
      return;
    }
    // carry: the lowest upper element with room rises, those below restart
    int e = 1;
#pragma unroll
    for (int i = 1; i < 5; ++i)
      if (i < k1 && e == i && x[i] + 1 == (i + 1 < k1 ? x[i < 4 ? i + 1 : 4] : tam - 1)) e = i + 1;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      if (i < e) x[i] = i;
      else if (i == e) ++x[i];
    }
    sketches<SH>(e, hc, hca);
  }
};

// The scan of one lane's v prefixes starting at colex rank q (KP: prefix length,
// 0 = runtime).  Per prefix: its sketch hu ^ hc[x0] (one staged load), one
// filter load and a three-bit test, whose outcome is only ORed into a flag:
// the scan has no data-dependent branch but the carry into the upper elements,
// so the loads of consecutive prefixes overlap.  A lane whose flag is set
// (rare) walks its prefixes again and looks each filter hit up in the buckets.
template <int KP, int K, bool ML, bool SH>
__device__ __forceinline__ void scan_lane(const SegView &sv, const LookView &lk,
                                          const unsigned long long *t, const uint32_t *sw,
                                          unsigned long long q, int v, LaneBest &lb) {
  const int k = sv.w - 1;
  const uint32_t *hc = sv.hcols;
  const uint32_t hca = SH ? smem_addr(hc) : 0u, fa = SH ? smem_addr(lk.filt) : 0u;
  const uint32_t wmask = lk.wmask;
  const int F = lk.F;
  PrefixWalk<KP> pw;
  pw.template start<SH>(t, q, k, sv.tam, sv.hs, hc, hca);
  unsigned flag = 0u;
#pragma unroll 4
  for (int s = 0; s < K; ++s) {
    const uint32_t h = pw.hu() ^ tab_word<SH>(hc, hca, (uint32_t)pw.x[0]);
    const uint32_t m = bloom_bits(h, F);
    flag |= ((tab_word<SH>(lk.filt, fa, h & wmask) & m) == m && s < v) ? 1u : 0u;
    if (s + 1 < v) pw.template next<SH>(hc, hca);
  }
  if (flag) {
    pw.template start<SH>(t, q, k, sv.tam, sv.hs, hc, hca);
    for (int s = 0; s < v; ++s) {
      const uint32_t h = pw.hu() ^ tab_word<SH>(hc, hca, (uint32_t)pw.x[0]);
      const uint32_t m = bloom_bits(h, F);
      if ((tab_word<SH>(lk.filt, fa, h & wmask) & m) == m)
        probe_bucket<ML>(sv, lk, t, sw, h, pw.x, k, pw.top(), lb);
      if (s + 1 < v) pw.template next<SH>(hc, hca);
    }
  }
}

// One lookup tile: lane l takes the K colex-consecutive prefixes
// tile * 32K + l * K + [0, K) of the block's C(tam - 1, w - 1) prefixes (ascending
// (w-1)-subsets of [0, tam - 1), so each has at least one j above it).
// SH: the tables are in the warp's stage (explicit shared-memory loads).  Not
// inlined: the scan gets the whole register budget instead of sharing it with
// the scheduling state of the persistent kernel around it (sv and lk are the
// warp's copies in shared memory).
template <int K, bool ML, bool SH>
__device__ __noinline__ LaneBest eval_lookup_tile(const SegView &sv, const LookView &lk,
                                                  const unsigned long long *t, const uint32_t *sw,
                                                  unsigned long long tile) {
  LaneBest lb;
  lb.reset();
  const int lane = threadIdx.x & 31;
  const int k = sv.w - 1;
  const unsigned long long q = tile * (32ull * K) + (unsigned long long)lane * K;
  if (q >= sv.nprefix) return lb;
  const int v = (sv.nprefix - q) < (unsigned long long)K ? (int)(sv.nprefix - q) : K;
  if (k == 0) {  // weight 1: the empty prefix, every j
    const int x[5] = {0, 1, 2, 3, 4};
    const uint32_t m = bloom_bits(sv.hs, lk.F);
    const uint32_t fw = SH ? tab_word<SH>(lk.filt, smem_addr(lk.filt), sv.hs & lk.wmask)
                           : lk.filt[sv.hs & lk.wmask];
    if ((fw & m) == m) probe_bucket<ML>(sv, lk, t, sw, sv.hs, x, 0, -1, lb);
    return lb;
  }
  switch (k) {
    case 1: scan_lane<1, K, ML, SH>(sv, lk, t, sw, q, v, lb); break;
    case 2: scan_lane<2, K, ML, SH>(sv, lk, t, sw, q, v, lb); break;
    case 3: scan_lane<3, K, ML, SH>(sv, lk, t, sw, q, v, lb); break;
    case 4: scan_lane<4, K, ML, SH>(sv, lk, t, sw, q, v, lb); break;
    default: scan_lane<0, K, ML, SH>(sv, lk, t, sw, q, v, lb); break;
  }
  return lb;
}

// Lookup tiles of a weight block with nprefix prefixes.
GRAND_HD inline unsigned long long lookup_tiles(unsigned long long nprefix) {
  const unsigned long long per = 32ull * (unsigned long long)kLookK;
  return (nprefix + per - 1ull) / per;
}

}  // namespace grand
