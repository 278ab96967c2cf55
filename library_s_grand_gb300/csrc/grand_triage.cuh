// grand_triage.cuh -- the per-shot work of a decoding launch (sm_103a), run by
// the warps of the persistent decode kernel (grand_decode.cuh).
//
// classify_chunk (kChunkShots launch slots, one lane per shot)
//   packs the 32 shots' records with coalesced ballots, forms each syndrome and
//   settles the common shots outright: an empty syndrome (grand_decoder.cu:1223-1241),
//   and a first threshold iteration with one active position whose column equals
//   the syndrome (weight-1 match, 1 candidate tested).  The others go to the slow
//   queue.
//
// triage_shot (one warp per shot)
//   packs the shot's record into bits, forms the syndrome, computes the
//   flagged-check count of every column (popc(col & s), upstream
//   grand_decoder.cu:67-81 / 352-374, with the irregular offset of :406-416),
//   the active sets of the <= 3 threshold iterations (:1284-1290, :495-504),
//   the upstream active-set cap and mode rules (:1296, :1327, :1550-1554), and
//   the weight blocks each searched iteration enumerates.  The iterations are
//   searched in upstream order by the same warp while each fits the light
//   budget; the first larger one and those after it become a Job whose tiles
//   every warp of the launch searches (grand_search.cuh).
#pragma once

#include "grand_kernels.cuh"

namespace grand {


// ---------------------------------------------------------------------------
// Planning: the threshold iterations and their weight blocks (lane 0 only).
// The planner is resumable: each call walks upstream's iteration loop
// (grand_decoder.cu:1284-1343) to the next iteration that is searched, appends
// it and its weight blocks to the Job and returns 1, or records the outcome
// fields of an exhausted loop and returns 0.  Shots usually resolve in their
// first searched iteration, so later iterations are only planned when needed.
// ---------------------------------------------------------------------------

static __device__ int plan_next(const DevCode &cd, int tam0, int tam1, int tam2, int L, int tile_k, Job &J,
                         PlanState &P) {
  while (P.i < L) {
    const int i = P.i++;
    P.passes = i + 1;
    int tam = i == 0 ? tam0 : (i == 1 ? tam1 : tam2);
    if (cd.family == kDem) {  // grand_decoder.cu:1550-1554
      if (tam > cd.cap) tam = P.tam_old;
      else P.tam_old = tam;
    }
    P.tam = tam;
    if (tam <= 0) continue;
    const bool gpu = (tam > cd.thr && tam <= cd.cap && cd.mode == 1) || cd.mode == 0;
    const bool cpu = !gpu && ((tam <= cd.thr && cd.mode == 1) || cd.mode == -1);
    if (!gpu && !cpu) continue;
    if (tam > kMaxTam) {
      J.failed = 1;
      continue;
    }
    IterInfo &I = J.it[J.n_it];
    I.it = i + 1;
    I.tam = tam;
    I.branch = gpu ? kBranchGpu : kBranchCpu;
    I.src = i;
    I.seg_lo = J.nseg;
    I.base = P.gbase;
    I.phase_end[0] = I.phase_end[1] = I.phase_end[2] = 0;
    unsigned long long tot = 0;
    unsigned seen = 0;
    // one weight block of weight w in phase position k, appended in search order
    auto emit = [&](int w, int k) {
      Seg &S = J.seg[J.nseg++];
      S.iter = J.n_it;
      S.w = w;
      S.phase = k;
      S.dup = (seen >> w) & 1u;
      seen |= 1u << w;
      S.count = binom(tam, w);
      S.base = P.gbase + tot;
      S.nprefix = binom(tam - 1, w - 1);
      S.runs = w >= 3 ? 1 : 0;
      S.K = S.runs ? kRunKKLight : tile_k;
      // tile counts of the light search: run tiles are counted run by run as
      // they are walked; colex blocks (w <= 2) have at most tam - 1 prefixes, so
      // a 32-bit division suffices.  A Job's blocks are searched in lookup tiles.
      S.ntiles = S.runs ? 0ull
                        : (unsigned long long)(((unsigned)S.nprefix + 32u * (unsigned)S.K - 1u) /
                                               (32u * (unsigned)S.K));
      tot += S.count;
      if (cd.variant == kProb) I.phase_end[k] = tot;
    };
    if (cd.variant == kProb) {
      int mi = cd.n_masks - 1;  // grand_decoder.cu:754-762
      for (int q = 0; q < cd.n_masks; ++q)
        if (tam <= cd.mask_tam_upper[q]) { mi = q; break; }
      for (int k = 0; k < cd.num_phases; ++k) {  // grand_decoder.cu:764-786
        const int pid = cd.mask_order[mi][k];
        if (pid == 0) {
          for (int w = 1; w <= 5 && w <= tam && w <= kMaxW; ++w) emit(w, k);
        } else if (pid == 1) {
          if (6 <= tam && 6 <= kMaxW) emit(6, k);
        }
      }
    } else {
      const int wmax = cd.Wc < tam ? cd.Wc : tam;
      for (int w = 1; w <= wmax; ++w) emit(w, 0);
    }
    if (cd.variant == kProb)  // phases without weights keep the running total
      for (int k = 1; k < 3; ++k)
        if (I.phase_end[k] < I.phase_end[k - 1]) I.phase_end[k] = I.phase_end[k - 1];
    I.seg_hi = J.nseg;
    I.total = tot;
    P.gbase += tot;
    J.n_it++;
    return 1;
  }
  J.final_iteration = P.passes;
  J.final_tam = P.tam;
  return 0;
}

// ---------------------------------------------------------------------------
// Staging of one iteration's active set (positions, columns, sketches, LLRs).
// ---------------------------------------------------------------------------
// pos, tmp (unsorted ML list) and key (ML sort keys) are the warp's working
// arrays: shared memory wherever they fit, so that the gathers below read the
// positions without a round trip to L2.
template <bool MLK>
__device__ void stage_iteration(const DevCode &cd, const uint32_t *am, int tam, int *pos,
                                int *tmp, float *key, uint32_t *cols, uint32_t *hcols,
                                float *llr) {
  const int lane = threadIdx.x & 31;
  const bool ml = MLK && cd.variant == kMl;
  int *dst = ml ? tmp : pos;
  // ascending column indices of the first tam set bits (upstream extract_positions)
  int base = 0;
  for (int q = 0; q < cd.mw && base < tam; ++q) {
    const uint32_t word = am[q];
    const bool bit = (word >> lane) & 1u;
    const int idx = base + __popc(word & ((1u << lane) - 1u));
    if (bit && idx < tam) dst[idx] = q * 32 + lane;
    base += __popc(word);
  }
  __syncwarp();
  if (ml) {
    // stable sort by LLR ascending (upstream insertion sort, grand_decoder.cu:598-610):
    // the keys in list order first, then each element's rank among them
    for (int i = lane; i < tam; i += 32) key[i] = __ldg(cd.llr + tmp[i]);
    __syncwarp();
    for (int i = lane; i < tam; i += 32) {
      const float ki = key[i];
      int r = 0;
      for (int j = 0; j < tam; ++j) {
        const float kj = key[j];
        r += (kj < ki) || (kj == ki && j < i);
      }
      pos[r] = tmp[i];
    }
    __syncwarp();
  }
  const int nwp = cd.nwp;
  for (int idx = lane; idx < tam * nwp; idx += 32) {
    const int i = idx / nwp;
    cols[idx] = __ldg(cd.cols + (size_t)pos[i] * nwp + (idx - i * nwp));
  }
  for (int i = lane; i < tam; i += 32) hcols[i] = __ldg(cd.hcol + pos[i]);
  if (ml)
    for (int i = lane; i < tam; i += 32) llr[i] = __ldg(cd.llr + pos[i]);
  __syncwarp();
}

// Every tile of one weight block, in order, by one warp (light path).
template <bool ML>
__device__ void eval_segment(const DevCode &cd, const SegView &sv, const Seg &S,
                             const unsigned long long *t, const uint32_t *sw, LaneBest &lb) {
  if (S.runs) {
    const unsigned long long per = 32ull * kRunKKLight;
    for (int c = S.w - 2; c <= sv.tam - 2; ++c) {
      const unsigned long long nt = run_tiles(t, c, S.w, kRunKKLight);
      for (unsigned long long q = 0; q < nt; ++q)
        eval_run_tile<kRunKKLight, ML>(sv, t, sw, c, q * per, lb);
    }
  } else {
    for (unsigned long long tile = 0; tile < S.ntiles; ++tile) eval_tile<ML>(sv, t, sw, tile, lb);
  }
}

// ---------------------------------------------------------------------------
// Record input.
// ---------------------------------------------------------------------------
// dst[q] = ballot(p[32q + lane] != 0) for the n entries of p (written by lane 0);
// returns the number of nonzero entries.  Eight words' loads are issued before
// their ballots, so a record costs one memory round trip per 256 entries rather
// than one per 32.
__device__ __forceinline__ int pack_ballots(const int *p, int n, uint32_t *dst) {
  const int lane = threadIdx.x & 31;
  int total = 0;
  for (int q0 = 0; q0 * 32 < n; q0 += 8) {
    int v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int i = (q0 + u) * 32 + lane;
      v[u] = i < n ? __ldcg(p + i) : 0;  // read once: kept out of L1
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      if ((q0 + u) * 32 < n) {
        const uint32_t bits = __ballot_sync(kFull, v[u] != 0);
        if (lane == 0) dst[q0 + u] = bits;
        total += __popc(bits);
      }
    }
  }
  return total;
}

// ---------------------------------------------------------------------------
// Small active sets: every subset as a bit mask.
// ---------------------------------------------------------------------------
constexpr int kSmallTam = 14;  // iterations with tam <= 14 take this path

// Exact test of a mask whose sketch is zero: the syndrome XOR the mask's
// columns is zero in every word.
__device__ __forceinline__ bool mask_matches(const uint32_t *cols, int nwp, int nw,
                                             const uint32_t *sw, unsigned mask) {
  for (int i = 0; i < nw; ++i) {
    uint32_t z = sw[i];
    for (unsigned mm = mask; mm; mm &= mm - 1u) z ^= cols[(__ffs(mm) - 1) * nwp + i];
    if (z != 0u) return false;
  }
  return true;
}

// All 2^tam subsets of a small active set in one pass.  Lane l walks the masks
// gray(g) = g ^ (g >> 1) for g in its own contiguous block, so each step flips
// one column: one shared-memory sketch load and one XOR, with no unranking and
// no per-weight tiles.  A mask of weight w that the iteration searches (bit w of
// wmask), whose sketch is zero and whose columns XOR to the syndrome word by
// word, is a match.
//   first-hit: its global index is the base of its weight block plus its
//     lexicographic rank; blocks are laid out in search order, so the lowest
//     index over the warp (best) is the candidate the block-by-block search
//     finds first;
//   ML: its cost is its LLRs summed in ascending position order (the order the
//     block-by-block search adds them), and each weight keeps the lowest
//     {cost key, lexicographic rank}; O[w], R[w] return the warp's minima
//     (0xffffffff / kNone: no match of weight w).
template <bool ML>
__device__ void small_iteration(const uint32_t *cols, const uint32_t *hcols, const float *llr,
                                const uint32_t *sw, uint32_t hs, int nwp, int nw, int tam,
                                const unsigned long long (&wbase)[kMaxW + 1], unsigned wmask,
                                const unsigned long long *t, unsigned long long &best,
                                unsigned &bmask, uint32_t (&O)[kMaxW + 1],
                                unsigned long long (&R)[kMaxW + 1]) {
  const int lane = threadIdx.x & 31;
  const int nm = 1 << tam;
  const int per = (nm + 31) >> 5;
  const int g0 = lane * per;
  const int g1 = g0 + per < nm ? g0 + per : nm;
  best = kNone;
  unsigned lmask = 0u;
#pragma unroll
  for (int q = 0; q <= kMaxW; ++q) {
    O[q] = 0xffffffffu;
    R[q] = kNone;
  }
  if (g0 < g1) {
    unsigned mask = (unsigned)(g0 ^ (g0 >> 1));
    uint32_t h = hs;  // sketch of the syndrome XOR the mask's columns
    for (unsigned mm = mask; mm; mm &= mm - 1u) h ^= hcols[__ffs(mm) - 1];
    for (int g = g0;;) {
      if (h == 0u) {
        const int w = __popc(mask);
        if (((wmask >> w) & 1u) && mask_matches(cols, nwp, nw, sw, mask)) {
          int x[5] = {0, 0, 0, 0, 0};
          int j = 0;
          float pc = 0.0f;
          unsigned mm = mask;
#pragma unroll
          for (int e = 0; e < 6; ++e) {  // set bits in ascending order; the last is j
            if (mm) {
              const int bit = __ffs(mm) - 1;
              mm &= mm - 1u;
              if constexpr (ML) pc = __fadd_rn(pc, llr[bit]);
              if (mm) {
                if (e < 5) x[e < 5 ? e : 4] = bit;
              } else {
                j = bit;
              }
            }
          }
          const unsigned long long r = lex_rank(t, tam, w, x, w - 1, j);
          if constexpr (!ML) {
            unsigned long long wbw = 0;
#pragma unroll
            for (int q = 1; q <= kMaxW; ++q)
              if (q == w) wbw = wbase[q];
            const unsigned long long g_idx = wbw + r;
            if (g_idx < best) {
              best = g_idx;
              lmask = mask;
            }
          } else {
            const uint32_t o = cost_key(pc);
#pragma unroll
            for (int q = 1; q <= kMaxW; ++q)
              if (q == w && (o < O[q] || (o == O[q] && r < R[q]))) {
                O[q] = o;
                R[q] = r;
              }
          }
        }
      }
      if (++g >= g1) break;
      const int bit = __ffs(g) - 1;  // gray(g) ^ gray(g - 1) = 1 << ctz(g)
      mask ^= 1u << bit;
      h ^= hcols[bit];
    }
  }
  if constexpr (!ML) {
    // the lane holding the lowest index hands its mask over (each mask is
    // visited by exactly one lane, so the index identifies one lane)
    const unsigned long long lbest = best;
    best = warp_min_u64(best);
    const unsigned who = __ballot_sync(kFull, best != kNone && lbest == best);
    bmask = __shfl_sync(kFull, lmask, who ? __ffs(who) - 1 : 0);
    if (!who) bmask = 0u;
  } else {
#pragma unroll
    for (int q = 1; q <= kMaxW; ++q) warp_min_key(O[q], R[q]);
  }
}

// ---------------------------------------------------------------------------
// Kernel 1: triage + light search.
// ---------------------------------------------------------------------------
// First-hit search of an iteration with one active position (most shots at low
// error rates): its only candidate is that column, weight 1, rank 0 of the
// first weight-1 block, and it matches when the column equals the syndrome.
// The same winner as the small-set path, without staging the iteration.
static __device__ void single_search(const DevCode &cd, Job &J, WarpArea &A, int ii, Winner &wn) {
  const int lane = threadIdx.x & 31;
  IterInfo &I = J.it[ii];
  int s = I.seg_lo;
  while (s < I.seg_hi && (J.seg[s].w != 1 || J.seg[s].dup)) ++s;
  if (s >= I.seg_hi) return;  // no weight-1 block: nothing to search
  // the active position: the lowest set bit of the iteration's threshold mask
  const uint32_t *am = A.am[I.src];
  int pos = -1;
  for (int q0 = 0; q0 < cd.mw && pos < 0; q0 += 32) {
    const uint32_t word = q0 + lane < cd.mw ? am[q0 + lane] : 0u;
    const unsigned nz = __ballot_sync(kFull, word != 0u);
    if (nz) {
      const int l = __ffs(nz) - 1;
      pos = (q0 + l) * 32 + __ffs(__shfl_sync(kFull, word, l)) - 1;
    }
  }
  if (pos < 0) return;
  const bool eq = lane >= cd.nw || __ldg(cd.cols + (size_t)pos * cd.nwp + lane) == A.sw[lane];
  if (!__all_sync(kFull, eq)) return;
  const Seg &S = J.seg[s];
  wn.found = 1;
  wn.ii = ii;
  wn.seg = s;
  wn.rank = 0;
  wn.count = I.branch == kBranchCpu ? S.base - I.base + 1ull             // grand_decoder.cu:547-548
             : cd.variant == kProb  ? I.phase_end[S.phase]              // grand_decoder.cu:1006
                                    : I.total;                          // grand_decoder.cu:1303-1304
  wn.cost = 0.0f;
  wn.mask = 1u;  // position 0 of the iteration's list
  if (lane == 0) {
    A.pos[0] = pos;
    I.pos = A.pos;
  }
  __syncwarp();
}

template <bool MLK>
__device__ void light_search(const DevBatch &b, const DevCode &cd, Job &J, WarpArea &A, int ii,
                             Winner &wn) {
  const int lane = threadIdx.x & 31;
  const bool ml = MLK && cd.variant == kMl;
  IterInfo &I = J.it[ii];
  stage_iteration<MLK>(cd, A.am[I.src], I.tam, A.pos, A.tmp, reinterpret_cast<float *>(A.hcols),
                       A.cols, A.hcols, A.llr);
  if (lane == 0) {
    I.pos = A.pos;
    I.cols = A.cols;
    I.hcols = A.hcols;
    I.llr = A.llr;
    if (ml) {
      float pf = 0.0f;
      I.prefix[0] = 0.0f;
      for (int w = 1; w <= kMaxW; ++w) {
        if (w <= I.tam) pf = __fadd_rn(pf, A.llr[w - 1]);
        I.prefix[w] = pf;
      }
    }
  }
  __syncwarp();
  // every subset at once only while that is not much more than the iteration's
  // candidates (weights above W would be most of the 2^tam masks)
  const bool small = I.tam <= kSmallTam && (1ull << I.tam) <= 4ull * I.total;
  uint32_t SO[kMaxW + 1];
  unsigned long long SR[kMaxW + 1];
  if (!ml) {
    if (small) {
      // weight -> base of the block that searches it first (a later listing of
      // the same weight never matches first)
      unsigned long long wb[kMaxW + 1] = {0, 0, 0, 0, 0, 0, 0};
      unsigned wm = 0;
      for (int s = I.seg_lo; s < I.seg_hi; ++s) {
        const Seg &S = J.seg[s];
        if (S.dup) continue;
#pragma unroll
        for (int q = 1; q <= kMaxW; ++q)  // constant indices keep wb in registers
          if (q == S.w) wb[q] = S.base;
        wm |= 1u << S.w;
      }
      unsigned long long g;
      unsigned gm;
      small_iteration<false>(A.cols, A.hcols, A.llr, A.sw, J.hs, cd.nwp, cd.nw, I.tam, wb, wm,
                             b.ncr, g, gm, SO, SR);
      if (g != kNone) {
        wn = winner_from_index(J, g, cd.variant == kProb);
        wn.mask = gm;
      }
      return;
    }
    for (int s = I.seg_lo; s < I.seg_hi && !wn.found; ++s) {
      const Seg &S = J.seg[s];
      if (S.dup) continue;
      SegView sv{A.hcols, A.cols, A.llr, J.hs, I.tam, S.w, S.K, cd.nwp, cd.nw, S.nprefix, S.base};
      LaneBest lb;
      lb.reset();
      eval_segment<false>(cd, sv, S, b.ncr, A.sw, lb);
      if (__any_sync(kFull, lb.g != kNone))
        wn = winner_from_index(J, warp_min_u64(lb.g), cd.variant == kProb);
    }
    return;
  }
  // upstream search_cpu_ml (grand_decoder.cu:620-656), one weight at a time
  if (small) {
    unsigned wm = 0;
    for (int s = I.seg_lo; s < I.seg_hi; ++s) wm |= 1u << J.seg[s].w;
    const unsigned long long none[kMaxW + 1] = {0, 0, 0, 0, 0, 0, 0};
    unsigned long long g;
    unsigned gm;
    small_iteration<true>(A.cols, A.hcols, A.llr, A.sw, J.hs, cd.nwp, cd.nw, I.tam, none, wm,
                          b.ncr, g, gm, SO, SR);
  }
  uint32_t bo = 0xffffffffu;
  unsigned long long br = kNone, proc = 0;
  int bseg = -1;
  for (int s = I.seg_lo; s < I.seg_hi; ++s) {
    const Seg &S = J.seg[s];
    if (bseg >= 0 && I.prefix[S.w] >= key_cost(bo)) break;
    proc += S.count;
    uint32_t o;
    unsigned long long r;
    if (small) {
      o = 0xffffffffu;
      r = kNone;
#pragma unroll
      for (int q = 1; q <= kMaxW; ++q)
        if (q == S.w) {
          o = SO[q];
          r = SR[q];
        }
    } else {
      SegView sv{A.hcols, A.cols, A.llr, J.hs, I.tam, S.w, S.K, cd.nwp, cd.nw, S.nprefix, S.base};
      LaneBest lb;
      lb.reset();
      eval_segment<true>(cd, sv, S, b.ncr, A.sw, lb);
      o = lb.o;
      r = lb.r;
      warp_min_key(o, r);
    }
    if (o != 0xffffffffu && (bseg < 0 || o < bo)) {
      bo = o;
      br = r;
      bseg = s;
    }
  }
  if (bseg >= 0) {
    wn.found = 1;
    wn.ii = ii;
    wn.seg = bseg;
    wn.rank = br;
    wn.count = (I.branch == kBranchCpu) ? proc : I.total;
    wn.cost = key_cost(bo);
  }
}

// The full per-shot path: one warp, launch slot `slot`.  P is the warp's planner
// state; tag (the launch epoch + 1) marks a published Job.
template <bool MLK>
__device__ void triage_shot(const DevBatch &b, int slot, WarpArea &A, PlanState &P, unsigned tag,
                            bool cached) {
  const int lane = threadIdx.x & 31;
  {
    const unsigned long long t_start = global_ns();
    unsigned long long tp = b.profile ? t_start : 0ull;
    const int shot = b.shot_map ? b.shot_map[slot] : slot;
    const int ci = b.shot_code ? b.shot_code[shot] : 0;
    const DevCode &cd = b.codes[ci];
    // a record the chunk step already read is taken from its packed copy in
    // rec_cache (device memory, in place of a second read of the caller's record)
    const int *rec = cached ? reinterpret_cast<const int *>(b.rec_cache + (size_t)slot * kRecCacheWords)
                            : b.in + (b.in_off ? b.in_off[shot] : (long long)shot * cd.rec_len);
    Job &J = A.job;

    // ---- pack the record ---------------------------------------------------
    uint32_t s_lane = 0;  // lane w holds syndrome word w
    int original_weight = 0;
    if (cd.packed || cached) {
      // bit-packed records: the words are the bits (bits past the last entry ignored)
      const int nwords = cd.input_kind == kInErrors ? cd.mw : cd.nw;
      const int nbits = cd.input_kind == kInErrors ? cd.m : cd.R;
      uint32_t *dst = cd.input_kind == kInErrors ? A.eb : A.sw;
      for (int q = lane; q < nwords; q += 32) {
        uint32_t v = __ldcg(reinterpret_cast<const uint32_t *>(rec) + q);
        if (q == nwords - 1 && (nbits & 31)) v &= (1u << (nbits & 31)) - 1u;
        dst[q] = v;
        original_weight += __popc(v);
      }
      if (cd.family == kDem) {
        const uint32_t *lg = (b.in_log && !cached)
                                 ? reinterpret_cast<const uint32_t *>(b.in_log) + (size_t)shot * cd.nlw
                                 : reinterpret_cast<const uint32_t *>(rec) + cd.nw;
        for (int q = lane; q < cd.nlw; q += 32) {
          uint32_t v = __ldcg(lg + q);
          if (q == cd.nlw - 1 && (cd.n_logicos & 31)) v &= (1u << (cd.n_logicos & 31)) - 1u;
          A.eb[q] = v;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) original_weight += __shfl_xor_sync(kFull, original_weight, o);
      if (cd.input_kind != kInErrors) original_weight = 0;
      __syncwarp();
      if (cd.input_kind == kInErrors) {
        for (int q = 0; q < cd.mw && original_weight != 0; ++q) {
          uint32_t word = A.eb[q];
          while (word) {
            const int c = q * 32 + __ffs(word) - 1;
            word &= word - 1u;
            if (lane < cd.nw) s_lane ^= __ldg(cd.cols + (size_t)c * cd.nwp + lane);
          }
        }
      } else {
        s_lane = lane < cd.nw ? A.sw[lane] : 0u;
      }
    } else if (cd.input_kind == kInErrors) {
      original_weight = pack_ballots(rec, cd.m, A.eb);
      __syncwarp();
      // s = XOR of the columns of the supplied error (grand_decoder.cu:476-486);
      // an error-free record (most shots at low error rates) skips the walk
      for (int q = 0; q < cd.mw && original_weight != 0; ++q) {
        uint32_t word = A.eb[q];
        while (word) {
          const int c = q * 32 + __ffs(word) - 1;
          word &= word - 1u;
          if (lane < cd.nw) s_lane ^= __ldg(cd.cols + (size_t)c * cd.nwp + lane);
        }
      }
    } else {
      pack_ballots(rec, cd.R, A.sw);
      if (cd.family == kDem)
        pack_ballots(b.in_log ? b.in_log + (size_t)shot * cd.n_logicos : rec + cd.R, cd.n_logicos,
                     A.eb);
      __syncwarp();
      s_lane = lane < cd.nw ? A.sw[lane] : 0u;
    }
    A.sw[lane] = (lane < cd.nw) ? s_lane : 0u;
    const bool empty = !__any_sync(kFull, s_lane != 0u);  // lanes >= nw hold 0
    __syncwarp();
    tp = prof_lap(b, kProfShotPack, tp);

    if (empty) {  // grand_decoder.cu:1223-1241: nothing to search
      // the 72-byte result as 18 words, one per lane: original_weight (word 2)
      // and hibrido = -2 (word 8), everything else 0
      if (lane < 18)
        reinterpret_cast<uint32_t *>(b.results + shot)[lane] =
            lane == 2 ? (uint32_t)original_weight : (lane == 8 ? (uint32_t)-2 : 0u);
      if (lane == 0 && b.ml_cost) b.ml_cost[shot] = 0.0f;
      if (b.dec_err)
        for (int c = lane; c < cd.m; c += 32) b.dec_err[(size_t)shot * cd.m + c] = 0;
      if (b.dec_log && cd.family == kDem)
        for (int j = lane; j < cd.n_logicos; j += 32) b.dec_log[(size_t)shot * cd.n_logicos + j] = 0;
      if (b.deferred && lane == 0) b.deferred[shot] = 0;
      __syncwarp();
      return;
    }

    // Sketch of the syndrome (XOR of the row hashes of its set rows), read by
    // the sketch scans only: a one-position iteration compares its column with
    // the syndrome itself, so most shots never form it.
    bool have_hs = false;
    auto syndrome_sketch = [&]() {
      if (have_hs) return;
      uint32_t hs = 0u;
      for (uint32_t word = s_lane; word; word &= word - 1u)
        hs ^= row_hash(lane * 32 + __ffs(word) - 1);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) hs ^= __shfl_xor_sync(kFull, hs, o);
      if (lane == 0) J.hs = hs;
      __syncwarp();
      have_hs = true;
    };

    // ---- flagged-check counts and threshold masks ---------------------------
    const int L = cd.max_soma < kMaxIters ? cd.max_soma : kMaxIters;
    // Four mask words (128 columns) per pass, with every column load of the
    // pass issued before the first use: one memory round trip per 128 columns.
    int tam_raw[3] = {0, 0, 0};
    for (int q0 = 0; q0 < cd.mw; q0 += 4) {
      int sum[4] = {0, 0, 0, 0};
      if (cd.nwp == 4) {  // R <= 128: a column is one 16-byte word group
        uint4 v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int c = (q0 + u) * 32 + lane;
          v[u] = c < cd.m ? __ldg(reinterpret_cast<const uint4 *>(cd.cols) + c)
                          : make_uint4(0u, 0u, 0u, 0u);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)  // words past nw meet zero syndrome words
          sum[u] = __popc(v[u].x & A.sw[0]) + __popc(v[u].y & A.sw[1]) +
                   __popc(v[u].z & A.sw[2]) + __popc(v[u].w & A.sw[3]);
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int c = (q0 + u) * 32 + lane;
          if (c < cd.m) {
            const uint32_t *col = cd.cols + (size_t)c * cd.nwp;
            for (int k = 0; k < cd.nw; ++k) sum[u] += __popc(__ldg(col + k) & A.sw[k]);
          }
        }
      }
      if (!cd.regular) {
        int cw[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int c = (q0 + u) * 32 + lane;
          cw[u] = c < cd.m ? __ldg(cd.colw + c) : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) sum[u] = cw[u] == 0 ? 0 : sum[u] + (cd.max_soma - cw[u]);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = q0 + u;
        if (q >= cd.mw) break;
        const int c = q * 32 + lane;
#pragma unroll
        for (int i = 0; i < kMaxIters; ++i) {
          const uint32_t bits =
              __ballot_sync(kFull, c < cd.m && i < L && sum[u] >= cd.max_soma - i);
          if (lane == 0) A.am[i][q] = bits;
          tam_raw[i] += __popc(bits);
        }
      }
    }
    if (lane == 0) {
      J.n_it = 0;
      J.nseg = 0;
      J.failed = 0;
      J.final_iteration = 0;
      J.final_tam = 0;
      P.i = 0;
      P.tam = 0;
      P.tam_old = 0;
      P.passes = 0;
      P.gbase = 0;
      J.shot = shot;
      J.code = ci;
      J.original_weight = original_weight;
      J.best = kNone;
      J.tiles_done = 0;
      J.t_start = t_start;
      J.t_counts = global_ns();
    }
    tp = prof_lap(b, kProfShotCounts, tp);

    // ---- iterations in upstream order; the first one over the light budget
    //      and everything after it become a Job that every warp searches -------
    const bool ml = MLK && cd.variant == kMl;
    const unsigned long long budget = 1ull << b.light_max_log2;
    Winner wn;
    wn.found = 0;
    wn.ii = wn.seg = 0;
    wn.rank = wn.count = 0;
    wn.cost = 0.0f;
    wn.mask = 0u;
    int heavy_from = -1;
    for (;;) {
      int more = 0;
      __syncwarp();  // every lane is done reading the Job before lane 0 extends it
      if (lane == 0) more = plan_next(cd, tam_raw[0], tam_raw[1], tam_raw[2], L, b.tile_k, J, P);
      more = __shfl_sync(kFull, more, 0);
      __syncwarp();
      if (!more) break;
      const int ii = J.n_it - 1;
      const IterInfo &I = J.it[ii];
      if (I.total > budget || I.tam > kLightTam || I.tam * cd.nwp > kLightWords) {
        heavy_from = ii;
        __syncwarp();  // every lane has read n_it before lane 0 plans the rest
        if (lane == 0)
          while (plan_next(cd, tam_raw[0], tam_raw[1], tam_raw[2], L, b.tile_k, J, P)) {
          }
        __syncwarp();
        break;
      }
      if (!ml && I.tam == 1) single_search(cd, J, A, ii, wn);
      else {
        syndrome_sketch();
        light_search<MLK>(b, cd, J, A, ii, wn);
      }
      if (wn.found) break;
    }
    tp = prof_lap(b, kProfShotLight, tp);
    if (heavy_from < 0) {
      finish_shot(b, cd, J, shot, wn, A.eb, A.delta);
      if (b.deferred && lane == 0) b.deferred[shot] = 0;
      __syncwarp();
      prof_lap(b, kProfShotFinish, tp);
      return;
    }

    // ---- heavy: publish a Job ------------------------------------------------
    unsigned long long tq = tp;
    syndrome_sketch();
    unsigned long long words = 0;
    for (int ii = heavy_from; ii < J.n_it; ++ii) {
      const unsigned long long tm = (unsigned long long)J.it[ii].tam;
      words += (tm * cd.nwp + 3ull) & ~3ull;                            // columns
      words += (unsigned long long)look_layout((int)tm, kWarpStage).words;  // lookup block
      words += ((ml ? 2ull : 1ull) * tm + 3ull) & ~3ull;  // positions (+ sort buffer)
      if (ml) words += (tm + 3ull) & ~3ull;               // LLRs
    }
    words += 128;  // supplied bits
    // whole 128-byte lines, so no line is shared with another Job's data
    words = (words + 31ull) & ~31ull;
    unsigned long long off = 0, jslot = 0, tbase = 0, ntl = 0;
    int ok = 1;
    if (lane == 0) {
      // One atomicAdd, after a check that the reservation fits what is left: a
      // shot larger than that touches nothing, so it does not make the shots
      // after it fail too, and the first reservation of a launch that fits the
      // arena always succeeds.  Reservations racing for the last words may all
      // overshoot; those shots are re-run like any other that did not fit.
      ok = 0;
      off = *reinterpret_cast<volatile unsigned long long *>(ctr_ptr(b.counters, kCtrScratchTop));
      if (off + words <= b.scratch_words) {
        off = atomicAdd(ctr_ptr(b.counters, kCtrScratchTop), words);
        ok = off + words <= b.scratch_words ? 1 : 0;
      }
      if (!ok) atomicOr(b.status, kStatusScratchOverflow);
    }
    ok = __shfl_sync(kFull, ok, 0);
    if (!ok) {
      if (lane == 0 && b.deferred) b.deferred[shot] = 1;
      __syncwarp();
      return;
    }
    off = __shfl_sync(kFull, off, 0);
    tq = prof_lap(b, kProfPubReserve, tq, kCtrProfMore);
    uint32_t *sp = b.scratch + off;
    for (int ii = heavy_from; ii < J.n_it; ++ii) {
      IterInfo &I = J.it[ii];
      const unsigned long long tm = (unsigned long long)I.tam;
      uint32_t *cols = sp;
      sp += (tm * cd.nwp + 3ull) & ~3ull;
      const LookLayout LL = look_layout((int)tm, kWarpStage);
      uint32_t *hcols = sp;  // the lookup block starts with the column sketches
      sp += (unsigned long long)LL.words;
      int *pos = reinterpret_cast<int *>(sp);
      int *tmp = pos + tm;
      sp += ((ml ? 2ull : 1ull) * tm + 3ull) & ~3ull;
      float *llr = nullptr;
      if (ml) {
        llr = reinterpret_cast<float *>(sp);
        sp += (tm + 3ull) & ~3ull;
      }
      // positions (and the ML sort) in the light search's arrays, which are
      // free now, when they fit; then copied to the scratch
      const bool sh = (ml ? 3 : 1) * I.tam <= kPublishWords;
      int *wpos = sh ? reinterpret_cast<int *>(A.cols) : pos;
      int *wtmp = sh ? wpos + I.tam : tmp;
      float *wkey = sh ? reinterpret_cast<float *>(wpos + 2 * I.tam) : reinterpret_cast<float *>(hcols);
      stage_iteration<MLK>(cd, A.am[I.src], I.tam, wpos, wtmp, wkey, cols, hcols, llr);
      if (sh) {
        for (int i = lane; i < I.tam; i += 32) pos[i] = wpos[i];
        __syncwarp();
      }
      // an active set too large for a search warp's stage: its tables are
      // built here, once, in the scratch
      if (LL.words > kWarpStage) build_lookup(hcols, I.tam, LL);
      if (lane == 0) {
        I.pos = pos;
        I.cols = cols;
        I.hcols = hcols;
        I.llr = llr;
        if (ml) {
          float pf = 0.0f;
          I.prefix[0] = 0.0f;
          for (int w = 1; w <= kMaxW; ++w) {
            if (w <= I.tam) pf = __fadd_rn(pf, llr[w - 1]);
            I.prefix[w] = pf;
          }
        }
      }
      __syncwarp();
    }
    tq = prof_lap(b, kProfPubStage, tq, kCtrProfMore);
    if (lane == 0) {
      J.it_lo = heavy_from;
      for (int sgi = 0; sgi < J.nseg; ++sgi) {
        Seg &S = J.seg[sgi];
        S.njt = (S.dup || S.iter < heavy_from) ? 0ull : lookup_tiles(S.nprefix);
        S.tile_lo = ntl;
        ntl += S.njt;
      }
      // A Job slot and the next ntl tiles (the job table permitting), by one
      // atomicAdd as for the scratch above.
      ok = 0;
      unsigned long long old = ld_ctr(b, kCtrJobs);
      if ((old >> 40) < (unsigned long long)b.max_jobs) {
        old = atomicAdd(ctr_ptr(b.counters, kCtrJobs), (1ull << 40) + ntl);
        ok = (old >> 40) < (unsigned long long)b.max_jobs ? 1 : 0;
      }
      if (!ok) atomicOr(b.status, kStatusJobOverflow);
      jslot = old >> 40;
      tbase = old & ((1ull << 40) - 1ull);
    }
    ok = __shfl_sync(kFull, ok, 0);
    if (!ok) {
      if (lane == 0 && b.deferred) b.deferred[shot] = 1;
      __syncwarp();
      return;
    }
    jslot = __shfl_sync(kFull, jslot, 0);
    tbase = __shfl_sync(kFull, tbase, 0);
    ntl = __shfl_sync(kFull, ntl, 0);
    for (int q = lane; q < 128; q += 32) sp[q] = A.eb[q];
    J.sw[lane] = A.sw[lane];
    if (lane == 0) {
      J.ebits = sp;
      J.tile_base = tbase;
      J.ntiles = ntl;
      J.ready = 0;
      for (int i = 0; i < kMaxIters; ++i)
        for (int w = 0; w <= kMaxW; ++w) J.mlkey[i][w][0] = J.mlkey[i][w][1] = kNone;
    }
    __syncwarp();
    {
      const uint32_t *src = reinterpret_cast<const uint32_t *>(&J);
      uint32_t *dst = reinterpret_cast<uint32_t *>(b.jobs + jslot);
      for (int i = lane; i < (int)(sizeof(Job) / 4); i += 32) dst[i] = src[i];
    }
    if (lane == 0 && b.deferred) b.deferred[shot] = 0;
    tq = prof_lap(b, kProfPubWrite, tq, kCtrProfMore);
    // The Job is searchable once its ready word holds this launch's tag: each
    // lane orders its part of the copy (and the staged scratch) before it.
    __threadfence();
    __syncwarp();
    if (lane == 0) {
      __threadfence();
      *reinterpret_cast<volatile unsigned *>(&b.jobs[jslot].ready) = tag;
      __threadfence();
    }
    __syncwarp();
    advance_front(b, tag);
    prof_lap(b, kProfPubReady, tq, kCtrProfMore);
    prof_lap(b, kProfShotPublish, tp);
  }
}

// ---------------------------------------------------------------------------
// Classification of 32 launch slots, one lane per shot.
// ---------------------------------------------------------------------------
constexpr int kFastWords = 4;       // syndrome / logical words a lane keeps (R, n_logicos <= 128)
constexpr int kFastErrWords = 16;   // error-record words a lane walks (m <= 512)
constexpr int kFastBallots = 512;   // ballot words of a chunk's records (16384 int32 entries)
constexpr int kFastLogBallots = 128;  // ballot words of a chunk's separate logical entries

// classify_chunk's part of the WarpArea.
struct FastArea {
  uint32_t bits[kFastBallots + 1];      // bit e: entry e of the chunk's records (flat)
  uint32_t lbits[kFastLogBallots + 1];  // the same for DEM logicals kept in their own array
  uint32_t res[32][18];                 // result words, one row per lane
};
static_assert(sizeof(FastArea) <= sizeof(WarpArea), "FastArea must fit the warp's area");

// Bits b0..b7 of x moved to bits 0, 4, .., 28.
__device__ __forceinline__ uint32_t spread4(uint32_t x) {
  x &= 0xffu;
  x = (x | (x << 12)) & 0x000F000Fu;
  x = (x | (x << 6)) & 0x03030303u;
  x = (x | (x << 3)) & 0x11111111u;
  return x;
}

// bits[k] = the nonzero flags of p[32k .. 32k + 31] for the n entries at p (bits
// past n are 0); bits[ceil(n/32)] = 0.  The entries are read once and kept out
// of L1 (the per-shot path may read them again from L2).  With p 16-byte
// aligned, lanes read four entries at a time, eight 16-byte loads each in
// flight (records read in place from host memory need the bytes in flight): a
// row of 32 lanes is 128 entries, and its four words are four ballots (ballot
// c holds entry 4l + c in bit l) interleaved by four lanes.  Otherwise, and for
// the last n % 128 entries, one entry per lane per ballot.
__device__ __forceinline__ void flat_ballots(const int *p, int n, uint32_t *bits) {
  const int lane = threadIdx.x & 31;
  const int nwords = (n + 31) >> 5;
  int done = 0;  // entries handled by the 16-byte path (a multiple of 128)
  if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0u) {
    const int4 *p4 = reinterpret_cast<const int4 *>(p);
    const int rows = n >> 7;  // full rows of 128 entries
    for (int r0 = 0; r0 < rows; r0 += 8) {
      int4 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        v[u] = r0 + u < rows ? __ldcg(p4 + (r0 + u) * 32 + lane) : make_int4(0, 0, 0, 0);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (r0 + u < rows) {
          const uint32_t b0 = __ballot_sync(kFull, v[u].x != 0);
          const uint32_t b1 = __ballot_sync(kFull, v[u].y != 0);
          const uint32_t b2 = __ballot_sync(kFull, v[u].z != 0);
          const uint32_t b3 = __ballot_sync(kFull, v[u].w != 0);
          if (lane < 4) {
            const int sh = 8 * lane;
            bits[(r0 + u) * 4 + lane] = spread4(b0 >> sh) | (spread4(b1 >> sh) << 1) |
                                        (spread4(b2 >> sh) << 2) | (spread4(b3 >> sh) << 3);
          }
        }
      }
    }
    done = rows << 7;
  }
  for (int k0 = done >> 5; k0 < nwords; k0 += 16) {
    int v[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int e = (k0 + u) * 32 + lane;
      v[u] = e < n ? __ldcg(p + e) : 0;
    }
    uint32_t mine = 0u;
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const uint32_t w = __ballot_sync(kFull, v[u] != 0);
      mine = lane == u ? w : mine;
    }
    if (lane < 16 && k0 + lane < nwords) bits[k0 + lane] = mine;
  }
  if (lane == 0) bits[nwords] = 0u;
}

// Word q of the nbits-entry bit vector that starts at entry `off` of a flat
// ballot array (entries past nbits masked off).
__device__ __forceinline__ uint32_t flat_word(const uint32_t *bits, int off, int q, int nbits) {
  const int e = off + 32 * q;
  uint32_t w = __funnelshift_r(bits[e >> 5], bits[(e >> 5) + 1], e & 31);
  const int rem = nbits - 32 * q;
  if (rem < 32) w &= (1u << rem) - 1u;
  return w;
}

// Upstream's planner (grand_decoder.cu:1284-1296, 1550-1554, 754-786) for a first
// threshold iteration with one active position: is it searched, and with a
// weight-1 block (its only candidate)?  *gpu: the branch upstream takes.
__device__ __forceinline__ bool one_position_searched(const DevCode &cd, bool *gpu) {
  if (cd.family == kDem && 1 > cd.cap) return false;  // the cap replaces the set by an empty one
  const bool g = (1 > cd.thr && 1 <= cd.cap && cd.mode == 1) || cd.mode == 0;
  const bool c = !g && ((1 <= cd.thr && cd.mode == 1) || cd.mode == -1);
  if (!g && !c) return false;
  *gpu = g;
  if (cd.variant != kProb) return true;  // weights 1..min(W, 1)
  int mi = cd.n_masks - 1;
  for (int q = 0; q < cd.n_masks; ++q)
    if (1 <= cd.mask_tam_upper[q]) {
      mi = q;
      break;
    }
  for (int k = 0; k < cd.num_phases; ++k)
    if (cd.mask_order[mi][k] == 0) return true;  // phase 0 lists weight 1
  return false;
}

// Settles the shots of launch slots kChunkShots*chunk + [0, kChunkShots) that need no search
// -- an empty syndrome, or a first iteration with one active position whose
// column equals the syndrome -- and appends the others to the slow queue.  The
// results are exactly those of triage_shot: the one position is the only
// candidate of the iteration (found at weight 1, rank 0; one candidate counted
// on either branch, hibrido 0 / -1), and its active set is the set of nonzero
// columns contained in the syndrome (flagged-check count = column weight, for
// 0/1 matrices regular or not), found through the columns grouped by their
// lowest row.  Shots the lanes cannot settle here (ML codes, supplied errors
// that differ from the match, wide codes, records that are not back to back)
// take the slow path: they are appended to the slow queue with tag (the launch
// epoch + 1).
template <bool MLK>
__device__ void classify_chunk(const DevBatch &b, int chunk, WarpArea &A, unsigned tag) {
  FastArea &F = *reinterpret_cast<FastArea *>(&A);
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int slot = chunk * kChunkShots + lane;
  const bool valid = lane < kChunkShots && slot < b.num_shots;
  const unsigned long long t_start = global_ns();
  unsigned long long tp = b.profile ? t_start : 0ull;
  const int shot = valid ? (b.shot_map ? b.shot_map[slot] : slot) : 0;
  const int ci = (valid && b.shot_code) ? b.shot_code[shot] : 0;
  const DevCode &cd = b.codes[ci];
  const bool errs = cd.input_kind == kInErrors;
  const bool dem = cd.family == kDem;
  const int nbits = errs ? cd.m : cd.R;       // entries of the record's leading bit vector
  const int nwords = (nbits + 31) >> 5;
  bool ok = valid && cd.nw <= kFastWords && (!errs || nwords <= kFastErrWords) &&
            (!dem || cd.nlw <= kFastWords);
  const long long rbase = valid ? (b.in_off ? b.in_off[shot] : (long long)shot * cd.rec_len) : 0;

  uint32_t s[kFastWords] = {0u, 0u, 0u, 0u};
  uint32_t lg[kFastWords] = {0u, 0u, 0u, 0u};
  int ow = 0, epos = -1;

  // ---- the records: int32 entries through coalesced ballots over runs of
  //      back-to-back records, bit-packed words read directly ------------------
  const bool packed = cd.packed != 0;
  bool extracted = false;  // this lane's record bits are in rec_cache
  const bool any_int = __any_sync(kFull, valid && !packed);
  if (any_int) {
    const int rlen = (dem && !b.in_log) ? cd.R + cd.n_logicos : nbits;
    // this lane's bits from a ballot array over the entries starting at `first`
    // (and, for DEM logicals kept in their own array, from `lfirst` there)
    // (and its words into rec_cache, for the per-shot path if the shot goes there)
    uint32_t *cache = b.rec_cache ? b.rec_cache + (size_t)slot * kRecCacheWords : nullptr;
    auto extract = [&](long long first, long long lfirst, long long lbase) {
      const int off = (int)(rbase - first);
      if (errs) {
        for (int q = 0; q < nwords; ++q) {
          uint32_t w = flat_word(F.bits, off, q, nbits);
          if (cache) cache[q] = w;
          ow += __popc(w);
          while (w) {
            const int c = q * 32 + __ffs(w) - 1;
            w &= w - 1u;
            epos = c;
#pragma unroll
            for (int k = 0; k < kFastWords; ++k)
              if (k < cd.nw) s[k] ^= __ldg(cd.cols + (size_t)c * cd.nwp + k);
          }
        }
      } else {
#pragma unroll
        for (int k = 0; k < kFastWords; ++k)
          if (k < cd.nw) {
            s[k] = flat_word(F.bits, off, k, cd.R);
            if (cache) cache[k] = s[k];
          }
        if (dem) {
#pragma unroll
          for (int k = 0; k < kFastWords; ++k)
            if (k < cd.nlw) {
              lg[k] = b.in_log ? flat_word(F.lbits, (int)(lbase - lfirst), k, cd.n_logicos)
                               : flat_word(F.bits, off + cd.R, k, cd.n_logicos);
              if (cache) cache[cd.nw + k] = lg[k];
            }
        }
      }
      extracted = cache != nullptr;
    };
    const bool sep_log = dem && b.in_log && valid;
    if (__any_sync(kFull, sep_log)) {
      // DEM logicals in their own array: both arrays back to back over the chunk
      const long long nb = __shfl_down_sync(kFull, rbase, 1);
      const bool nv = __shfl_down_sync(kFull, valid ? 1 : 0, 1) != 0;
      const bool joined = !valid || lane == 31 || !nv || nb == rbase + rlen;
      const long long first = __shfl_sync(kFull, rbase, 0);
      long long end = valid ? rbase + rlen : first;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(kFull, end, o);
        end = u > end ? u : end;
      }
      bool flat = __all_sync(kFull, joined && !(valid && packed)) && end - first <= 32ll * kFastBallots;
      const long long lbase = sep_log ? (long long)shot * cd.n_logicos : 0;
      const long long lnb = __shfl_down_sync(kFull, lbase, 1);
      const bool ljoined = !valid || lane == 31 || !nv || lnb == lbase + cd.n_logicos;
      const long long lfirst = __shfl_sync(kFull, lbase, 0);
      long long lend = valid ? lbase + cd.n_logicos : lfirst;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const long long u = __shfl_xor_sync(kFull, lend, o);
        lend = u > lend ? u : lend;
      }
      flat = flat && __all_sync(kFull, ljoined && sep_log == (valid && dem)) &&
             lend - lfirst <= 32ll * kFastLogBallots;
      if (flat) {
        flat_ballots(b.in + first, (int)(end - first), F.bits);
        flat_ballots(b.in_log + lfirst, (int)(lend - lfirst), F.lbits);
        __syncwarp();
        if (ok) extract(first, lfirst, lbase);
      } else {
        ok = ok && packed;  // records that are not back to back: slow path
      }
    } else {
      // Runs of consecutive lanes whose int32 records lie back to back (one run
      // for a batch packed in slot order; a few where requests' records sit in
      // separate buffers): each run's entries through one pass of ballots.
      const bool mine = valid && !packed;
      const long long pend = __shfl_up_sync(kFull, rbase + rlen, 1);
      const bool pint = __shfl_up_sync(kFull, mine ? 1 : 0, 1) != 0;
      const unsigned members_all = __ballot_sync(kFull, mine);
      unsigned starts = __ballot_sync(kFull, mine && (lane == 0 || !pint || pend != rbase));
      while (starts) {
        const int l0 = __ffs(starts) - 1;
        starts &= starts - 1u;
        const int lnext = starts ? __ffs(starts) - 1 : 32;
        const unsigned span = (lnext == 32 ? kFull : ((1u << lnext) - 1u)) & ~((1u << l0) - 1u);
        const unsigned members = members_all & span;  // l0 .. the run's last lane, no gaps
        const int llast = 31 - __clz(members);
        const long long first = __shfl_sync(kFull, rbase, l0);
        const long long end = __shfl_sync(kFull, rbase + rlen, llast);
        const bool in_run = (members >> lane) & 1u;
        if (end - first > 32ll * kFastBallots) {
          if (in_run) ok = false;  // longer than the chunk's ballot area: slow path
          continue;
        }
        flat_ballots(b.in + first, (int)(end - first), F.bits);
        __syncwarp();
        if (in_run && ok) extract(first, 0, 0);
        __syncwarp();  // every lane has read the run's bits before the next run's
      }
    }
  }
  if (ok && packed) {
    const uint32_t *rw = reinterpret_cast<const uint32_t *>(b.in) + rbase;
    if (errs) {
      for (int q = 0; q < nwords; ++q) {
        uint32_t w = __ldcg(rw + q);
        if (q == nwords - 1 && (nbits & 31)) w &= (1u << (nbits & 31)) - 1u;
        ow += __popc(w);
        while (w) {
          const int c = q * 32 + __ffs(w) - 1;
          w &= w - 1u;
          epos = c;
#pragma unroll
          for (int k = 0; k < kFastWords; ++k)
            if (k < cd.nw) s[k] ^= __ldg(cd.cols + (size_t)c * cd.nwp + k);
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < kFastWords; ++k)
        if (k < cd.nw) {
          uint32_t w = __ldcg(rw + k);
          if (k == cd.nw - 1 && (cd.R & 31)) w &= (1u << (cd.R & 31)) - 1u;
          s[k] = w;
        }
      if (dem) {
        const uint32_t *lw = b.in_log ? reinterpret_cast<const uint32_t *>(b.in_log) + (size_t)shot * cd.nlw
                                      : rw + cd.nw;
#pragma unroll
        for (int k = 0; k < kFastWords; ++k)
          if (k < cd.nlw) {
            uint32_t w = __ldcg(lw + k);
            if (k == cd.nlw - 1 && (cd.n_logicos & 31)) w &= (1u << (cd.n_logicos & 31)) - 1u;
            lg[k] = w;
          }
      }
    }
  }
  if (!errs) ow = 0;
  tp = prof_lap(b, kProfChunkRead, tp);

  // ---- settle: empty syndrome, or a one-position first iteration matched ----
  const bool empty = ok && (s[0] | s[1] | s[2] | s[3]) == 0u;
  bool found = false, gpu = false;
  int pos = -1, deg = 0, iseq = 0;
  if (ok && !empty && cd.variant != kMl && cd.solo_cols && cd.binary && cd.max_soma >= 1 &&
      one_position_searched(cd, &gpu)) {
    // the first iteration's active set is the nonzero columns contained in s:
    // it is one column whose only candidate matches exactly when s equals a
    // solo column, found by s's sketch in the solo table
    uint32_t hs = 0u;
#pragma unroll
    for (int q = 0; q < kFastWords; ++q)
      for (uint32_t rows = q < cd.nw ? s[q] : 0u; rows; rows &= rows - 1u)
        hs ^= row_hash(q * 32 + __ffs(rows) - 1);
    uint32_t i = hs & cd.solo_mask;
    for (uint32_t probe = 0; probe <= cd.solo_mask && !found; ++probe) {
      const int c = __ldg(cd.solo_cols + i);
      if (c < 0) break;
      if (__ldg(cd.solo_keys + i) == hs) {
        bool eq = true;
#pragma unroll
        for (int k = 0; k < kFastWords; ++k)
          if (k < cd.nw) eq = eq && __ldg(cd.cols + (size_t)c * cd.nwp + k) == s[k];
        if (eq) {
          found = true;
          pos = c;
        }
      }
      i = (i + 1u) & cd.solo_mask;
    }
    if (found) {
      if (!dem && errs) {
        iseq = (ow == 1 && epos == pos) ? 1 : 0;
        deg = 1;
        found = iseq != 0;  // a different supplied error needs the degeneracy test
      } else if (dem) {
        deg = 1;
#pragma unroll
        for (int k = 0; k < kFastWords; ++k)
          if (k < cd.nlw && __ldg(cd.lcols + (size_t)pos * cd.nlw + k) != lg[k]) deg = 0;
      }
    }
  }
  const bool done = empty || found;
  if (!found) pos = -1;
  tp = prof_lap(b, kProfChunkTest, tp);

  // ---- results of the settled shots ----------------------------------------
  if (done) {
    const unsigned long long now = global_ns();
    uint32_t *r = F.res[lane];
#pragma unroll
    for (int w = 0; w < 18; ++w) r[w] = 0u;
    r[2] = (uint32_t)ow;
    if (empty) {
      r[8] = (uint32_t)-2;
    } else {
      const unsigned long long half = t_start + (now - t_start) / 2;  // counts ~ half the time
      const double t_sum = 1e-6 * (double)(half - t_start);
      const double t_search = 1e-6 * (double)(now - half);
      const double t_all = 1e-6 * (double)(now - t_start);
      r[0] = 1u;
      r[1] = 1u;
      r[3] = (uint32_t)deg;
      r[4] = (uint32_t)iseq;
      r[5] = 1u;
      r[6] = 1u;
      r[8] = gpu ? 0u : (uint32_t)-1;
      r[9] = 1u;
      const unsigned long long a = (unsigned long long)__double_as_longlong(t_sum);
      const unsigned long long bb = (unsigned long long)__double_as_longlong(t_search);
      const unsigned long long d = (unsigned long long)__double_as_longlong(t_all);
      r[10] = (uint32_t)a;
      r[11] = (uint32_t)(a >> 32);
      r[12] = (uint32_t)bb;
      r[13] = (uint32_t)(bb >> 32);
      r[16] = (uint32_t)d;
      r[17] = (uint32_t)(d >> 32);
    }
    if (b.ml_cost) b.ml_cost[shot] = 0.0f;
    if (b.deferred) b.deferred[shot] = 0;
  }
  __syncwarp();
  const unsigned settled = __ballot_sync(kFull, done);
  if (lane == 0 && settled)
    atomicAdd(ctr_ptr(b.counters, kCtrSettled), (unsigned long long)__popc(settled));
  for (unsigned mm = settled; mm; mm &= mm - 1u) {
    const int j = __ffs(mm) - 1;
    const int sj = __shfl_sync(kFull, shot, j);
    if (lane < 18) reinterpret_cast<uint32_t *>(b.results + sj)[lane] = F.res[j][lane];
    if (b.dec_err || b.dec_log) {
      const int cj = __shfl_sync(kFull, ci, j);
      const int pj = __shfl_sync(kFull, pos, j);
      const DevCode &cdj = b.codes[cj];
      if (b.dec_err)
        for (int c = lane; c < cdj.m; c += 32) b.dec_err[(size_t)sj * cdj.m + c] = c == pj ? 1 : 0;
      if (b.dec_log && cdj.family == kDem)
        for (int c = lane; c < cdj.n_logicos; c += 32)
          b.dec_log[(size_t)sj * cdj.n_logicos + c] =
              pj >= 0 ? (unsigned char)((__ldg(cdj.lcols + (size_t)pj * cdj.nlw + (c >> 5)) >> (c & 31)) & 1u)
                      : 0;
    }
  }

  // ---- the others: appended to the slow queue --------------------------------
  const bool slow = valid && !done;
  const unsigned sm = __ballot_sync(kFull, slow);
  if (sm) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(ctr_ptr(b.counters, kCtrQueueReserved), (unsigned long long)__popc(sm));
    base = __shfl_sync(kFull, base, 0);
    // the entry carries this launch's tag: a ticket holder that reads it knows it
    // is not a leftover of an earlier launch
    if (slow)
      *reinterpret_cast<volatile unsigned long long *>(b.queue + base + __popc(sm & lt_mask)) =
          ((unsigned long long)tag << 32) | (unsigned)slot | (extracted && ok ? 0x80000000u : 0u);
  }
  __syncwarp();
  prof_lap(b, kProfChunkWrite, tp);
}

}  // namespace grand
