// grand_search.cuh -- the search of a decoding launch (sm_103a), run by the warps
// of the persistent decode kernel (grand_decode.cuh).
//
// search_tiles: a warp evaluates a range of tiles (K colex prefixes per lane of
//   one weight block of one Job, each probing the iteration's lookup tables,
//   grand_lookup.cuh) it drew from the launch's tile counter, stages the
//   iteration's lookup block in its own shared-memory slice, publishes the
//   lowest matching global index (atomicMin) or the lowest {cost, rank} key
//   (128-bit CAS), and the warp that completes a Job's last tile writes its
//   result.  Tiles whose candidates all rank above an already-found match are
//   skipped.  No warp waits for another here: there are no block barriers.
#pragma once

#include "grand_kernels.cuh"

namespace grand {

// ---------------------------------------------------------------------------
// Skip test and ML winner.
// ---------------------------------------------------------------------------
static __device__ bool tile_skip(const Job &J, const Seg &S, const IterInfo &I, bool ml) {
  if (!ml) {
    const unsigned long long best = *reinterpret_cast<const volatile unsigned long long *>(&J.best);
    return S.base >= best;
  }
  for (int i = 0; i < S.iter; ++i)
    for (int w = 1; w <= kMaxW; ++w)
      if (*reinterpret_cast<const volatile unsigned long long *>(&J.mlkey[i][w][0]) != kNone)
        return true;
  for (int w = 1; w < S.w; ++w) {
    const unsigned long long o =
        *reinterpret_cast<const volatile unsigned long long *>(&J.mlkey[S.iter][w][0]);
    if (o != kNone && I.prefix[S.w] >= key_cost((uint32_t)o)) return true;
  }
  return false;
}

static __device__ Winner winner_ml(const Job &J) {
  Winner wn;
  wn.found = 0;
  wn.ii = wn.seg = 0;
  wn.rank = wn.count = 0;
  wn.cost = 0.0f;
  wn.mask = 0u;
  for (int ii = J.it_lo; ii < J.n_it; ++ii) {
    const IterInfo &I = J.it[ii];
    uint32_t bo = 0xffffffffu;
    unsigned long long br = kNone, proc = 0;
    int bseg = -1;
    for (int s = I.seg_lo; s < I.seg_hi; ++s) {
      const Seg &S = J.seg[s];
      if (bseg >= 0 && I.prefix[S.w] >= key_cost(bo)) break;
      proc += S.count;
      const unsigned long long o = J.mlkey[ii][S.w][0];
      if (o != kNone && (bseg < 0 || (uint32_t)o < bo)) {
        bo = (uint32_t)o;
        br = J.mlkey[ii][S.w][1];
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
      return wn;
    }
  }
  return wn;
}

// What a tile evaluation reads about its weight block and lookup tables: one
// copy per warp in shared memory, written by lane 0 when the warp moves to
// another block, so that none of it occupies registers between tiles.
struct TileView {
  SegView sv;
  LookView lk;
};

// Per-warp state carried from one drawn tile range to the next: the last Job
// and weight block looked up (tiles of one draw are consecutive, so the lookups
// are mostly reused) and which iteration's lookup block is in the stage.
struct SearchCache {
  int st_job, st_it;
  int cj, cs;
  unsigned long long cj_lo, cj_hi, cs_lo, cs_hi;
  Job *Jp;
  const DevCode *cdp;
  int staged;  // the lookup block is in the warp's stage
  int s_iter, s_ml, s_prob;
  __device__ void reset() {
    st_job = st_it = -1;
    cj = cs = -1;
    cj_lo = cj_hi = cs_lo = cs_hi = 0;
    Jp = nullptr;
    cdp = nullptr;
    staged = s_iter = s_ml = s_prob = 0;
  }
  // the stage was used for other work: its tables are gone
  __device__ void stage_lost() { st_job = st_it = -1; }
};

// Search tiles [t0, t1) of the written Jobs (njobs of them, from slot 0; every
// tile below their total belongs to one).  The warp's WarpArea holds the staged
// sketches (or, while a Job is finished, the Job).
template <bool MLK>
__device__ void search_tiles(const DevBatch &b, unsigned long long t0, unsigned long long t1,
                             unsigned long long njobs, WarpArea &A, SearchCache &c, TileView &V) {
  const int lane = threadIdx.x & 31;
  uint32_t *stage = reinterpret_cast<uint32_t *>(&A);
  uint32_t *sw = stage + kWarpStage;
  uint32_t *delta = sw + kMaxRows / 32;
  static_assert(sizeof(WarpArea) >= sizeof(uint32_t) * (kWarpStage + kMaxRows / 32 + kMaxCols / 32),
                "the search stage must fit the warp's area");
  bool skip_known = false, skip = false;
  unsigned long long pending = 0;
  bool fenced = false;
  for (unsigned long long t = t0; t < t1; ++t) {
    unsigned long long tp = b.profile ? global_ns() : 0ull;
    if (c.cj < 0 || t < c.cj_lo || t >= c.cj_hi) {
      const int lo = warp_search_le(0, (int)njobs - 1, t,
                                    [&](int j) { return b.jobs[j].tile_base; });
      c.cj = lo;
      c.Jp = &b.jobs[lo];
      c.cdp = &b.codes[c.Jp->code];
      c.cj_lo = c.Jp->tile_base;
      c.cj_hi = c.cj_lo + c.Jp->ntiles;
      c.cs = -1;
    }
    Job &J = *c.Jp;
    const unsigned long long lt = t - c.cj_lo;
    if (c.cs < 0 || lt < c.cs_lo || lt >= c.cs_hi) {
      // the weight block holding job tile lt: every lane tests one block
      const int nseg = J.nseg;
      int sg = -1;
      for (int i0 = 0; i0 < nseg && sg < 0; i0 += 32) {
        bool hit = false;
        if (i0 + lane < nseg) {
          const Seg &C = J.seg[i0 + lane];
          const unsigned long long njt = C.njt, tlo = C.tile_lo;
          hit = njt && lt >= tlo && lt < tlo + njt;
        }
        const unsigned m = __ballot_sync(kFull, hit);
        if (m) sg = i0 + __ffs(m) - 1;
      }
      if (sg < 0) sg = nseg - 1;
      const Seg &S = J.seg[sg];
      const IterInfo &I = J.it[S.iter];
      c.cs = sg;
      c.cs_lo = S.tile_lo;
      c.cs_hi = c.cs_lo + S.njt;
      c.s_iter = S.iter;
      c.s_ml = MLK && c.cdp->variant == kMl;
      c.s_prob = c.cdp->variant == kProb;
      // the iteration's lookup block (sketches, filter, buckets) is built in
      // the stage when it fits (otherwise the publisher built it in the
      // scratch); the full columns stay in the Job's scratch for exact tests
      const LookLayout L = look_layout(I.tam, kWarpStage);
      c.staged = L.words <= kWarpStage;
      const uint32_t *blk = c.staged ? stage : I.hcols;
      __syncwarp();  // every lane is done with the previous view
      if (lane == 0) {
        V.sv = SegView{blk, I.cols, I.llr, J.hs, I.tam, S.w, kLookK, c.cdp->nwp,
                       c.cdp->nw, S.nprefix, S.base};
        V.lk = look_view(blk, L);
      }
      if (c.st_job != c.cj || c.st_it != S.iter) {
        if (c.staged) {
          const uint4 *src = reinterpret_cast<const uint4 *>(I.hcols);
          uint4 *dst = reinterpret_cast<uint4 *>(stage);
          const int n4 = (I.tam + 3) / 4;
          for (int i = lane; i < n4; i += 32) dst[i] = __ldcg(src + i);
          __syncwarp();
          build_lookup(stage, I.tam, L);
        }
        sw[lane] = J.sw[lane];
        c.st_job = c.cj;
        c.st_it = S.iter;
      }
      __syncwarp();
      skip_known = false;
    }
    tp = prof_lap(b, kProfTileSetup, tp);
    if (!skip_known || c.s_ml) {
      // one decision for the warp: other warps lower the bound while lanes read it
      skip = __any_sync(kFull, tile_skip(J, J.seg[c.cs], J.it[c.s_iter], c.s_ml));
      skip_known = true;
    }
    bool published = false;
    if (!skip) {
      const unsigned long long st = lt - c.cs_lo;
      LaneBest lb;
      if (c.staged) {
        if (MLK && c.s_ml) lb = eval_lookup_tile<kLookK, MLK, true>(V.sv, V.lk, b.ncr, sw, st);
        else lb = eval_lookup_tile<kLookK, false, true>(V.sv, V.lk, b.ncr, sw, st);
      } else {
        if (MLK && c.s_ml) lb = eval_lookup_tile<kLookK, MLK, false>(V.sv, V.lk, b.ncr, sw, st);
        else lb = eval_lookup_tile<kLookK, false, false>(V.sv, V.lk, b.ncr, sw, st);
      }
      // a tile without a match (nearly every tile) skips the reductions
      if (!c.s_ml) {
        if (__any_sync(kFull, lb.g != kNone)) {
          const unsigned long long g = warp_min_u64(lb.g);
          published = true;
          skip_known = false;
          if (lane == 0) atomicMin(&J.best, g);
        }
      } else if (__any_sync(kFull, lb.o != 0xffffffffu)) {
        uint32_t o = lb.o;
        unsigned long long r = lb.r;
        warp_min_key(o, r);
        published = true;
        if (lane == 0 && !atomic_min_key(J.mlkey[c.s_iter][J.seg[c.cs].w], o, r))
          atomicOr(b.status, kStatusCasLimit);
      }
    }
    // tiles of this range done for the current Job: posted once per Job per range
    pending += 1ull;
    fenced = fenced || published;
    const bool flush = (t + 1 == t1) || (t + 1 >= c.cj_hi);
    if (flush) {
      int last = 0;
      if (lane == 0) {
        if (fenced) __threadfence();  // order the published minima before the count
        last = (atomicAdd(&J.tiles_done, pending) + pending == J.ntiles) ? 1 : 0;
      }
      pending = 0;
      fenced = false;
      last = __shfl_sync(kFull, last, 0);
      if (last) {
        __threadfence();
        // The Job as the other warps left it, read from L2 (past this SM's
        // L1) into this warp's stage in one pass, so the winner lookup and
        // the result writer walk shared memory instead of chains of global
        // loads.  The stage holds no sketches afterwards.
        static_assert(sizeof(Job) <= sizeof(uint32_t) * kWarpStage, "Job must fit the stage");
        const uint4 *src = reinterpret_cast<const uint4 *>(&J);
        uint4 *dst = reinterpret_cast<uint4 *>(stage);
        for (int i = lane; i < (int)(sizeof(Job) / 16); i += 32) dst[i] = __ldcg(src + i);
        __syncwarp();
        c.st_job = -1;
        c.cs = -1;
        const Job &F = *reinterpret_cast<const Job *>(stage);
        Winner wn;
        if (!c.s_ml) wn = winner_from_index(F, F.best, c.s_prob != 0);
        else wn = winner_ml(F);
        finish_shot(b, *c.cdp, F, F.shot, wn, F.ebits, delta);
        __syncwarp();
        prof_lap(b, kProfTileFinish, tp);
      }
    }
  }
}
}  // namespace grand
