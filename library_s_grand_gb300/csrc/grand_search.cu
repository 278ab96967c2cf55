// grand_search.cu -- kernel 2 of a decoding launch (sm_103a).
//
// search_kernel (persistent, every warp an independent worker)
//   every warp repeatedly takes the next tiles (K colex prefixes per lane of
//   one weight block of one Job) from a global counter, stages the iteration's
//   column sketches in its own shared-memory slice, evaluates them, publishes
//   the lowest matching global index (atomicMin) or the lowest {cost, rank}
//   key (128-bit CAS), and the warp that completes a Job's last tile writes its
//   result.  Tiles whose candidates all rank above an already-found match are
//   skipped.  No warp ever waits for another: there are no block barriers.
#include "grand_host.h"
#include "grand_kernels.cuh"

namespace grand {

// ---------------------------------------------------------------------------
// Kernel 2: persistent work-stealing search over the Jobs' tiles.
// ---------------------------------------------------------------------------
__device__ bool tile_skip(const Job &J, const Seg &S, const IterInfo &I, bool ml) {
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

__device__ Winner winner_ml(const Job &J) {
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

// MLK = false: a build without the ML paths for batches without ML codes.
template <bool MLK>
__global__ void __launch_bounds__(kSearchThreads, 3) search_kernel(DevBatch b) {
  __shared__ __align__(16) uint32_t s_stage[kSearchWarps][kWarpStage];
  __shared__ uint32_t s_sw[kSearchWarps][kMaxRows / 32];
  __shared__ uint32_t s_delta[kSearchWarps][kMaxCols / 32];

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  uint32_t *stage = s_stage[warp];
  uint32_t *sw = s_sw[warp];
  const unsigned long long packed = *reinterpret_cast<volatile unsigned long long *>(b.counters);
  unsigned long long njobs = packed >> 40;
  unsigned long long total = packed & ((1ull << 40) - 1ull);
  if (njobs > (unsigned long long)b.max_jobs) {
    njobs = b.max_jobs;
    total = njobs ? b.jobs[njobs - 1].tile_base + b.jobs[njobs - 1].ntiles : 0ull;
  }
  int st_job = -1, st_it = -1;
  // per-warp caches of the last job / weight block / run looked up, and a
  // register copy of the current weight block's parameters
  int cj = -1, cs = -1, cc = -1;
  unsigned long long cj_lo = 0, cj_hi = 0, cs_lo = 0, cs_hi = 0, cc_lo = 0, cc_hi = 0;
  Job *Jp = nullptr;
  const DevCode *cdp = nullptr;
  SegView sv{};
  int s_runs = 0, s_iter = 0, s_ml = 0, s_prob = 0;
  const unsigned long long *s_cum = nullptr;

  // Tiles are drawn several at a time when there are many per warp (the
  // lookups and the Job's tile count are then paid once per draw), one at a
  // time when there are few, so that a handful of expensive Jobs still spread
  // over every warp: the largest power of two up to kTilesPerFetch that leaves
  // each warp at least 8 draws.
  unsigned long long fetch = kTilesPerFetch;
  while (fetch > 1ull && total < 8ull * fetch * gridDim.x * kSearchWarps) fetch >>= 1;
  // the next draw is issued before the current tiles run, so its atomic's
  // round trip overlaps them
  unsigned long long draw = 0;
  if (lane == 0) draw = atomicAdd(&b.counters[1], fetch);
  for (;;) {
    const unsigned long long t0 = __shfl_sync(kFull, draw, 0);
    if (t0 >= total) break;
    if (lane == 0) draw = atomicAdd(&b.counters[1], fetch);
    const unsigned long long t1 = (t0 + fetch < total) ? t0 + fetch : total;
    bool skip_known = false, skip = false;
    unsigned long long pending = 0;
    bool fenced = false;
    for (unsigned long long t = t0; t < t1; ++t) {
      if (cj < 0 || t < cj_lo || t >= cj_hi) {
        const int lo = warp_search_le(0, (int)njobs - 1, t,
                                      [&](int j) { return b.jobs[j].tile_base; });
        cj = lo;
        Jp = &b.jobs[lo];
        cdp = &b.codes[Jp->code];
        cj_lo = Jp->tile_base;
        cj_hi = cj_lo + Jp->ntiles;
        cs = -1;
      }
      Job &J = *Jp;
      const unsigned long long lt = t - cj_lo;
      if (cs < 0 || lt < cs_lo || lt >= cs_hi) {
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
        cs = sg;
        cs_lo = S.tile_lo;
        cs_hi = cs_lo + S.njt;
        cc = -1;
        s_runs = S.runs;
        s_cum = S.cum;
        s_iter = S.iter;
        s_ml = MLK && cdp->variant == kMl;
        s_prob = cdp->variant == kProb;
        // the scans read only the column sketches: those are staged (the full
        // columns are read from the Job's scratch for the rare exact tests)
        const bool staged = I.tam <= kWarpStage;
        sv = SegView{staged ? stage : I.hcols, I.cols, I.llr, J.hs, I.tam, S.w, S.K, cdp->nwp,
                     cdp->nw, S.nprefix, S.base};
        if (st_job != cj || st_it != S.iter) {
          __syncwarp();
          if (staged) {
            const uint4 *src = reinterpret_cast<const uint4 *>(I.hcols);
            uint4 *dst = reinterpret_cast<uint4 *>(stage);
            const int n4 = (I.tam + 3) / 4;
            for (int i = lane; i < n4; i += 32) dst[i] = src[i];
          }
          sw[lane] = J.sw[lane];
          __syncwarp();
          st_job = cj;
          st_it = S.iter;
        }
        skip_known = false;
      }
      if (!skip_known || s_ml) {
        // one decision for the warp: other warps lower the bound while lanes read it
        skip = __any_sync(kFull, tile_skip(J, J.seg[cs], J.it[s_iter], s_ml));
        skip_known = true;
      }
      bool published = false;
      if (!skip) {
        LaneBest lb;
        lb.reset();
        const unsigned long long st = lt - cs_lo;
        if (s_runs) {
          if (cc < 0 || st < cc_lo || st >= cc_hi) {
            // run c holding segment tile st: largest c with cum[c] <= st
            const unsigned long long *cum = s_cum;
            const int clo = warp_search_le(0, sv.tam - 2, st, [&](int i) { return cum[i]; });
            cc = clo;
            cc_lo = s_cum[clo];
            cc_hi = cc_lo + run_tiles(b.ncr, clo, sv.w, kRunKK);
          }
          const unsigned long long r0 = (st - cc_lo) * (32ull * kRunKK);
          if (s_ml) eval_run_tile<kRunKK, true>(sv, b.ncr, sw, cc, r0, lb);
          else eval_run_tile<kRunKK, false>(sv, b.ncr, sw, cc, r0, lb);
        } else {
          if (s_ml) eval_tile<true>(sv, b.ncr, sw, st, lb);
          else eval_tile<false>(sv, b.ncr, sw, st, lb);
        }
        // a tile without a match (nearly every tile) skips the reductions
        if (!s_ml) {
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
          if (lane == 0 && !atomic_min_key(J.mlkey[s_iter][sv.w], o, r))
            atomicOr(b.status, kStatusCasLimit);
        }
      }
      // tiles of this fetch done for the current job: posted once per job per fetch
      pending += 1ull;
      fenced = fenced || published;
      const bool flush = (t + 1 == t1) || (t + 1 >= cj_hi);
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
          // loads.  The stage holds no columns afterwards.
          static_assert(sizeof(Job) <= sizeof(uint32_t) * kWarpStage, "Job must fit the stage");
          const uint4 *src = reinterpret_cast<const uint4 *>(&J);
          uint4 *dst = reinterpret_cast<uint4 *>(stage);
          for (int i = lane; i < (int)(sizeof(Job) / 16); i += 32) dst[i] = __ldcg(src + i);
          __syncwarp();
          st_job = -1;
          cs = -1;
          const Job &F = *reinterpret_cast<const Job *>(stage);
          Winner wn;
          if (!s_ml) wn = winner_from_index(F, F.best, s_prob != 0);
          else wn = winner_ml(F);
          finish_shot(b, *cdp, F, F.shot, wn, F.ebits, s_delta[warp]);
          __syncwarp();
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Host-callable launcher.
// ---------------------------------------------------------------------------
#ifndef GRAND_HOST_EMULATION  // launchers: device builds only
cudaError_t launch_search(const DevBatch &b, int grid, cudaStream_t s) {
  if (b.has_ml) search_kernel<true><<<grid, kSearchThreads, 0, s>>>(b);
  else search_kernel<false><<<grid, kSearchThreads, 0, s>>>(b);
  return cudaGetLastError();
}

int search_threads_per_block() { return kSearchThreads; }

cudaError_t occupancy(int *triage_blocks_per_sm, int *search_blocks_per_sm) {
  cudaError_t e = triage_occupancy(triage_blocks_per_sm);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(search_blocks_per_sm, search_kernel<true>,
                                                       kSearchThreads, 0);
}

#endif

}  // namespace grand
