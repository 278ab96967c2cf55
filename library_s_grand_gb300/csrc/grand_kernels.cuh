// grand_kernels.cuh -- what the decode kernel's work steps share (classification,
// the per-shot path and the search, grand_decode.cuh): launch constants, the
// per-warp shared area, bounded waits, the Job front, the per-shot result writer
// and the first-hit winner lookup.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include "grand_device.cuh"
#include "grand_lookup.cuh"

namespace grand {

constexpr int kDecodeWarps = 4;                 // warps per block of the decode kernel
constexpr int kLightTam = 96;                   // largest active set the triage warp searches
constexpr int kLightWords = kLightTam * 8;      // its staged column words (nwp <= 8)
// per search warp: the staged lookup block of an iteration, or the Job at its
// end (the rest of the warp's area holds the syndrome and the degeneracy delta)
constexpr int kWarpStage = 2720;
constexpr int kTilesPerFetch = 16;  // most tiles a search warp draws at once
// Launch slots per classification chunk (one lane each): fewer than 32 spreads a
// batch's classification over more warps, so it ends sooner.
constexpr int kChunkShots = 32;
constexpr int kRunKKLight = 4;  // prefixes per lane in a run tile of the triage warp's light search

// Per-warp shared memory of the decode kernel.  A warp does one kind of work at
// a time and reuses the same bytes for it: a shot's triage (the fields below), a
// chunk's classification (FastArea, grand_triage.cuh) or search tiles (the first
// kWarpStage words hold the staged lookup block or a Job being finished, then
// the syndrome and the degeneracy delta).  While a Job is published, the light
// search's arrays (cols .. tmp) are the scratch that builds its lookup tables.
struct alignas(128) WarpArea {
  uint32_t cols[kLightWords];
  uint32_t hcols[kLightTam];
  float llr[kLightTam];
  int pos[kLightTam];
  int tmp[kLightTam];
  uint32_t sw[kMaxRows / 32];
  uint32_t eb[kMaxCols / 32];
  uint32_t am[kMaxIters][kMaxCols / 32];
  uint32_t delta[kMaxCols / 32];
  Job job;
};

// Words of the light search's arrays (cols .. tmp), the publishing warp's
// working space for a heavy iteration's positions.
constexpr int kPublishWords = kLightWords + 4 * kLightTam;
static_assert(offsetof(WarpArea, sw) - offsetof(WarpArea, cols) == sizeof(uint32_t) * kPublishWords,
              "the light search's arrays are contiguous");

// Planner state of one shot (resumable walk over upstream's iteration loop).
struct PlanState {
  int i, tam, tam_old, passes;
  unsigned long long gbase;
};

// Bounded waits.  A warp that waits for another warp's progress sleeps between
// polls, longer as the wait goes on; after kWaitPolls polls it gives up and
// raises kStatusWaitLimit (never expected: every wait is for a warp that is
// running and waits for nothing this warp holds).  kShortPolls bounds the
// waits for an entry or Job another warp has reserved and is writing.
constexpr int kWaitPolls = 1 << 21;
constexpr int kShortPolls = 1 << 16;

__device__ __forceinline__ void nap(int polls) {
#ifdef GRAND_HOST_EMULATION
  grand_host_nap(polls);
#else
  __nanosleep(polls < 4 ? 200u : (polls < 32 ? 800u : 2000u));
#endif
}

__device__ __forceinline__ unsigned long long ld_ctr(const DevBatch &b, int ctr) {
  return *reinterpret_cast<volatile unsigned long long *>(ctr_ptr(b.counters, ctr));
}

// Profile (DevBatch::profile): lane 0 adds the time since t0 to profile sums
// word w; returns the current time (0 when not profiling).
__device__ __forceinline__ unsigned long long prof_lap(const DevBatch &b, int w,
                                                       unsigned long long t0,
                                                       int line = kCtrProfSums) {
  if (!b.profile) return 0ull;
  const unsigned long long t = global_ns();
  if ((threadIdx.x & 31) == 0) atomicAdd(ctr_ptr(b.counters, line) + w, t - t0);
  return t;
}

// The whole warp.  Jobs are searchable from the front: the leading Jobs whose
// ready words carry this launch's tag.  Whoever finds Jobs at the front written
// moves the front past them: the warp reads the ready words of the next 32 Jobs
// at once and passes the written run among them (their tiles summed across the
// lanes) with one compare-and-swap, so a long run of Jobs published together
// costs a few round trips, not one per Job.  A publisher calls this after
// marking its Job ready, so every written Job is passed: the publisher of the
// last Job to become ready finds all before it written.
__device__ __forceinline__ void advance_front(const DevBatch &b, unsigned tag) {
  const int lane = threadIdx.x & 31;
  unsigned long long f = 0, lim = 0;
  if (lane == 0) {
    f = ld_ctr(b, kCtrFront);
    lim = ld_ctr(b, kCtrJobs) >> 40;
    if (lim > (unsigned long long)b.max_jobs) lim = (unsigned long long)b.max_jobs;
  }
  f = __shfl_sync(kFull, f, 0);
  lim = __shfl_sync(kFull, lim, 0);
  for (int guard = 0; guard < (1 << 16); ++guard) {
    const unsigned long long j = (f >> 40) + (unsigned long long)lane;
    const bool ready =
        j < lim && *reinterpret_cast<const volatile unsigned *>(&b.jobs[j].ready) == tag;
    const unsigned m = __ballot_sync(kFull, ready);
    const int run = (m == kFull) ? 32 : __ffs(~m) - 1;  // written Jobs at the front
    if (run == 0) return;
    unsigned long long nt =
        lane < run ? *reinterpret_cast<const volatile unsigned long long *>(&b.jobs[j].ntiles) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nt += __shfl_xor_sync(kFull, nt, o);
    unsigned long long seen = 0;
    if (lane == 0)
      seen = atomicCAS(ctr_ptr(b.counters, kCtrFront), f,
                       f + ((unsigned long long)run << 40) + nt);
    seen = __shfl_sync(kFull, seen, 0);
    f = seen == f ? f + ((unsigned long long)run << 40) + nt : seen;
  }
}

// ---------------------------------------------------------------------------
// Result writer shared by the per-shot path and the Job search (one warp).
// ---------------------------------------------------------------------------
struct Winner {
  int found;
  int ii;                   // index into J.it
  int seg;                  // index into J.seg
  unsigned long long rank;  // lexicographic rank inside the weight block
  unsigned long long count; // candidates the winning iteration reports
  float cost;
  unsigned mask;            // the winner's active positions as a bit mask (0: from rank)
};

static __device__ void finish_shot(const DevBatch &b, const DevCode &cd, const Job &J, int shot,
                            const Winner &wn, const uint32_t *ebits, uint32_t *delta) {
  const int lane = threadIdx.x & 31;
  int p[kMaxW];
  int w = 0;
  if (wn.found) {
    const Seg &S = J.seg[wn.seg];
    const IterInfo &I = J.it[wn.ii];
    w = S.w;
    int c[kMaxW];
    if (wn.mask) {  // the small-set path hands over the positions themselves
      unsigned mm = wn.mask;
#pragma unroll
      for (int i = 0; i < kMaxW; ++i) {
        c[i] = mm ? __ffs(mm) - 1 : 0;
        mm &= mm - 1u;
      }
    } else {
      lex_unrank_warp(wn.rank, I.tam, w, c);
    }
#pragma unroll
    for (int i = 0; i < kMaxW; ++i) p[i] = (i < w) ? I.pos[c[i]] : -1;
  } else {
#pragma unroll
    for (int i = 0; i < kMaxW; ++i) p[i] = -1;
  }

  int degenerate = 0, is_equal = 0;
  if (wn.found && cd.family == kCss && cd.input_kind == kInErrors) {
    // is_equal: supplied error == decoded error (grand_decoder.cu:1362).
    bool eq = true;
    for (int q = lane; q < cd.mw; q += 32) {
      uint32_t e = 0;
#pragma unroll
      for (int i = 0; i < kMaxW; ++i)
        if (i < w && (p[i] >> 5) == q) e |= 1u << (p[i] & 31);
      uint32_t d = ebits[q] ^ e;
      delta[q] = d;
      eq = eq && d == 0u;
    }
    is_equal = __all_sync(kFull, eq) ? 1 : 0;
    __syncwarp();
  }
  if (is_equal) {
    degenerate = 1;  // delta = 0 lies in every row space
  } else if (wn.found && cd.family == kCss && cd.input_kind == kInErrors) {
    // degenerate: (e ^ e_est) in the row space of the other matrix
    // (grand_decoder.cu:456-474).  In reduced row echelon form the vector's own
    // bits at pivot columns decide alone which rows upstream adds, so the test
    // is delta == XOR of the rows pivoted on delta's set bits.
    // Each lane looks up the pivot row of one set bit of a delta word, then the
    // warp XORs those rows four at a time (their loads issued together).
    uint32_t acc[4] = {0u, 0u, 0u, 0u};  // words lane, lane+32, lane+64, lane+96
    for (int q = 0; q < cd.mw; ++q) {
      const uint32_t word = delta[q];
      if (word == 0u) continue;
      const int r = ((word >> lane) & 1u) ? __ldg(cd.pivrow + q * 32 + lane) : -1;
      unsigned m = __ballot_sync(kFull, r >= 0);
      while (m) {
        int rb[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          rb[u] = -1;
          if (m) {
            rb[u] = __shfl_sync(kFull, r, __ffs(m) - 1);
            m &= m - 1u;
          }
        }
        uint32_t v[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int k = 0; k < 4; ++k)
            v[u][k] = (rb[u] >= 0 && lane + 32 * k < cd.mw)
                          ? __ldg(cd.rref + (size_t)rb[u] * cd.mw + lane + 32 * k)
                          : 0u;
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int k = 0; k < 4; ++k) acc[k] ^= v[u][k];
      }
    }
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (lane + 32 * k < cd.mw) ok = ok && acc[k] == delta[lane + 32 * k];
    degenerate = __all_sync(kFull, ok) ? 1 : 0;
  } else if (wn.found && cd.family == kDem) {
    // decoded logical flips vs the supplied true flips (grand_decoder.cu:1623-1644)
    bool eq = true;
    for (int q = lane; q < cd.nlw; q += 32) {
      uint32_t le = 0;
#pragma unroll
      for (int i = 0; i < kMaxW; ++i)
        if (i < w) le ^= __ldg(cd.lcols + (size_t)p[i] * cd.nlw + q);
      eq = eq && le == ebits[q];
      if (b.dec_log) {
        for (int j = 0; j < 32 && q * 32 + j < cd.n_logicos; ++j)
          b.dec_log[(size_t)shot * cd.n_logicos + q * 32 + j] = (unsigned char)((le >> j) & 1u);
      }
    }
    degenerate = __all_sync(kFull, eq) ? 1 : 0;
  } else if (cd.family == kDem && b.dec_log) {
    for (int j = lane; j < cd.n_logicos; j += 32) b.dec_log[(size_t)shot * cd.n_logicos + j] = 0;
  }

  if (b.dec_err) {
    for (int c = lane; c < cd.m; c += 32) {
      unsigned char v = 0;
#pragma unroll
      for (int i = 0; i < kMaxW; ++i)
        if (i < w && p[i] == c) v = 1;
      b.dec_err[(size_t)shot * cd.m + c] = v;
    }
  }

  // The 72-byte result, written by lanes 0..17 as one coalesced store of 32-bit
  // words (every lane holds the same fields; lane l stores word l).
  int h = -2;
  unsigned long long tested = 0;
  const int last = wn.found ? wn.ii : J.n_it - 1;
  for (int k = 0; k <= last; ++k) {
    h = (J.it[k].branch == kBranchGpu) ? (h == -1 ? 1 : 0) : -1;
    if (k < last || !wn.found) tested += J.it[k].total;
  }
  if (wn.found) tested += wn.count;
  // Per-shot times from the global timer: the flagged-check count step, the
  // search from its end to this result (light search, plus queueing and the
  // search kernel for a published Job), and, when found, the whole shot.
  // Records move in one batch (or are read in place), so no copy time is
  // attributed to a shot.  Lanes 10..17 each convert the double they store.
  const unsigned long long now = __shfl_sync(kFull, global_ns(), 0);
  const unsigned long long dt = lane < 12   ? J.t_counts - J.t_start
                                : lane < 14 ? now - J.t_counts
                                : lane < 16 ? 0ull
                                            : (wn.found ? now - J.t_start : 0ull);
  const unsigned long long dbits = (unsigned long long)__double_as_longlong(1e-6 * (double)dt);
  // a chain of selects rather than a switch on the lane, which would run its
  // cases one after another
  const uint32_t f_tam = (uint32_t)(wn.found ? J.it[wn.ii].tam : J.final_tam);
  const uint32_t f_it = (uint32_t)(wn.found ? J.it[wn.ii].it : J.final_iteration);
  uint32_t v = (lane & 1) ? (uint32_t)(dbits >> 32) : (uint32_t)dbits;
  v = lane == 9 ? f_it : v;
  v = lane == 8 ? (uint32_t)h : v;
  v = lane == 7 ? (uint32_t)(tested >> 32) : v;
  v = lane == 6 ? (uint32_t)tested : v;
  v = lane == 5 ? f_tam : v;
  v = lane == 4 ? (uint32_t)is_equal : v;
  v = lane == 3 ? (uint32_t)degenerate : v;
  v = lane == 2 ? (uint32_t)J.original_weight : v;
  v = lane == 1 ? (uint32_t)w : v;
  v = lane == 0 ? (uint32_t)wn.found : v;
  static_assert(sizeof(GrandDecoderResult) == 72, "result layout");
  if (lane < 18) reinterpret_cast<uint32_t *>(b.results + shot)[lane] = v;
  if (lane == 0) {
    if (b.ml_cost) b.ml_cost[shot] = wn.found ? wn.cost : 0.0f;
    if (J.failed) atomicOr(b.status, kStatusTamLimit);
  }
}

// Winner of a first-hit search from the lowest matching global index.
static __device__ Winner winner_from_index(const Job &J, unsigned long long g, bool prob) {
  Winner wn;
  wn.found = 0;
  wn.ii = wn.seg = 0;
  wn.rank = wn.count = 0;
  wn.cost = 0.0f;
  wn.mask = 0u;
  if (g == kNone) return wn;
  for (int ii = 0; ii < J.n_it; ++ii) {
    const IterInfo &I = J.it[ii];
    if (g < I.base || g >= I.base + I.total) continue;
    for (int s = I.seg_lo; s < I.seg_hi; ++s) {
      const Seg &S = J.seg[s];
      if (S.dup || g < S.base || g >= S.base + S.count) continue;
      wn.found = 1;
      wn.ii = ii;
      wn.seg = s;
      wn.rank = g - S.base;
      if (I.branch == kBranchCpu) wn.count = g - I.base + 1ull;  // grand_decoder.cu:547-548
      else if (prob) wn.count = I.phase_end[S.phase];            // grand_decoder.cu:1006
      else wn.count = I.total;                                   // grand_decoder.cu:1303-1304
      return wn;
    }
  }
  return wn;
}

}  // namespace grand
