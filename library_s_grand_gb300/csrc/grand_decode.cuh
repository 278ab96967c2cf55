// grand_decode.cuh -- the persistent decode kernel (sm_103a): one launch per batch.
//
// Every warp of the grid loops over whatever work the batch has left, in this
// order of preference:
//   1. classification chunks: 32 launch slots, one lane per shot; empty
//      syndromes and weight-1 matches of a one-position first iteration are
//      settled there, the other shots go to the slow queue (classify_chunk);
//   2. slow-queue shots: one warp per shot, the full threshold-iteration walk
//      with the light search, publishing a Job for iterations over the light
//      budget (triage_shot);
//   3. search tiles of published Jobs (search_tiles); the warp that completes
//      a Job's last tile writes its result.
// So a heavy shot's search starts as soon as its Job is published, while other
// warps are still classifying and triaging, and triage and search share the GPU
// instead of running as two launches one after the other.
//
// Drawing: chunks by atomicAdd (a draw past the end is dropped), queue entries
// by compare-and-swap below the published count, tiles by atomicAdd below the
// published tile total -- a tile drawn past it stays with the warp (held) until
// a Job covering it is published or the batch has no more work.  Queue entries
// and Jobs are published in reservation order, each once it is fully written.
//
// A warp that finds nothing to do sleeps and polls (bounded, kStatusWaitLimit on
// exhaustion).  It waits only for work that running warps are producing -- they
// never wait for it -- and leaves once every chunk and slow shot is finished and
// no published tile is left undrawn.
#pragma once

#include "grand_search.cuh"
#include "grand_triage.cuh"

namespace grand {

constexpr int kDecodeMinBlocks = 4;  // resident blocks per SM the register budget allows

__device__ __forceinline__ unsigned long long ld_ctr(const DevBatch &b, int ctr) {
  return *reinterpret_cast<volatile unsigned long long *>(b.counters + ctr);
}

// Lane 0: the next slow-queue entry below the published count (-1 if none now).
__device__ __forceinline__ int draw_slow(const DevBatch &b) {
  unsigned long long h = ld_ctr(b, kCtrQueueHead);
  for (int guard = 0; guard < 64; ++guard) {
    const unsigned long long avail = b.fast ? ld_ctr(b, kCtrQueuePublished)
                                            : (unsigned long long)b.num_shots;
    if (h >= avail) return -1;
    const unsigned long long seen = atomicCAS(&b.counters[kCtrQueueHead], h, h + 1ull);
    if (seen == h) {
      if (!b.fast) return (int)h;  // every slot takes the per-shot path
      return *reinterpret_cast<volatile int *>(b.queue + h);
    }
    h = seen;
  }
  return -1;
}

// What a warp does next (decided by lane 0 from the control words, then
// broadcast, so that the whole warp takes the same path).
enum Step { kStepWait = 0, kStepChunk = 1, kStepShot = 2, kStepTiles = 3, kStepExit = 4 };

template <bool MLK>
__global__ void __launch_bounds__(kDecodeWarps * 32, kDecodeMinBlocks) decode_kernel(DevBatch b) {
  __shared__ WarpArea areas[kDecodeWarps];
  __shared__ PlanState plans[kDecodeWarps];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  WarpArea &A = areas[wib];
  SearchCache cache;
  cache.reset();
  const unsigned long long nchunks = b.fast ? (unsigned long long)((b.num_shots + 31) / 32) : 0ull;
  const unsigned long long nwarps = (unsigned long long)gridDim.x * kDecodeWarps;
  constexpr unsigned long long kTileMask = (1ull << 40) - 1ull;
  unsigned long long held_lo = 0, held_hi = 0;  // lane 0: tiles drawn and not yet run
  int polls = 0;
  for (;;) {
    int step = kStepWait;
    unsigned long long a0 = 0, a1 = 0, a2 = 0;
    if (lane == 0) {
      // 1. classification chunks (a draw past the end is dropped)
      if (nchunks && ld_ctr(b, kCtrNextChunk) < nchunks) {
        const unsigned long long k = atomicAdd(&b.counters[kCtrNextChunk], 1ull);
        if (k < nchunks) {
          step = kStepChunk;
          a0 = k;
        }
      }
      // 2. the per-shot path
      if (step == kStepWait) {
        const int slot = draw_slow(b);
        if (slot >= 0) {
          step = kStepShot;
          a0 = (unsigned long long)slot;
        }
      }
      // 3. search tiles.  Several tiles per draw when many are left (the
      // lookups are then paid once per draw), one at a time when few are, so
      // that a handful of expensive Jobs still spreads over every warp.
      if (step == kStepWait) {
        const unsigned long long pub = ld_ctr(b, kCtrJobsPublished);
        const unsigned long long njobs = pub >> 40, ptiles = pub & kTileMask;
        if (held_lo >= held_hi) {
          const unsigned long long next = ld_ctr(b, kCtrNextTile);
          if (next < ptiles) {
            unsigned long long f = kTilesPerFetch;
            while (f > 1ull && ptiles - next < 8ull * f * nwarps) f >>= 1;
            held_lo = atomicAdd(&b.counters[kCtrNextTile], f);
            held_hi = held_lo + f;
          }
        }
        if (held_lo < held_hi && held_lo < ptiles) {
          step = kStepTiles;
          a0 = held_lo;
          a1 = held_hi < ptiles ? held_hi : ptiles;
          a2 = njobs;
          held_lo = a1;
        }
      }
      // 4. done, or wait for the warps still producing work
      if (step == kStepWait && ld_ctr(b, kCtrChunksDone) >= nchunks) {
        __threadfence();
        const unsigned long long queued =
            b.fast ? ld_ctr(b, kCtrQueuePublished) : (unsigned long long)b.num_shots;
        if (ld_ctr(b, kCtrQueueHead) >= queued && ld_ctr(b, kCtrSlowDone) >= queued) {
          // every Job is published: tiles past the total will never exist
          __threadfence();
          const unsigned long long total = ld_ctr(b, kCtrJobsPublished) & kTileMask;
          if (held_lo >= total) held_lo = held_hi = 0;
          if (held_lo >= held_hi && ld_ctr(b, kCtrNextTile) >= total) step = kStepExit;
        }
      }
    }
    step = __shfl_sync(kFull, step, 0);
    if (step == kStepExit) break;
    if (step == kStepWait) {
      if (++polls > kWaitPolls) {
        if (lane == 0) atomicOr(b.status, kStatusWaitLimit);
        break;
      }
      nap(polls);
      continue;
    }
    polls = 0;
    a0 = __shfl_sync(kFull, a0, 0);
    if (step == kStepChunk) {
      classify_chunk<MLK>(b, (int)a0, A);
      cache.stage_lost();
      if (lane == 0) {
        __threadfence();
        atomicAdd(&b.counters[kCtrChunksDone], 1ull);
      }
    } else if (step == kStepShot) {
      triage_shot<MLK>(b, (int)a0, A, plans[wib]);
      cache.stage_lost();
      if (lane == 0) {
        __threadfence();
        atomicAdd(&b.counters[kCtrSlowDone], 1ull);
      }
    } else {
      a1 = __shfl_sync(kFull, a1, 0);
      a2 = __shfl_sync(kFull, a2, 0);
      search_tiles<MLK>(b, a0, a1, a2, A, cache);
    }
  }
}

}  // namespace grand
