// grand_decode.cuh -- the persistent decode kernel (sm_103a): one launch per batch.
//
// Every warp of the grid loops over whatever work the batch has left, in this
// order of preference:
//   1. classification chunks: 32 launch slots, one lane per shot; empty
//      syndromes and weight-1 matches of a one-position first iteration (a
//      syndrome equal to a solo column, found by one sketch lookup) are settled
//      there, the other shots go to the slow queue (classify_chunk);
//   2. slow-queue shots: one warp per shot, the full threshold-iteration walk
//      with the light search, publishing a Job for iterations over the light
//      budget (triage_shot);
//   3. search tiles of published Jobs (search_tiles); the warp that completes
//      a Job's last tile writes its result.
// So a heavy shot's search starts as soon as its Job is published, while other
// warps are still classifying and triaging, and triage and search share the GPU
// instead of running as two launches one after the other.
//
// Drawing: chunks by atomicAdd (a draw past the end is dropped); slow-queue
// entries by atomicAdd tickets -- a ticket past the reserved count stays with the
// warp until its entry is reserved or the batch has no more -- and each entry is
// read once it carries this launch's tag; search tiles by atomicAdd below the
// tiles of the front -- the leading Jobs all marked ready with the tag, which
// any warp advances past a ready Job -- a tile drawn past it stays with the warp
// until a Job covering it is written.  One atomic per draw, whatever the number
// of waiting warps, and no warp waits for another to publish in order.
//
// A warp that finds nothing to do sleeps and polls (bounded, kStatusWaitLimit on
// exhaustion).  It waits only for work that running warps are producing -- they
// never wait for it -- and leaves once every chunk and slow shot is finished and
// every Job's tiles are drawn.  The last warp to leave advances the launch epoch.
#pragma once

#include "grand_search.cuh"
#include "grand_triage.cuh"

namespace grand {

constexpr int kDecodeMinBlocks = 4;  // resident blocks per SM the register budget allows

// What a warp does next (decided by lane 0 from the control words, then
// broadcast, so that the whole warp takes the same path).
enum Step { kStepWait = 0, kStepChunk = 1, kStepShot = 2, kStepTiles = 3, kStepExit = 4,
            kStepHelp = 5 };

template <bool MLK>
__global__ void __launch_bounds__(kDecodeWarps * 32, kDecodeMinBlocks) decode_kernel(DevBatch b) {
  __shared__ WarpArea areas[kDecodeWarps];
  __shared__ PlanState plans[kDecodeWarps];
  __shared__ TileView views[kDecodeWarps];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  WarpArea &A = areas[wib];
  SearchCache cache;
  cache.reset();
  // this launch's tag: entries and Jobs written now carry epoch + 1 (the epoch
  // changes only once every warp of the launch has left)
  const unsigned epoch = *reinterpret_cast<volatile unsigned *>(b.epoch);
  const unsigned tag = epoch + 1u;
  const unsigned long long nchunks =
      b.fast ? (unsigned long long)((b.num_shots + kChunkShots - 1) / kChunkShots) : 0ull;
  const unsigned long long nwarps = (unsigned long long)gridDim.x * kDecodeWarps;
  constexpr unsigned long long kTileMask = (1ull << 40) - 1ull;
  unsigned long long ticket = kNone;            // lane 0: a slow-queue ticket not yet used
  unsigned long long held_lo = 0, held_hi = 0;  // lane 0: tiles drawn and not yet run
  int polls = 0;
  // profile (b.profile): lane 0 adds the time of each step to its kind's total
  unsigned long long *psum = ctr_ptr(b.counters, kCtrProfSums);
  unsigned long long *pend = ctr_ptr(b.counters, kCtrProfEnds);
  const unsigned long long t_enter = b.profile ? global_ns() : 0ull;
  unsigned long long t_busy = 0;
  if (b.profile && lane == 0) atomicMax(pend + kProfStart, ~t_enter);
  for (;;) {
    int step = kStepWait;
    unsigned long long a0 = 0, a1 = 0, a2 = 0;
    if (lane == 0) {
      // 1. classification chunks (a draw past the end is dropped)
      if (nchunks && ld_ctr(b, kCtrNextChunk) < nchunks) {
        const unsigned long long k = atomicAdd(ctr_ptr(b.counters, kCtrNextChunk), 1ull);
        if (k < nchunks) {
          step = kStepChunk;
          a0 = k;
        }
      }
      // 2. the per-shot path
      if (step == kStepWait) {
        const unsigned long long reserved =
            b.fast ? ld_ctr(b, kCtrQueueReserved) : (unsigned long long)b.num_shots;
        if (ticket == kNone && ld_ctr(b, kCtrQueueHead) < reserved)
          ticket = atomicAdd(ctr_ptr(b.counters, kCtrQueueHead), 1ull);
        if (ticket != kNone && ticket < reserved) {
          if (!b.fast) {
            step = kStepShot;
            a0 = ticket;
          } else {
            // the appending warp writes the entry right after reserving it
            volatile unsigned long long *e = b.queue + ticket;
            unsigned long long v = *e;
            for (int p = 0; (unsigned)(v >> 32) != tag; ++p) {
              if (p >= kShortPolls) break;
              nap(p);
              v = *e;
            }
            if ((unsigned)(v >> 32) == tag) {
              step = kStepShot;
              a0 = v & 0x7fffffffull;
              a1 = (v >> 31) & 1ull;  // the chunk step left the record's bits in rec_cache
            } else {
              atomicOr(b.status, kStatusWaitLimit);
            }
          }
          ticket = kNone;
        }
      }
      // 3. search tiles of the Jobs before the front.  Several tiles per draw
      // when many are left (the lookups are then paid once per draw), one at a
      // time when few are, so that a handful of expensive Jobs still spreads
      // over every warp; a draw past the front's tiles is held until they exist.
      if (step == kStepWait) {
        const unsigned long long front = ld_ctr(b, kCtrFront);
        const unsigned long long njobs = front >> 40, ptiles = front & kTileMask;
        if (held_lo >= held_hi) {
          const unsigned long long next = ld_ctr(b, kCtrNextTile);
          if (next < ptiles) {
            unsigned long long f = kTilesPerFetch;
            while (f > 1ull && ptiles - next < 2ull * f * nwarps) f >>= 1;
            held_lo = atomicAdd(ctr_ptr(b.counters, kCtrNextTile), f);
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
        const unsigned long long reserved =
            b.fast ? ld_ctr(b, kCtrQueueReserved) : (unsigned long long)b.num_shots;
        if (ld_ctr(b, kCtrSlowDone) >= reserved) {
          // every slow shot is done and its Job written (a ticket past the
          // entries will never be filled); once the front has passed every Job,
          // tiles past its total will never exist
          ticket = kNone;
          __threadfence();
          const unsigned long long front = ld_ctr(b, kCtrFront);
          if ((front >> 40) >= (ld_ctr(b, kCtrJobs) >> 40) ||
              (front >> 40) >= (unsigned long long)b.max_jobs) {
            const unsigned long long total = front & kTileMask;
            if (held_lo >= total) held_lo = held_hi = 0;
            if (held_lo >= held_hi && ld_ctr(b, kCtrNextTile) >= total) step = kStepExit;
          } else {
            step = kStepHelp;  // a publisher's advance can lose a race: help it
          }
        }
      }
    }
    step = __shfl_sync(kFull, step, 0);
    if (step == kStepExit) break;
    if (step == kStepHelp) {
      advance_front(b, tag);
      step = kStepWait;
    }
    if (step == kStepWait) {
      if (++polls > kWaitPolls) {
        if (lane == 0) atomicOr(b.status, kStatusWaitLimit);
        break;
      }
      nap(polls);
      continue;
    }
    polls = 0;
    const unsigned long long t_step = b.profile ? global_ns() : 0ull;
    a0 = __shfl_sync(kFull, a0, 0);
    if (step == kStepChunk) {
      classify_chunk<MLK>(b, (int)a0, A, tag);
      cache.stage_lost();
      if (lane == 0) {
        __threadfence();
        atomicAdd(ctr_ptr(b.counters, kCtrChunksDone), 1ull);
      }
    } else if (step == kStepShot) {
      a1 = __shfl_sync(kFull, a1, 0);
      triage_shot<MLK>(b, (int)a0, A, plans[wib], tag, a1 != 0ull);
      cache.stage_lost();
      if (lane == 0) {
        __threadfence();
        atomicAdd(ctr_ptr(b.counters, kCtrSlowDone), 1ull);
      }
    } else {
      a1 = __shfl_sync(kFull, a1, 0);
      a2 = __shfl_sync(kFull, a2, 0);
      search_tiles<MLK>(b, a0, a1, a2, A, cache, views[wib]);
    }
    if (b.profile && lane == 0) {
      const unsigned long long t = global_ns();
      const int kind = step == kStepChunk ? kProfChunk : (step == kStepShot ? kProfShot : kProfTiles);
      atomicAdd(psum + kind, t - t_step);
      atomicAdd(psum + kProfSteps, 1ull);
      atomicMax(pend + kind, t);
      if (step == kStepShot) {
        atomicMax(pend + kProfLastShotStart, t_step);
        atomicMax(pend + kProfLongestShot, t - t_step);
      } else if (step == kStepTiles) {
        atomicMax(pend + kProfLongestTiles, t - t_step);
      }
      t_busy += t - t_step;
    }
  }
  if (b.profile && lane == 0) {
    const unsigned long long t = global_ns();
    atomicAdd(psum + kProfWait, t - t_enter - t_busy);
    atomicMax(pend + kProfWait, t);
  }
  // the last warp to leave advances the epoch for the next launch
  __syncwarp();
  if (lane == 0) {
    __threadfence();
    if (atomicAdd(ctr_ptr(b.counters, kCtrWarpsDone), 1ull) + 1ull == nwarps)
      *reinterpret_cast<volatile unsigned *>(b.epoch) = tag;
  }
}

}  // namespace grand
