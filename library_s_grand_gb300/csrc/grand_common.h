// grand_common.h -- definitions shared by the host driver and the sm_103a kernels.
//
// Layout in HBM (all device-resident, built once per code and cached):
//   cols   : m columns of H, each packed LSB-first into nwp uint32 words
//            (nw = ceil(R/32) meaningful words, padded to nwp = 1,2,4,8 or 4k
//            so a column is one vector load); bit r of column c = H[r][c].
//   rows   : R rows of H packed into mw = ceil(m/32) words (syndrome of a
//            supplied error pattern, CSS family).
//   rref   : reduced row echelon form of the other CSS matrix, rank x mw words,
//            with its pivot columns (degeneracy test).
//   lcols  : m rows of L_dem packed into nlw words (DEM logical flips).
//   llr    : m FP32 LLRs (ML variant).
//   ncr    : C(n, k) for n <= GRAND_MAX_TAM, k <= 6, as uint64.
//   hcol   : m 32-bit column sketches, hcol[c] = h(column c) with the GF(2)-linear
//            hash h(v) = XOR of row_hash(r) over the set rows r of v.
#pragma once

#include <stdint.h>

#include "grand_decoder.h"

#ifdef __CUDACC__
#define GRAND_HD __host__ __device__
#else
#define GRAND_HD
#endif

namespace grand {

// Hash of one check row for the column sketches: MurmurHash3's 32-bit finalizer
// (fmix32) of the row index.  The sketch of a vector is the XOR of its rows'
// hashes, so it is linear over GF(2): the sketch of (syndrome XOR the columns of
// a candidate) is the XOR of their sketches, and a candidate that matches has
// sketch 0.  fmix32 is a bijection, so no two rows share a hash.
GRAND_HD inline uint32_t row_hash(int r) {
  uint32_t x = (uint32_t)r * 0x9E3779B9u + 0x7F4A7C15u;
  x ^= x >> 16;
  x *= 0x85EBCA6Bu;
  x ^= x >> 13;
  x *= 0xC2B2AE35u;
  x ^= x >> 16;
  return x;
}

constexpr int kMaxW = GRAND_MAX_W;        // searched weights 1..6
constexpr int kMaxTam = GRAND_MAX_TAM;    // largest active set searched
constexpr int kMaxRows = 1024;            // R <= 1024  -> nw <= 32
constexpr int kMaxCols = 4096;            // m <= 4096  -> mw <= 128
constexpr int kMaxLogicals = 1024;
constexpr int kMaxMasks = 20;             // upstream GRAND_MAX_MASKS (grand_decoder.cu:11)
constexpr int kMaxIters = 3;              // upstream threshold iterations (grand_decoder.cu:1284)
constexpr int kMaxSegsPerIter = 15;       // 3 phases x 5 weights
constexpr int kMaxSegs = kMaxIters * kMaxSegsPerIter;

enum Family { kCss = 0, kDem = 1 };
enum Variant { kUniform = 0, kProb = 1, kMl = 2 };
enum InputKind { kInSyndromes = 0, kInErrors = 1, kInDetectors = 2 };
enum Branch { kBranchGpu = 0, kBranchCpu = 1 };

// Status bits raised by the kernels (read back after every launch).
enum StatusBits : unsigned {
  kStatusTamLimit = 1u << 0,      // an active set exceeded GRAND_MAX_TAM
  kStatusJobOverflow = 1u << 1,   // heavy-job table full: shot deferred
  kStatusScratchOverflow = 1u << 2,
  kStatusCasLimit = 1u << 3,      // bounded CAS loop gave up (never expected)
  kStatusWaitLimit = 1u << 4,     // a bounded wait for another warp gave up (never expected)
};

// Batch control block (DevBatch::counters, kCtlBytes zeroed before every launch):
// each control word sits alone on a 128-byte line (word k at counters[k * kCtrStride]),
// so that warps polling or drawing from one do not queue behind traffic on another;
// the status word has the last line.
constexpr int kCtrStride = 16;           // u64 per line
constexpr int kCtlBytes = 2048;          // 15 control lines + the status line
constexpr int kStatusByteOffset = 1920;  // DevBatch::status within the block
// The workspace's launch epoch (DevBatch::epoch) follows the block on a line of its
// own and is not zeroed: the last warp of a launch advances it.  Slow-queue
// entries and Jobs carry the epoch of the launch that wrote them, so a reader can
// tell an entry written in this launch from one left by an earlier launch without
// clearing the arrays between launches (they are zeroed once, when allocated).
constexpr int kCtlAllocBytes = kCtlBytes + 128;
enum Counter {
  kCtrJobs = 0,           // (Jobs << 40) | tiles reserved, in slot order
  kCtrFront = 1,          // (Jobs << 40) | tiles of the leading Jobs that are all written
  kCtrNextTile = 12,      // next search tile to draw (tiles numbered over all Jobs)
  kCtrScratchTop = 2,     // words of the scratch arena in use
  kCtrNextChunk = 3,      // next 32-slot classification chunk to draw
  kCtrQueueReserved = 4,  // slow-queue entries reserved (each is written right after)
  kCtrQueueHead = 5,      // slow-queue tickets drawn (a ticket past the reserved
                          // count is held until its entry exists or the batch ends)
  kCtrChunksDone = 6,     // classification chunks finished
  kCtrSlowDone = 7,       // per-shot-path shots finished (their Jobs published)
  kCtrWarpsDone = 8,      // warps that left the kernel (the last advances the epoch)
  kCtrSettled = 10,       // shots settled by classification (statistics)
  kCtrProfSums = 11,      // profile (DevBatch::profile): warp-ns per kind of work, steps
  kCtrProfEnds = 13,      // profile: latest end per kind of work, ~(first warp start)
  kCtrProfMore = 14,      // profile: the Job publication's steps (kProfPub*)
};
// Words of the two profile lines: kinds of work in the order of the decode
// kernel's steps (classification chunks, per-shot path, search tiles, waiting),
// then the number of steps (sums line) and the complemented start (ends line).
// Sums words 6.. split the work further: classification (records read and
// syndromes formed; one-position test; results and queue), per-shot path (record
// packed; flagged-check counts; planning and light search; Job staging and
// publication; result written) and search (Job / block lookup and staging; a
// completed Job's result).
// The ends line also keeps the latest start of a per-shot-path shot, the longest
// per-shot-path shot and the longest tile draw (durations in ns).
enum ProfWord { kProfChunk = 0, kProfShot = 1, kProfTiles = 2, kProfWait = 3, kProfKinds = 4,
                kProfSteps = 4, kProfStart = 5, kProfLastShotStart = 6, kProfLongestShot = 7,
                kProfLongestTiles = 8,
                kProfChunkRead = 6, kProfChunkTest = 7, kProfChunkWrite = 8,
                kProfShotPack = 9, kProfShotCounts = 10, kProfShotLight = 11,
                kProfShotPublish = 12, kProfShotFinish = 13,
                kProfTileSetup = 14, kProfTileFinish = 15, kProfDetails = 10 };
// Words of the kCtrProfMore line: a Job's publication split into its scratch
// and slot reservations, the staging of its iterations, the Job written, and
// the fences and front advance that make it searchable.
enum ProfPubWord { kProfPubReserve = 0, kProfPubStage = 1, kProfPubWrite = 2, kProfPubReady = 3,
                   kProfPubWords = 4 };

// Words per shot of DevBatch::rec_cache: a record's bits as the chunk step read
// them (error words, or syndrome / detector words then DEM logical words).
constexpr int kRecCacheWords = 16;

// Address of control word k.
GRAND_HD inline unsigned long long *ctr_ptr(unsigned long long *counters, int k) {
  return counters + k * kCtrStride;
}

// Immutable per-code tables plus the per-call search parameters.
struct DevCode {
  int R, m, nw, nwp, mw;
  int max_soma, regular;
  int family, variant, input_kind;
  int W, Wc;                 // configured weight and min(W, 6)
  int mode, thr, cap;        // mode_of_search, threshold_for_hybrid, max_size_active_positions
  int num_phases, n_masks;
  int mask_tam_upper[kMaxMasks];
  int mask_order[kMaxMasks][3];
  int n_logicos, nlw;
  int rank;                  // rank of RREF(H_other), CSS
  int rec_len;               // int32 entries (or packed words) per shot record
  int packed;                // 1: records are bit-packed uint32 words (bit i of word k =
                             // entry 32k + i): ceil(R/32) syndrome / detector words (then
                             // ceil(n_logicos/32) logical words for DEM), ceil(m/32) error words
  const uint32_t *cols;      // m * nwp
  const int *colw;           // m
  const uint32_t *rows;      // R * mw (CSS, errors input)
  const uint32_t *rref;      // rank * mw
  const int *pivrow;         // m: RREF row whose pivot is column c, or -1
  const uint32_t *lcols;     // m * nlw
  const float *llr;          // m
  const uint32_t *hcol;      // m column sketches
  int binary;                // every entry of H is 0 or 1 (column weights are popcounts)
  const uint32_t *solo_keys; // solo columns (nonzero, containing no other nonzero column)
  const int *solo_cols;      //   by sketch: open addressing, column -1 = empty slot
  uint32_t solo_mask;        //   (solo_cols nullptr: no table)
};

// One searched weight block of one threshold iteration.
struct Seg {
  int iter;                  // index into Job::it
  int w;                     // weight
  int dup;                   // weight already listed earlier in this iteration: never matches first
  int phase;                 // phase position k (prob) or 0
  unsigned long long base;   // first global candidate index of this block within the shot
  unsigned long long count;  // C(tam, w)
  unsigned long long nprefix;// number of (w-1)-prefixes, C(tam-1, w-1)
  unsigned long long ntiles; // light search: colex tiles of 32 lanes x K prefixes (w <= 2)
  unsigned long long tile_lo;// first lookup tile of this block within the Job
  unsigned long long njt;    // lookup tiles the Job's searchers run for this block (0: none)
  int K;                     // light search: prefixes per lane in a tile
  int runs;                  // light search: 1 run tiles (w >= 3), 0 colex tiles (w <= 2)
};

struct IterInfo {
  int it;                    // upstream iteration counter value (1-based)
  int tam;
  int branch;                // kBranchGpu / kBranchCpu bookkeeping
  int seg_lo, seg_hi;
  int src;                   // which threshold mask the active set comes from
  unsigned long long total;  // full candidate count of the iteration
  unsigned long long base;   // first global index of the iteration
  unsigned long long phase_end[3]; // prob: cumulative full count through phase k
  float prefix[kMaxW + 1];   // ML: FP32 sums of the w smallest LLRs
  uint32_t *cols;            // tam * nwp staged columns (scratch)
  uint32_t *hcols;           // tam staged column sketches (scratch)
  int *pos;                  // tam H-column indices (sorted by LLR for ML)
  float *llr;                // tam LLRs in the same order (ML)
};

// A shot whose search space is too large for one warp: searched by every warp
// of the launch, tile by tile.  Aligned to (and a multiple of) 128 bytes, so no
// cache line holds parts of two Jobs: a Job is written once before it is
// published, and a line another SM cached from a published Job never carries
// bytes of a Job published later.  (The ML minima, updated with 128-bit
// compare-and-swap, need 16-byte alignment.)
struct alignas(128) Job {
  int shot, code;
  int n_it;
  int nseg;
  int final_iteration, final_tam; // outcome fields if nothing is found
  int it_lo;                      // first iteration of the Job (searched in lookup tiles)
  unsigned long long tile_base;   // first tile of the Job (tiles numbered over all Jobs)
  unsigned long long ntiles;
  unsigned ready;                 // launch tag (epoch + 1) once the Job is fully written
  unsigned long long best;        // lowest matching global index (atomicMin)
  unsigned long long tiles_done;
  int original_weight;
  int failed;                     // an active set exceeded the kernel limits
  uint32_t hs;                    // sketch of the syndrome
  unsigned long long t_start;     // %globaltimer (ns) when the shot's triage began,
  unsigned long long t_counts;    //   and when its flagged-check counts were done
  uint32_t *ebits;                // mw words: supplied error (CSS) / truth logicals (DEM)
  uint32_t sw[kMaxRows / 32];     // syndrome bits
  IterInfo it[kMaxIters];
  Seg seg[kMaxSegs];
  alignas(16) unsigned long long mlkey[kMaxIters][kMaxW + 1][2]; // ML: {cost key, lex rank} minima
};
static_assert(sizeof(Job) % 128 == 0, "Job must fill whole 128-byte lines in arrays");

// Everything one batched launch needs.
struct DevBatch {
  int num_shots;
  int num_codes;
  const DevCode *codes;          // device array
  const int *in;                 // int32 shot records
  const long long *in_off;       // per-shot offset into in (nullptr: shot * rec_len of code 0)
  const int *in_log;             // DEM truth logicals, n_logicos per shot (nullptr: they
                                 // follow the detector entries inside the record)
  const int *shot_code;          // per-shot code index (nullptr: code 0)
  const int *shot_map;           // launch slot -> shot index (nullptr: identity)
  GrandDecoderResult *results;
  unsigned char *dec_err;        // num_shots x m (single-code calls) or nullptr
  unsigned char *dec_log;        // num_shots x n_logicos or nullptr
  float *ml_cost;                // num_shots or nullptr
  const unsigned long long *ncr; // (kMaxTam + 1) x (kMaxW + 1)
  Job *jobs;
  int max_jobs;
  unsigned long long *counters;  // control words (enum Counter)
  uint32_t *scratch;
  unsigned long long scratch_words;
  unsigned *status;
  int *deferred;                 // per shot: 1 if the shot must be re-run
  uint32_t *rec_cache;           // num_shots x kRecCacheWords: a slow-queue shot's record as
                                 // packed words, written by the chunk step (nullptr: none; set
                                 // when records are read in place from host memory)
  unsigned long long *queue;     // num_shots entries: ((epoch + 1) << 32) | launch slot of a
                                 // shot that needs the per-shot path
  unsigned *epoch;               // the workspace's launch epoch (kCtlAllocBytes layout)
  int profile;                   // 1: record per-phase times in the profile lines
  int fast;                      // 1: settle shots 32 at a time first (empty syndromes, and
                                 //    weight-1 matches of a one-position first iteration)
  int light_max_log2;            // light-path budget (candidates, log2)
  int tile_k;                    // prefixes per lane per colex tile (weights <= 2)
  int has_ml;                    // some code of the batch is ML: launch the kernels' ML builds
};

}  // namespace grand
