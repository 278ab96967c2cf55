// grand_host.h -- host-side driver of the GB300 GRAND decoder.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "grand_common.h"

namespace grand {

// Kernel launchers (grand_decode_plain.cu, grand_decode_ml.cu, grand_sample.cu).
cudaError_t launch_decode(const DevBatch &b, int grid, cudaStream_t s);
cudaError_t decode_occupancy(int *blocks_per_sm);
cudaError_t launch_sample(const DevCode &cd, const float *d_p, unsigned long long seed,
                          unsigned long long first_shot, int num_shots, int *d_records,
                          int sm_count, cudaStream_t s);

void set_error(const char *fmt, ...);

// Device-resident tables of one matrix set; shared by every call that decodes
// with the same matrices (cached by content).
struct CodeTables {
  int family = 0;
  int R = 0, m = 0, nw = 0, nwp = 0, mw = 0;
  int max_soma = 0, regular = 1, rank = 0;
  int n_logicos = 0, nlw = 0;
  uint32_t *cols = nullptr;
  int *colw = nullptr;
  uint32_t *rref = nullptr;
  int *pivrow = nullptr;
  uint32_t *lcols = nullptr;
  uint32_t *hcol = nullptr;  // column sketches (row_hash XOR over each column's rows)
  int binary = 1;             // every entry is 0 or 1
  uint32_t *solo_keys = nullptr;  // solo-column table (grand_solo.h): sketches
  int *solo_cols = nullptr;        //   and columns per slot (-1: empty)
  uint32_t solo_mask = 0;
  std::vector<int> key;  // exact content the tables were built from
  size_t bytes = 0;
  ~CodeTables();
};

// Per-call parameters that complete a CodeTables into a DevCode.
struct CallParams {
  int variant = kUniform;
  int input_kind = kInSyndromes;
  int W = 1;
  int mode = -1, thr = 0, cap = 0;
  int num_phases = 0, n_masks = 0;
  int mask_tam_upper[kMaxMasks] = {};
  int mask_order[kMaxMasks][3] = {};
  const float *d_llr = nullptr;   // device LLRs (ML)
  int rec_len = 0;                 // int32 entries per record (0: R, or m for errors)
  int packed = 0;                  // records are bit-packed words (rec_len then counts words)
};

DevCode make_devcode(const CodeTables &t, const CallParams &p);

// Growable device/host buffers and a stream, reused across calls.
struct Workspace {
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[6] = {};
  void *d_in = nullptr; size_t cap_in = 0;
  void *d_in2 = nullptr; size_t cap_in2 = 0;
  void *d_res = nullptr; size_t cap_res = 0;
  void *d_dec = nullptr; size_t cap_dec = 0;
  void *d_declog = nullptr; size_t cap_declog = 0;
  void *d_cost = nullptr; size_t cap_cost = 0;
  void *d_jobs = nullptr; size_t cap_jobs = 0;
  void *d_scratch = nullptr; size_t cap_scratch = 0;
  void *d_small = nullptr;  // counters, status
  void *d_deferred = nullptr; size_t cap_deferred = 0;  // shot_buffer_bytes: flags, slow queue
  void *d_map = nullptr; size_t cap_map = 0;
  void *d_codes = nullptr; size_t cap_codes = 0;
  void *h_codes = nullptr; size_t cap_hcodes = 0;  // pinned staging of the DevCode array
  std::vector<unsigned char> sent_codes;           // DevCode bytes now in d_codes
  unsigned *h_status = nullptr;                    // pinned: the launch status word
  void *d_llr = nullptr; size_t cap_llr = 0;
  void *d_off = nullptr; size_t cap_off = 0;
  void *d_shotcode = nullptr; size_t cap_shotcode = 0;
  ~Workspace();
};

cudaError_t ensure(void **p, size_t *cap, size_t bytes);
// As ensure, and a new allocation starts zeroed (buffers whose entries carry a
// launch tag: zero is no launch's tag).
cudaError_t ensure_zeroed(void **p, size_t *cap, size_t bytes);

// Bytes of the per-shot buffer: num_shots re-run flags (int), then, 8-byte
// aligned, num_shots slow-queue entries (u64), then, 16-byte aligned, num_shots
// record-cache rows (kRecCacheWords words each).
inline size_t shot_queue_offset(size_t num_shots) { return (4 * num_shots + 7) & ~(size_t)7; }
inline size_t shot_cache_offset(size_t num_shots) {
  return (shot_queue_offset(num_shots) + 8 * num_shots + 15) & ~(size_t)15;
}
inline size_t shot_buffer_bytes(size_t num_shots) {
  return shot_cache_offset(num_shots) + sizeof(uint32_t) * kRecCacheWords * num_shots;
}
inline unsigned long long *shot_queue(void *shot_buffer, size_t num_shots) {
  return reinterpret_cast<unsigned long long *>(static_cast<char *>(shot_buffer) +
                                                shot_queue_offset(num_shots));
}
inline uint32_t *shot_rec_cache(void *shot_buffer, size_t num_shots) {
  return reinterpret_cast<uint32_t *>(static_cast<char *>(shot_buffer) + shot_cache_offset(num_shots));
}

class Context {
 public:
  static Context *get(int *err);
  int device = 0;
  int sm_count = 0;
  int decode_bps = 1;  // resident decode-kernel blocks per SM
  unsigned long long *d_ncr = nullptr;
  int pageable_access = 0;

  std::shared_ptr<CodeTables> tables(int family, const int *H, const int *H_other,
                                     const int *L, int n, int m, int n_logicos, int *err);
  Workspace *acquire();
  void release(Workspace *w);

 private:
  std::mutex mu_;
  std::vector<std::shared_ptr<CodeTables>> cache_;  // most recent last
  std::vector<Workspace *> pool_;
  size_t cache_bytes_ = 0;
};

// One batched decode of shots that may mix several codes.
struct BatchRequest {
  int num_shots = 0;
  std::vector<DevCode> codes;        // host copies (device pointers inside)
  const int *h_in = nullptr;         // host int32 records (copied to the device)
  size_t in_ints = 0;
  const int *h_in_log = nullptr;     // DEM truth logicals in a separate array
  size_t in_log_ints = 0;
  const long long *h_off = nullptr;  // per-shot record offsets (multi-code)
  const int *h_shot_code = nullptr;
  GrandDecoderResult *h_results = nullptr;
  unsigned char *h_dec_err = nullptr;
  unsigned char *h_dec_log = nullptr;
  float *h_cost = nullptr;
  int dec_m = 0, dec_nl = 0;
};

struct BatchTiming {
  float h2d_ms = 0, reset_ms = 0, decode_ms = 0, d2h_ms = 0;
  int rounds = 0;
};

// Tunables (environment overrides, autotuner results).
struct Tuning {
  int light_max_log2 = 10;
  int tile_k = 4;
  int search_grid_mult = 0;  // CTAs per SM of the decode kernel; 0: occupancy maximum
  int fast = 1;              // settle shots 32 at a time before the per-shot path (GRAND_FAST)
  int zero_copy = 1;         // read records / write results in the caller's host memory
                             // when the device can access pageable memory (GRAND_ZERO_COPY)
  int profile = 0;           // the decode kernel records per-phase times (GRAND_PROFILE)
};
Tuning &tuning();  // process defaults (GRAND_LIGHT_LOG2, GRAND_TILE_K, GRAND_SEARCH_GRID_MULT)

// Runs the batch; returns 0 or a GRAND_ERR_* code.
int run_batch(Context *ctx, Workspace *ws, const BatchRequest &req, BatchTiming *timing,
              const Tuning *tn = nullptr);

// Enqueue one decoding launch (control-word reset, decode kernel) on s.
cudaError_t launch_pipeline(const Context *ctx, const DevBatch &b, const Tuning &tn,
                            cudaStream_t s, cudaEvent_t mid = nullptr);

// Blocks of the decode kernel per SM for a tuning (CTAs-per-SM override or the
// occupancy maximum).
int decode_blocks_per_sm(int occupancy_bps, const Tuning &tn);

}  // namespace grand
