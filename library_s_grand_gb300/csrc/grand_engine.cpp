// grand_engine.cpp -- batched mixed-code decoding (include/grand_engine.h).
#include "grand_engine.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "grand_engine_internal.h"
#include "grand_host.h"

namespace grand {
double measure_lop3_peak(int sm_count);
int read_masks_into(const char *path, CallParams *p, int W);
bool read_llr_file(const char *path, std::vector<float> &llr, int m);
}  // namespace grand

using namespace grand;

extern "C" {

int grand_engine_create(GrandEngine **engine) {
  if (!engine) return GRAND_ERR_INVALID;
  int err = 0;
  Context *ctx = Context::get(&err);
  if (!ctx) return err;
  GrandEngine *e = new GrandEngine();
  e->ctx = ctx;
  e->tn = tuning();
  *engine = e;
  return 0;
}

void grand_engine_destroy(GrandEngine *engine) { delete engine; }

int grand_engine_add_css(GrandEngine *e, const int *Hx, const int *Hz, int n, int m,
                         char type_of_error, int records_are_errors,
                         const GrandDecoderConfig *config, const char *probability_file,
                         int *code_id) {
  if (!e || !config || !Hx || !Hz) return GRAND_ERR_INVALID;
  const int *H, *Ho;
  if (type_of_error == 'x' || type_of_error == 'X') { H = Hz; Ho = Hx; }
  else if (type_of_error == 'z' || type_of_error == 'Z') { H = Hx; Ho = Hz; }
  else {
    fprintf(stderr, "Invalid type_of_error: %c. Must be 'x' or 'z'.\n", type_of_error);
    return GRAND_ERR_INVALID;
  }
  const int W = config->max_error_weight;
  CallParams p;
  p.variant = probability_file ? kProb : kUniform;
  if (!probability_file && (W <= 0 || W > 7)) {
    fprintf(stderr, "Invalid max_error_weight: %d. Must be between 1 and 7.\n", W);
    return GRAND_ERR_INVALID;
  }
  if (probability_file) {
    int rc = read_masks_into(probability_file, &p, W);
    if (rc) return rc;
  }
  if (n <= 0 || m <= 0 || n > kMaxRows || m > kMaxCols) return GRAND_ERR_LIMIT;
  int err = 0;
  auto tab = e->ctx->tables(kCss, H, Ho, nullptr, n, m, 0, &err);
  if (!tab) return err;
  p.input_kind = records_are_errors ? kInErrors : kInSyndromes;
  p.W = W;
  p.mode = config->mode_of_search;
  p.thr = config->threshold_for_hybrid;
  p.cap = config->max_size_active_positions;
  std::lock_guard<std::mutex> lk(e->mu);
  e->codes.push_back(make_devcode(*tab, p));
  e->tabs.push_back(tab);
  e->llr.push_back(nullptr);
  e->rec_len.push_back(records_are_errors ? m : n);
  e->dirty = true;
  if (code_id) *code_id = (int)e->codes.size() - 1;
  return 0;
}

int grand_engine_add_dem(GrandEngine *e, const int *H, const int *L, int n, int m, int nl,
                         const GrandDecoderConfig *config, int variant, const char *file,
                         int *code_id) {
  if (!e || !config || !H || (nl > 0 && !L) || nl < 0) return GRAND_ERR_INVALID;
  const int W = config->max_error_weight;
  if (W <= 0 || W > 7) {
    fprintf(stderr, "Invalid max_error_weight: %d. Must be between 1 and 7.\n", W);
    return GRAND_ERR_INVALID;
  }
  if (variant < 0 || variant > 2) return GRAND_ERR_INVALID;
  CallParams p;
  p.variant = variant;
  std::vector<float> llr;
  if (variant == kMl && !read_llr_file(file, llr, m)) return GRAND_ERR_INVALID;
  if (variant == kProb) {
    int rc = read_masks_into(file, &p, W);
    if (rc) return rc;
  }
  if (n <= 0 || m <= 0 || n > kMaxRows || m > kMaxCols || nl > kMaxLogicals) return GRAND_ERR_LIMIT;
  int err = 0;
  auto tab = e->ctx->tables(kDem, H, nullptr, L, n, m, nl, &err);
  if (!tab) return err;
  float *d_llr = nullptr;
  if (variant == kMl) {
    if (cudaMalloc(&d_llr, sizeof(float) * m) != cudaSuccess ||
        cudaMemcpy(d_llr, llr.data(), sizeof(float) * m, cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("grand: LLR upload failed");
      cudaFree(d_llr);
      return GRAND_ERR_CUDA;
    }
    p.d_llr = d_llr;
  }
  p.input_kind = kInDetectors;
  p.rec_len = n + nl;  // detectors followed by the true logical flips
  p.W = W;
  p.mode = config->mode_of_search;
  p.thr = config->threshold_for_hybrid;
  p.cap = config->max_size_active_positions;
  std::lock_guard<std::mutex> lk(e->mu);
  e->codes.push_back(make_devcode(*tab, p));
  e->tabs.push_back(tab);
  e->llr.push_back(d_llr);
  e->rec_len.push_back(n + nl);
  e->dirty = true;
  if (code_id) *code_id = (int)e->codes.size() - 1;
  return 0;
}

int grand_engine_sample(GrandEngine *e, int code_id, const float *d_p, unsigned long long seed,
                        unsigned long long first_shot, int num_shots, int *d_records,
                        void *stream) {
  if (!e || num_shots < 0 || !d_p || (num_shots > 0 && !d_records)) return GRAND_ERR_INVALID;
  DevCode cd;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    if (code_id < 0 || code_id >= (int)e->codes.size()) return GRAND_ERR_INVALID;
    cd = e->codes[code_id];
  }
  cudaError_t r = launch_sample(cd, d_p, seed, first_shot, num_shots, d_records,
                                e->ctx->sm_count, (cudaStream_t)stream);
  if (r != cudaSuccess) {
    set_error("grand_engine_sample: %s", cudaGetErrorString(r));
    return GRAND_ERR_CUDA;
  }
  return 0;
}

int grand_engine_record_len(GrandEngine *e, int code_id) {
  if (!e || code_id < 0 || code_id >= (int)e->rec_len.size()) return GRAND_ERR_INVALID;
  return e->rec_len[code_id];
}

int grand_engine_set_tuning(GrandEngine *e, int light_log2, int tile_k, int search_ctas_per_sm) {
  if (!e || light_log2 < 0 || light_log2 > 40 || tile_k < 1 || tile_k > 64 ||
      search_ctas_per_sm < 0)
    return GRAND_ERR_INVALID;
  std::lock_guard<std::mutex> lk(e->mu);
  e->tn.light_max_log2 = light_log2;
  e->tn.tile_k = tile_k;
  e->tn.search_grid_mult = search_ctas_per_sm;
  for (auto &g : e->graphs) cudaGraphExecDestroy(g.second);
  e->graphs.clear();
  return 0;
}

int grand_engine_decode(GrandEngine *e, int num_shots, const int *shot_code, const int *records,
                        GrandDecoderResult *results, const GrandDecodeOutputs *out) {
  if (!e || num_shots < 0) return GRAND_ERR_INVALID;
  if (num_shots == 0) return 0;
  if (!records || !results || e->codes.empty()) return GRAND_ERR_INVALID;
  std::vector<long long> off;
  long long tot = 0;
  bool single = true;
  if (shot_code) {
    off.resize(num_shots);
    for (int i = 0; i < num_shots; ++i) {
      const int c = shot_code[i];
      if (c < 0 || c >= (int)e->codes.size()) return GRAND_ERR_INVALID;
      if (c != 0) single = false;
      off[i] = tot;
      tot += e->rec_len[c];
    }
  } else {
    tot = (long long)num_shots * e->rec_len[0];
  }
  Workspace *ws = e->ctx->acquire();
  if (!ws) return GRAND_ERR_CUDA;
  BatchRequest req;
  req.num_shots = num_shots;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    req.codes = e->codes;
  }
  req.h_in = records;
  req.in_ints = (size_t)tot;
  req.h_off = (shot_code && !single) ? off.data() : nullptr;
  req.h_shot_code = (shot_code && !single) ? shot_code : nullptr;
  req.h_results = results;
  if (out && out->decoded_errors) {
    // decoded patterns need one common width: only for single-code batches
    if (!single && shot_code) {
      e->ctx->release(ws);
      return GRAND_ERR_INVALID;
    }
    req.h_dec_err = out->decoded_errors;
    req.dec_m = req.codes[0].m;
  }
  if (out && out->decoded_logicals && (single || !shot_code)) {
    req.h_dec_log = out->decoded_logicals;
    req.dec_nl = req.codes[0].n_logicos;
  }
  if (out && out->ml_cost) req.h_cost = out->ml_cost;
  BatchTiming t;
  int rc = run_batch(e->ctx, ws, req, &t, &e->tn);
  {
    std::lock_guard<std::mutex> lk(e->mu);
    e->last = t;
  }
  e->ctx->release(ws);
  return rc;
}

int grand_engine_decode_device(GrandEngine *e, int num_shots, const int *d_shot_code,
                               const long long *d_offsets, const int *d_records,
                               GrandDecoderResult *d_results, void *stream, int use_graph) {
  if (!e || num_shots < 0) return GRAND_ERR_INVALID;
  if (num_shots == 0) return 0;
  if (!d_records || !d_results || e->codes.empty()) return GRAND_ERR_INVALID;
  std::lock_guard<std::mutex> lk(e->mu);
  int rc = upload_codes(e);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  EngineSlot *&slot = e->slots[stream];
  if (!slot) {
    slot = new EngineSlot();
    for (auto &ev : slot->ev) cudaEventCreate(&ev);
  }
  const int max_jobs = num_shots;
  const size_t scratch_words = 64ull << 20;
  cudaError_t r = ensure_zeroed(&slot->d_jobs, &slot->cap_jobs, sizeof(Job) * (size_t)max_jobs);
  if (r == cudaSuccess) r = ensure(&slot->d_scratch, &slot->cap_scratch, scratch_words * 4);
  if (r == cudaSuccess) r = ensure_zeroed(&slot->d_small, &slot->cap_small, kCtlAllocBytes);
  if (r == cudaSuccess)
    r = ensure_zeroed(&slot->d_deferred, &slot->cap_deferred, shot_buffer_bytes(num_shots));
  if (r != cudaSuccess) {
    set_error("grand: device workspace allocation failed (%s)", cudaGetErrorString(r));
    return GRAND_ERR_CUDA;
  }
  DevBatch b;
  memset(&b, 0, sizeof(b));
  b.num_shots = num_shots;
  b.num_codes = (int)e->codes.size();
  b.codes = (const DevCode *)e->d_codes;
  b.in = d_records;
  b.in_off = d_offsets;
  b.shot_code = d_shot_code;
  b.results = d_results;
  b.ncr = e->ctx->d_ncr;
  b.jobs = (Job *)slot->d_jobs;
  b.max_jobs = max_jobs;
  b.counters = (unsigned long long *)slot->d_small;
  b.status = (unsigned *)((char *)slot->d_small + kStatusByteOffset);
  b.scratch = (uint32_t *)slot->d_scratch;
  b.scratch_words = scratch_words;
  b.deferred = (int *)slot->d_deferred;
  b.queue = shot_queue(slot->d_deferred, num_shots);
  // records in device memory: the per-shot path reads them again from L2 (the
  // record cache pays off only for records read in place from host memory)
  b.rec_cache = nullptr;
  b.epoch = (unsigned *)((char *)slot->d_small + kCtlBytes);
  b.fast = e->tn.fast;
  b.profile = e->tn.profile;
  b.light_max_log2 = e->tn.light_max_log2;
  b.tile_k = e->tn.tile_k;
  for (const DevCode &c : e->codes) b.has_ml |= c.variant == kMl;
  if (!use_graph) {
    cudaEventRecord(slot->ev[0], s);
    r = launch_pipeline(e->ctx, b, e->tn, s, slot->ev[1]);
    cudaEventRecord(slot->ev[2], s);
    slot->timed = true;
  } else {
    slot->timed = false;
    GraphKey key{num_shots, d_shot_code, d_offsets, d_records, d_results};
    auto it = e->graphs.find(key);
    cudaGraphExec_t exec = nullptr;
    if (it != e->graphs.end() && it->first.a == key.a) {
      exec = it->second;
    }
    if (!exec) {
      cudaStream_t cs;
      r = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
      if (r == cudaSuccess) r = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      if (r == cudaSuccess) {
        cudaError_t lr = launch_pipeline(e->ctx, b, e->tn, cs);
        cudaGraph_t g = nullptr;
        r = cudaStreamEndCapture(cs, &g);
        if (lr != cudaSuccess) r = lr;
        if (r == cudaSuccess) r = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
      }
      cudaStreamDestroy(cs);
      if (r == cudaSuccess) e->graphs[key] = exec;
    }
    if (r == cudaSuccess) r = cudaGraphLaunch(exec, s);
  }
  if (r != cudaSuccess) {
    set_error("grand: device decode launch failed (%s)", cudaGetErrorString(r));
    return GRAND_ERR_CUDA;
  }
  return 0;
}

int grand_engine_sync_status(GrandEngine *e, void *stream) {
  if (!e) return GRAND_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t r = cudaStreamSynchronize(s);
  if (r != cudaSuccess) {
    set_error("grand: stream synchronize failed (%s)", cudaGetErrorString(r));
    return GRAND_ERR_CUDA;
  }
  unsigned st = 0;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    auto it = e->slots.find(stream);
    if (it == e->slots.end()) return 0;
    r = cudaMemcpy(&st, (char *)it->second->d_small + kStatusByteOffset, sizeof(unsigned),
                   cudaMemcpyDeviceToHost);
  }
  if (r != cudaSuccess) return GRAND_ERR_CUDA;
  if (st & (kStatusJobOverflow | kStatusScratchOverflow)) {
    set_error("grand: device decode ran out of job table or scratch space; use grand_engine_decode");
    return GRAND_ERR_LIMIT;
  }
  if (st & kStatusTamLimit) {
    set_error("grand: an active-position set exceeded GRAND_MAX_TAM=%d", kMaxTam);
    return GRAND_ERR_LIMIT;
  }
  if (st & kStatusCasLimit) return GRAND_ERR_CUDA;
  return 0;
}

int grand_engine_launch_stats(GrandEngine *e, void *stream, long long *out) {
  if (!e || !out) return GRAND_ERR_INVALID;
  std::lock_guard<std::mutex> lk(e->mu);
  auto it = e->slots.find(stream);
  if (it == e->slots.end()) return GRAND_ERR_INVALID;
  std::vector<unsigned long long> c(kCtlBytes / 8);
  if (cudaMemcpy(c.data(), it->second->d_small, kCtlBytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    return GRAND_ERR_CUDA;
  out[0] = (long long)c[kCtrSettled * kCtrStride];
  out[1] = (long long)c[kCtrSlowDone * kCtrStride];
  out[2] = (long long)(c[kCtrJobs * kCtrStride] >> 40);
  out[3] = (long long)(c[kCtrJobs * kCtrStride] & ((1ull << 40) - 1ull));
  out[4] = (long long)c[kCtrScratchTop * kCtrStride];
  // phase profile (GRAND_PROFILE=1): times in ns from the first warp's start
  const unsigned long long *pa = c.data() + kCtrProfSums * kCtrStride;
  const unsigned long long *pb = c.data() + kCtrProfEnds * kCtrStride;
  const unsigned long long t0 = ~pb[kProfStart];
  for (int i = 0; i < kProfKinds; ++i) {
    out[5 + i] = (long long)pa[i];                                        // warp-ns spent
    out[5 + kProfKinds + i] = pb[i] ? (long long)(pb[i] - t0) : -1;       // last end
  }
  out[5 + 2 * kProfKinds] = (long long)pa[kProfSteps];
  for (int i = 0; i < kProfDetails; ++i) out[14 + i] = (long long)pa[kProfChunkRead + i];
  const unsigned long long *pm = c.data() + kCtrProfMore * kCtrStride;
  for (int i = 0; i < kProfPubWords; ++i) out[24 + i] = (long long)pm[i];
  out[28] = pb[kProfLastShotStart] ? (long long)(pb[kProfLastShotStart] - t0) : -1;
  out[29] = (long long)pb[kProfLongestShot];
  out[30] = (long long)pb[kProfLongestTiles];
  return 0;
}

int grand_engine_batch_times(GrandEngine *e, float *h2d_ms, float *reset_ms, float *decode_ms,
                             float *d2h_ms) {
  if (!e) return GRAND_ERR_INVALID;
  std::lock_guard<std::mutex> lk(e->mu);
  if (h2d_ms) *h2d_ms = e->last.h2d_ms;
  if (reset_ms) *reset_ms = e->last.reset_ms;
  if (decode_ms) *decode_ms = e->last.decode_ms;
  if (d2h_ms) *d2h_ms = e->last.d2h_ms;
  return 0;
}

int grand_engine_kernel_times(GrandEngine *e, void *stream, float *reset_ms, float *decode_ms) {
  if (!e) return GRAND_ERR_INVALID;
  std::lock_guard<std::mutex> lk(e->mu);
  auto it = e->slots.find(stream);
  if (it == e->slots.end() || !it->second->timed) return GRAND_ERR_INVALID;
  float a = 0, b = 0;
  if (cudaEventElapsedTime(&a, it->second->ev[0], it->second->ev[1]) != cudaSuccess ||
      cudaEventElapsedTime(&b, it->second->ev[1], it->second->ev[2]) != cudaSuccess)
    return GRAND_ERR_CUDA;
  if (reset_ms) *reset_ms = a;
  if (decode_ms) *decode_ms = b;
  return 0;
}

int grand_device_info(char *buf, int len) {
  int err = 0;
  Context *ctx = Context::get(&err);
  if (!ctx) return err;
  if (!buf || len <= 0) return GRAND_ERR_INVALID;
  return snprintf(buf, (size_t)len,
                  "device=%d sms=%d decode_ctas_per_sm=%d pageable_memory_access=%d",
                  ctx->device, ctx->sm_count, ctx->decode_bps,
                  ctx->pageable_access);
}

double grand_measure_int_peak(void) {
  int err = 0;
  Context *ctx = Context::get(&err);
  if (!ctx) return -1.0;
  return measure_lop3_peak(ctx->sm_count);
}

int grand_engine_decode_plain(GrandEngine *e, int num_shots, const int *shot_code,
                              const int *records, GrandDecoderResult *results) {
  if (!e || num_shots < 0) return GRAND_ERR_INVALID;
  if (num_shots == 0) return 0;
  if (!records || !results || e->codes.empty()) return GRAND_ERR_INVALID;
  Workspace *ws = e->ctx->acquire();
  if (!ws) return GRAND_ERR_CUDA;
  std::vector<DevCode> codes;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    codes = e->codes;
  }
  long long off = 0;
  int rc = 0;
  for (int i = 0; i < num_shots && rc == 0; ++i) {
    const int c = shot_code ? shot_code[i] : 0;
    if (c < 0 || c >= (int)codes.size()) {
      rc = GRAND_ERR_INVALID;
      break;
    }
    BatchRequest req;
    req.num_shots = 1;
    req.codes.push_back(codes[c]);
    req.h_in = records + off;
    req.in_ints = (size_t)e->rec_len[c];
    req.h_results = results + i;
    rc = run_batch(e->ctx, ws, req, nullptr, &e->tn);
    off += e->rec_len[c];
  }
  e->ctx->release(ws);
  return rc;
}

}  // extern "C"
