// grand_server.cpp -- continuous-batching decode server (include/grand_server.h).
//
// One dispatcher thread owns the slots.  Each slot has a CUDA stream, pinned
// host staging, device buffers sized at creation, and its own job table and
// scratch arena, so slots run independently on the GPU.  The dispatcher:
//   * reaps slots whose work finished (a host callback on the slot's stream
//     wakes it), copies each request's results out and wakes its waiters;
//   * fills every free slot with the oldest waiting requests that fit
//     (max_shots_per_batch, and the search scratch expected from the recent
//     batches' scratch per shot within 3/4 of the slot's arena), packs their
//     offsets (records are read in place where the GPU can reach pageable
//     memory, copied through pinned staging otherwise), and enqueues copy-in, counter
//     reset, the decode kernel and copy-out on the slot's stream; each slot's
//     persistent kernel gets 1/slots of the resident blocks, so all slots'
//     kernels are on the GPU at once.
// Requests arriving while slots run simply wait for the next free slot, so the
// GPU always has up to `slots` micro-batches in flight.
#include "grand_server.h"

#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "grand_engine_internal.h"
#include "grand_host.h"

using namespace grand;
using Clock = std::chrono::steady_clock;

namespace {

struct SrvRequest {
  unsigned long long id = 0;
  int n = 0;
  const int *shot_code = nullptr;
  const int *records = nullptr;
  GrandDecoderResult *results = nullptr;
  Clock::time_point t_submit, t_done;
  bool done = false;
  int rc = 0;
};

struct SrvSlot {
  cudaStream_t s = nullptr;
  // pinned host staging
  void *h_block = nullptr;
  int *h_rec = nullptr;
  const int *in_base = nullptr;  // records read in place from here (nullptr: staged in h_rec)
  long long *h_off = nullptr;
  int *h_code = nullptr;
  GrandDecoderResult *h_res = nullptr;
  unsigned *h_status = nullptr;
  unsigned long long *h_top = nullptr;  // scratch words the last batch staged
  // device buffers
  void *d_block = nullptr;
  int *d_rec = nullptr;
  long long *d_off = nullptr;
  int *d_code = nullptr;
  GrandDecoderResult *d_res = nullptr;
  Job *d_jobs = nullptr;
  uint32_t *d_scratch = nullptr;
  unsigned long long *d_small = nullptr;
  int *d_deferred = nullptr;
  std::vector<std::shared_ptr<SrvRequest>> reqs;
  std::vector<int> first;  // first shot of each request in the batch
  int nshots = 0;
  bool busy = false;
  std::atomic<int> completed{0};
  struct GrandServer *owner = nullptr;
};

constexpr unsigned long long kSrvArenaWords = 4ull << 20;  // 16 MiB of staged search data per slot

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

struct GrandServer {
  GrandEngine *eng = nullptr;
  int max_shots = 0;
  int max_rec = 0;  // largest record length over the engine's codes
  std::vector<SrvSlot *> slots;
  size_t dev_bytes = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<SrvRequest>> queue;
  std::unordered_map<unsigned long long, std::shared_ptr<SrvRequest>> live;
  unsigned long long next_id = 1;
  // Search scratch staged per shot on recent batches (moving average): the
  // dispatcher admits requests into a micro-batch while the expected scratch
  // stays within the arena's headroom.
  double scratch_per_shot = 0.0;
  bool stop = false;
  std::thread th;
};

namespace {

void CUDART_CB slot_done(void *p) {
  SrvSlot *sl = static_cast<SrvSlot *>(p);
  sl->completed.store(1);
  GrandServer *S = sl->owner;
  std::lock_guard<std::mutex> lk(S->mu);
  S->cv_work.notify_one();
}

// Records, offsets, codes of the queued requests into the slot, then launch.
// Called without the server lock; the slot is owned by the dispatcher.
cudaError_t start_slot(GrandServer *S, SrvSlot *sl) {
  GrandEngine *e = S->eng;
  // Where the GPU can read pageable host memory (NVLink-C2C on GB300) the kernel
  // reads every request's records in place: offsets are taken from the lowest
  // record address of the batch, and no record is copied on the host or to the
  // device.  Otherwise the records are packed into the slot's pinned staging
  // and copied in.
  const bool in_place = e->tn.zero_copy && e->ctx->pageable_access;
  const int *base = nullptr;
  if (in_place)
    for (const auto &r : sl->reqs)
      if (!base || reinterpret_cast<uintptr_t>(r->records) < reinterpret_cast<uintptr_t>(base))
        base = r->records;
  long long off = 0;
  int shot = 0;
  for (size_t i = 0; i < sl->reqs.size(); ++i) {
    const SrvRequest &r = *sl->reqs[i];
    sl->first[i] = shot;
    const long long at =
        in_place ? (long long)((reinterpret_cast<uintptr_t>(r.records) -
                                reinterpret_cast<uintptr_t>(base)) / sizeof(int))
                 : off;
    long long req_ints = 0;
    for (int j = 0; j < r.n; ++j) {
      const int c = r.shot_code ? r.shot_code[j] : 0;
      sl->h_off[shot + j] = at + req_ints;
      sl->h_code[shot + j] = c;
      req_ints += e->rec_len[c];
    }
    if (!in_place) memcpy(sl->h_rec + off, r.records, sizeof(int) * (size_t)req_ints);
    off += req_ints;
    shot += r.n;
  }
  sl->nshots = shot;
  sl->in_base = base;
  cudaStream_t s = sl->s;
  cudaError_t err = cudaSuccess;
  if (!in_place)
    err = cudaMemcpyAsync(sl->d_rec, sl->h_rec, sizeof(int) * (size_t)off,
                          cudaMemcpyHostToDevice, s);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(sl->d_off, sl->h_off, sizeof(long long) * shot, cudaMemcpyHostToDevice, s);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(sl->d_code, sl->h_code, sizeof(int) * shot, cudaMemcpyHostToDevice, s);
  DevBatch b;
  memset(&b, 0, sizeof(b));
  b.num_shots = shot;
  b.num_codes = (int)e->codes.size();
  b.codes = (const DevCode *)e->d_codes;
  b.in = in_place ? base : sl->d_rec;
  b.in_off = sl->d_off;
  b.shot_code = sl->d_code;
  b.results = sl->d_res;
  b.ncr = e->ctx->d_ncr;
  b.jobs = sl->d_jobs;
  b.max_jobs = S->max_shots;
  b.counters = sl->d_small;
  b.status = (unsigned *)((char *)sl->d_small + kStatusByteOffset);
  b.scratch = sl->d_scratch;
  b.scratch_words = kSrvArenaWords;
  b.deferred = sl->d_deferred;
  b.queue = shot_queue(sl->d_deferred, S->max_shots);
  b.rec_cache = in_place ? shot_rec_cache(sl->d_deferred, S->max_shots) : nullptr;
  b.epoch = (unsigned *)((char *)sl->d_small + kCtlBytes);
  b.fast = e->tn.fast;
  b.light_max_log2 = e->tn.light_max_log2;
  b.tile_k = e->tn.tile_k;
  for (const DevCode &c : e->codes) b.has_ml |= c.variant == kMl;
  // each slot's persistent grid takes its share of the resident blocks, so the
  // slots' kernels are resident together and their batches overlap on the GPU
  Tuning tn = e->tn;
  const int share = std::max(1, e->ctx->decode_bps / std::max(1, (int)S->slots.size()));
  tn.search_grid_mult = tn.search_grid_mult ? std::min(tn.search_grid_mult, share) : share;
  if (err == cudaSuccess) err = launch_pipeline(e->ctx, b, tn, s);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(sl->h_res, sl->d_res, sizeof(GrandDecoderResult) * shot,
                          cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(sl->h_status, b.status, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(sl->h_top, ctr_ptr(b.counters, kCtrScratchTop), sizeof(unsigned long long),
                          cudaMemcpyDeviceToHost, s);
  sl->completed.store(0);
  if (err == cudaSuccess) err = cudaLaunchHostFunc(s, slot_done, sl);
  return err;
}

// A finished slot: results out to the requests (dispatcher thread, no lock).
void finish_slot(GrandServer *S, SrvSlot *sl, int rc) {
  if (rc == 0 && (*sl->h_status & (kStatusJobOverflow | kStatusScratchOverflow))) {
    // The batch outgrew the slot's job table or arena: decode it again through
    // the synchronous path, which re-runs the shots that did not fit.
    Workspace *ws = S->eng->ctx->acquire();
    BatchRequest req;
    req.num_shots = sl->nshots;
    req.codes = S->eng->codes;
    req.h_in = sl->in_base ? sl->in_base : sl->h_rec;
    long long extent = 0;
    for (int i = 0; i < sl->nshots; ++i)
      extent = std::max(extent, sl->h_off[i] + (long long)S->eng->rec_len[sl->h_code[i]]);
    req.in_ints = (size_t)extent;
    req.h_off = sl->h_off;
    req.h_shot_code = sl->h_code;
    req.h_results = sl->h_res;
    rc = ws ? run_batch(S->eng->ctx, ws, req, nullptr, &S->eng->tn) : GRAND_ERR_CUDA;
    if (ws) S->eng->ctx->release(ws);
  } else if (rc == 0 && (*sl->h_status & kStatusTamLimit)) {
    rc = GRAND_ERR_LIMIT;
  }
  if (rc == 0 && sl->nshots > 0) {
    // an overflowing batch staged at least the whole arena
    const double top = (*sl->h_status & kStatusScratchOverflow) ? (double)kSrvArenaWords
                                                                 : (double)*sl->h_top;
    const double per = top / (double)sl->nshots;
    std::lock_guard<std::mutex> lk(S->mu);
    S->scratch_per_shot = S->scratch_per_shot == 0.0 ? per : 0.75 * S->scratch_per_shot + 0.25 * per;
  }
  const Clock::time_point now = Clock::now();
  for (size_t i = 0; i < sl->reqs.size(); ++i) {
    SrvRequest &r = *sl->reqs[i];
    if (rc == 0) memcpy(r.results, sl->h_res + sl->first[i], sizeof(GrandDecoderResult) * r.n);
    r.rc = rc;
    r.t_done = now;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  for (auto &r : sl->reqs) r->done = true;
  sl->reqs.clear();
  sl->busy = false;
  S->cv_done.notify_all();
}

void dispatcher(GrandServer *S) {
  std::unique_lock<std::mutex> lk(S->mu);
  while (!S->stop) {
    bool progress = false;
    for (SrvSlot *sl : S->slots) {
      if (!sl->busy || !sl->completed.load()) continue;
      lk.unlock();
      cudaError_t q = cudaStreamSynchronize(sl->s);  // already complete: returns at once
      finish_slot(S, sl, q == cudaSuccess ? 0 : GRAND_ERR_CUDA);
      lk.lock();
      progress = true;
    }
    for (SrvSlot *sl : S->slots) {
      if (sl->busy || S->queue.empty()) continue;
      int shots = 0;
      sl->reqs.clear();
      // admission: the slot's shots, and the search scratch they are expected
      // to stage within 3/4 of its arena (at least one request per batch)
      const double room = 0.75 * (double)kSrvArenaWords;
      while (!S->queue.empty() && shots + S->queue.front()->n <= S->max_shots &&
             (shots == 0 || (shots + S->queue.front()->n) * S->scratch_per_shot <= room)) {
        shots += S->queue.front()->n;
        sl->reqs.push_back(S->queue.front());
        S->queue.pop_front();
      }
      if (sl->reqs.empty()) break;
      sl->first.assign(sl->reqs.size(), 0);
      sl->busy = true;
      lk.unlock();
      cudaError_t err = start_slot(S, sl);
      if (err != cudaSuccess) {
        set_error("grand server: launch failed (%s)", cudaGetErrorString(err));
        cudaStreamSynchronize(sl->s);
        finish_slot(S, sl, GRAND_ERR_CUDA);
      }
      lk.lock();
      progress = true;
    }
    if (!progress) S->cv_work.wait_for(lk, std::chrono::milliseconds(2));
  }
}

void free_slot(SrvSlot *sl) {
  if (sl->s) {
    cudaStreamSynchronize(sl->s);
    cudaStreamDestroy(sl->s);
  }
  if (sl->h_block) cudaFreeHost(sl->h_block);
  if (sl->d_block) cudaFree(sl->d_block);
  delete sl;
}

}  // namespace

extern "C" {

int grand_server_create(GrandEngine *e, int slots, int max_shots, size_t budget, GrandServer **out) {
  if (!e || !out || slots <= 0 || max_shots <= 0) return GRAND_ERR_INVALID;
  GrandServer *S = new GrandServer();
  S->eng = e;
  S->max_shots = max_shots;
  {
    std::lock_guard<std::mutex> lk(e->mu);
    if (e->codes.empty()) {
      delete S;
      set_error("grand server: register codes with the engine first");
      return GRAND_ERR_INVALID;
    }
    int rc = upload_codes(e);
    if (rc) {
      delete S;
      return rc;
    }
    for (int r : e->rec_len) S->max_rec = std::max(S->max_rec, r);
  }
  // Device bytes of one slot.
  const size_t rec = align256(sizeof(int) * (size_t)max_shots * S->max_rec);
  const size_t offb = align256(sizeof(long long) * max_shots);
  const size_t codeb = align256(sizeof(int) * max_shots);
  const size_t resb = align256(sizeof(GrandDecoderResult) * max_shots);
  const size_t jobb = align256(sizeof(Job) * max_shots);
  const size_t arena = align256(sizeof(uint32_t) * kSrvArenaWords);
  const size_t smallb = align256(kCtlAllocBytes);
  const size_t defb = align256(shot_buffer_bytes(max_shots));  // re-run flags, then the slow queue
  const size_t per_slot = rec + offb + codeb + resb + jobb + arena + smallb + defb;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    delete S;
    return GRAND_ERR_CUDA;
  }
  if (budget == 0) budget = free_b / 4;
  budget = std::min(budget, free_b - free_b / 16);  // admission by memory
  const int fit = (int)std::min<size_t>((size_t)slots, budget / per_slot);
  if (fit < 1) {
    delete S;
    set_error("grand server: one slot needs %zu bytes, the budget allows %zu", per_slot, budget);
    return GRAND_ERR_LIMIT;
  }
  for (int i = 0; i < fit; ++i) {
    SrvSlot *sl = new SrvSlot();
    sl->owner = S;
    cudaError_t err = cudaStreamCreateWithFlags(&sl->s, cudaStreamNonBlocking);
    const size_t hb = rec + offb + codeb + resb + 256;
    if (err == cudaSuccess) err = cudaHostAlloc(&sl->h_block, hb, cudaHostAllocDefault);
    if (err == cudaSuccess) err = cudaMalloc(&sl->d_block, per_slot);
    if (err == cudaSuccess) err = cudaMemset(sl->d_block, 0, per_slot);  // no launch's tags
    if (err != cudaSuccess) {
      free_slot(sl);
      break;
    }
    char *h = (char *)sl->h_block;
    sl->h_rec = (int *)h;
    sl->h_off = (long long *)(h + rec);
    sl->h_code = (int *)(h + rec + offb);
    sl->h_res = (GrandDecoderResult *)(h + rec + offb + codeb);
    sl->h_status = (unsigned *)(h + rec + offb + codeb + resb);
    sl->h_top = (unsigned long long *)(h + rec + offb + codeb + resb + 8);
    char *d = (char *)sl->d_block;
    sl->d_rec = (int *)d;
    d += rec;
    sl->d_off = (long long *)d;
    d += offb;
    sl->d_code = (int *)d;
    d += codeb;
    sl->d_res = (GrandDecoderResult *)d;
    d += resb;
    sl->d_jobs = (Job *)d;
    d += jobb;
    sl->d_scratch = (uint32_t *)d;
    d += arena;
    sl->d_small = (unsigned long long *)d;
    d += smallb;
    sl->d_deferred = (int *)d;
    S->slots.push_back(sl);
    S->dev_bytes += per_slot;
  }
  if (S->slots.empty()) {
    delete S;
    set_error("grand server: could not allocate a slot");
    return GRAND_ERR_CUDA;
  }
  S->th = std::thread(dispatcher, S);
  *out = S;
  return 0;
}

void grand_server_destroy(GrandServer *S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv_work.notify_all();
  }
  if (S->th.joinable()) S->th.join();
  for (SrvSlot *sl : S->slots) free_slot(sl);
  delete S;
}

int grand_server_info(GrandServer *S, int *slots, size_t *device_bytes) {
  if (!S) return GRAND_ERR_INVALID;
  if (slots) *slots = (int)S->slots.size();
  if (device_bytes) *device_bytes = S->dev_bytes;
  return 0;
}

int grand_server_submit(GrandServer *S, int n, const int *shot_code, const int *records,
                        GrandDecoderResult *results, unsigned long long *request_id) {
  if (!S || n <= 0 || n > S->max_shots || !records || !results) return GRAND_ERR_INVALID;
  const int ncodes = (int)S->eng->rec_len.size();
  if (shot_code)
    for (int i = 0; i < n; ++i)
      if (shot_code[i] < 0 || shot_code[i] >= ncodes) return GRAND_ERR_INVALID;
  auto r = std::make_shared<SrvRequest>();
  r->n = n;
  r->shot_code = shot_code;
  r->records = records;
  r->results = results;
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(S->mu);
  r->id = S->next_id++;
  S->live[r->id] = r;
  S->queue.push_back(r);
  S->cv_work.notify_one();
  if (request_id) *request_id = r->id;
  return 0;
}

int grand_server_wait(GrandServer *S, unsigned long long id, int timeout_ms, double *latency_ms) {
  if (!S) return GRAND_ERR_INVALID;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->live.find(id);
  if (it == S->live.end()) return GRAND_ERR_INVALID;
  std::shared_ptr<SrvRequest> r = it->second;
  if (timeout_ms < 0) {
    S->cv_done.wait(lk, [&] { return r->done; });
  } else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; })) {
    return 1;
  }
  S->live.erase(id);
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  return r->rc;
}

int grand_server_replay(GrandServer *S, int nreq, const double *arrival_s, const int *num_shots,
                        const int *shot_code, const int *records, GrandDecoderResult *results,
                        double *latency_ms, double *wall_s) {
  if (!S || nreq < 0 || (nreq > 0 && (!arrival_s || !num_shots || !records || !results)))
    return GRAND_ERR_INVALID;
  std::vector<long long> shot0(nreq + 1, 0), rec0(nreq + 1, 0);
  for (int i = 0; i < nreq; ++i) {
    if (num_shots[i] <= 0 || num_shots[i] > S->max_shots) return GRAND_ERR_INVALID;
    shot0[i + 1] = shot0[i] + num_shots[i];
    long long ints = 0;
    for (int j = 0; j < num_shots[i]; ++j) {
      const int c = shot_code ? shot_code[shot0[i] + j] : 0;
      if (c < 0 || c >= (int)S->eng->rec_len.size()) return GRAND_ERR_INVALID;
      ints += S->eng->rec_len[c];
    }
    rec0[i + 1] = rec0[i] + ints;
  }
  std::vector<unsigned long long> ids(nreq, 0);
  std::atomic<int> submit_rc{0};
  const Clock::time_point t0 = Clock::now();
  std::thread submitter([&] {
    for (int i = 0; i < nreq; ++i) {
      const Clock::time_point at = t0 + std::chrono::duration_cast<Clock::duration>(
                                            std::chrono::duration<double>(arrival_s[i]));
      while (Clock::now() < at) {
      }
      int rc = grand_server_submit(S, num_shots[i], shot_code ? shot_code + shot0[i] : nullptr,
                                   records + rec0[i], results + shot0[i], &ids[i]);
      if (rc) submit_rc.store(rc);
    }
  });
  submitter.join();
  int rc = submit_rc.load();
  Clock::time_point last = t0;
  for (int i = 0; i < nreq; ++i) {
    double lat = 0.0;
    const int w = ids[i] ? grand_server_wait(S, ids[i], -1, &lat) : GRAND_ERR_INVALID;
    if (w && !rc) rc = w;
    if (latency_ms) latency_ms[i] = lat;
    const Clock::time_point done =
        t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i])) +
        std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double, std::milli>(lat));
    if (done > last) last = done;
  }
  if (wall_s) {
    const double first = nreq ? arrival_s[0] : 0.0;
    *wall_s = std::chrono::duration<double>(last - t0).count() - first;
  }
  return rc;
}

}  // extern "C"
