// grand_noalloc.cu -- grand_decode_cc_noalloc: a decode that allocates nothing.
//
// Who needs it: callers that must not allocate device memory once they are
// running -- a real-time decoding loop in a quantum-control stack that reserves
// its memory up front and may not stall in the allocator mid-experiment, or a
// host process whose device memory is already entirely owned by another
// framework's pool.  The regular entry points allocate their workspaces with
// cudaMalloc on first use (and grow them); this one keeps everything it needs
// beyond the caller's inputs and outputs in one fixed, file-scope device array.
//
// The batch runs through the same decode kernel as the other entry points.  Only the place their scratch lives differs: the binomial table, the
// packed columns, the code descriptor, the counters, the job table and the
// scratch arena are carved out of g_noalloc_scratch.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "grand_common.h"
#include "grand_host.h"

namespace grand {
namespace {

// Limits of the no-allocation path.
constexpr int kNaMaxRows = 256;                     // R <= 256 (8 words per column)
constexpr int kNaMaxCols = 1024;                    // m <= 1024
constexpr int kNaChunk = 2048;                      // shots per launch = job slots
constexpr unsigned long long kNaArenaWords = 4ull << 20;  // 16 MiB of staged search data

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffNcr = 0;
constexpr size_t kOffCode = align256(kOffNcr + sizeof(unsigned long long) * (kMaxTam + 1) * (kMaxW + 1));
constexpr size_t kOffCols = align256(kOffCode + sizeof(DevCode));
constexpr size_t kOffColw = align256(kOffCols + sizeof(uint32_t) * kNaMaxCols * 8);
constexpr size_t kOffHcol = align256(kOffColw + sizeof(int) * kNaMaxCols);
constexpr size_t kOffSmall = align256(kOffHcol + sizeof(uint32_t) * kNaMaxCols);  // control block
constexpr size_t kOffDeferred = align256(kOffSmall + kCtlAllocBytes);
constexpr size_t kOffMap = align256(kOffDeferred + sizeof(int) * kNaChunk);     // re-run list
constexpr size_t kOffMapCount = align256(kOffMap + sizeof(int) * kNaChunk);     // its length
constexpr size_t kOffQueue = align256(kOffMapCount + 256);                       // slow queue
constexpr size_t kOffJobs = align256(kOffQueue + sizeof(unsigned long long) * kNaChunk);
constexpr size_t kOffArena = align256(kOffJobs + sizeof(Job) * kNaChunk);
constexpr size_t kScratchBytes = align256(kOffArena + sizeof(uint32_t) * kNaArenaWords);

}  // namespace

// All no-allocation calls on a device share this array; it exists for the life
// of the process on every device that loads this part of the library.  It starts
// zeroed, as the launch tags of its queue entries and Jobs require.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

// C(n, k) by the same multiplicative formula as the host table.
__global__ void noalloc_ncr_kernel(unsigned long long *t) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n > kMaxTam) return;
  for (int k = 0; k <= kMaxW; ++k) {
    unsigned long long r = 0;
    if (k <= n) {
      r = 1;
      if (k != 0 && k != n)
        for (int i = 1; i <= k; ++i) r = r * (unsigned long long)(n - i + 1) / (unsigned long long)i;
    }
    t[n * (kMaxW + 1) + k] = r;
  }
}

// One thread per column: packed bits (LSB-first, nwp words), the column weight
// and the column sketch.
__global__ void noalloc_pack_kernel(const int *H, int n, int m, int nwp, uint32_t *cols, int *colw,
                                    uint32_t *hcol) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m) return;
  uint32_t w[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
  uint32_t h = 0u;
  int sum = 0;
  for (int r = 0; r < n; ++r) {
    const int v = H[(size_t)r * m + c];
    sum += v;
    if (v != 0) {
      w[r >> 5] |= 1u << (r & 31);
      h ^= row_hash(r);
    }
  }
  for (int i = 0; i < nwp; ++i) cols[(size_t)c * nwp + i] = w[i];
  colw[c] = sum;
  hcol[c] = h;
}

// One block: maximum column weight and regularity, then the code descriptor.
__global__ void noalloc_code_kernel(DevCode tmpl, const int *colw, int m, DevCode *out) {
  __shared__ int s_max, s_irregular;
  if (threadIdx.x == 0) {
    s_max = 0;
    s_irregular = 0;
  }
  __syncthreads();
  int mx = 0, irr = 0;
  const int c0 = colw[0];
  for (int c = threadIdx.x; c < m; c += blockDim.x) {
    mx = max(mx, colw[c]);
    irr |= colw[c] != c0;
  }
  atomicMax(&s_max, mx);
  if (irr) atomicOr(&s_irregular, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    tmpl.max_soma = s_max;
    tmpl.regular = s_irregular ? 0 : 1;
    *out = tmpl;
  }
}

// One warp: the ascending list of the chunk's shots that the last round deferred
// (their heavy-shot staging did not fit the arena), and its length.  Every shot
// of the chunk had its flag written in the first round, and a re-run rewrites
// the flags of the shots it runs, so the flags are current for all cnt shots.
__global__ void noalloc_deferred_kernel(const int *deferred, int cnt, int *map, int *count) {
  const int lane = threadIdx.x & 31;
  int base = 0;
  for (int i0 = 0; i0 < cnt; i0 += 32) {
    const bool d = i0 + lane < cnt && deferred[i0 + lane] != 0;
    const unsigned bits = __ballot_sync(0xffffffffu, d);
    if (d) map[base + __popc(bits & ((1u << lane) - 1u))] = i0 + lane;
    base += __popc(bits);
  }
  if (lane == 0) *count = base;
}

// Shots that could not be searched within the arena even one at a time: a
// zero result record (found = 0), so that no stale bytes are left behind.
__global__ void noalloc_clear_kernel(const int *map, int count, GrandDecoderResult *results) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count * 18) return;
  reinterpret_cast<uint32_t *>(results + map[i / 18])[i % 18] = 0u;
}

std::mutex g_mu;
unsigned char *g_base[64] = {};  // device address of g_noalloc_scratch per device
int g_sms[64] = {}, g_bps[64] = {};

}  // namespace
}  // namespace grand

using namespace grand;

extern "C" int grand_decode_cc_noalloc(const int *d_H, int n, int m, const int *d_syndromes,
                                       int num_shots, const GrandDecoderConfig *config,
                                       GrandDecoderResult *d_results, void *stream) {
  if (!config) {
    fprintf(stderr, "grand: config is NULL\n");
    return GRAND_ERR_INVALID;
  }
  const int W = config->max_error_weight;
  if (W <= 0 || W > 7) {
    fprintf(stderr, "Invalid max_error_weight: %d. Must be between 1 and 7.\n", W);
    return GRAND_ERR_INVALID;
  }
  if (num_shots < 0) {
    fprintf(stderr, "grand_decode_cc_noalloc: negative shot count\n");
    return GRAND_ERR_INVALID;
  }
  if (num_shots == 0) return 0;
  if (!d_H || !d_syndromes || !d_results) {
    fprintf(stderr, "grand_decode_cc_noalloc: NULL matrix, syndrome or result pointer\n");
    return GRAND_ERR_INVALID;
  }
  if (n <= 0 || n > kNaMaxRows || m <= 0 || m > kNaMaxCols) {
    fprintf(stderr,
            "grand_decode_cc_noalloc: H is %d x %d; this entry point supports at most %d rows and "
            "%d columns (its scratch is a fixed %zu-byte device array)\n",
            n, m, kNaMaxRows, kNaMaxCols, (size_t)kScratchBytes);
    return GRAND_ERR_LIMIT;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    fprintf(stderr, "grand_decode_cc_noalloc: no usable CUDA device (%s)\n", cudaGetErrorString(e));
    return GRAND_ERR_CUDA;
  }
  unsigned char *base = nullptr;
  {
    // Set-up, once per device, with that device current: the device address of
    // the scratch array and its binomial table.
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess) {
        fprintf(stderr, "grand_decode_cc_noalloc: cudaGetSymbolAddress failed (%s)\n",
                cudaGetErrorString(e));
        return GRAND_ERR_CUDA;
      }
      int sms = 0, bps = 0;
      e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e == cudaSuccess) e = decode_occupancy(&bps);
      if (e == cudaSuccess) {
        noalloc_ncr_kernel<<<(kMaxTam + 256) / 256, 256, 0, s>>>(
            reinterpret_cast<unsigned long long *>((unsigned char *)ptr + kOffNcr));
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) {
        fprintf(stderr, "grand_decode_cc_noalloc: set-up failed (%s)\n", cudaGetErrorString(e));
        return GRAND_ERR_CUDA;
      }
      g_sms[dev] = sms;
      g_bps[dev] = bps > 0 ? bps : 1;
      g_base[dev] = (unsigned char *)ptr;
    }
    base = g_base[dev];
  }

  const int nw = (n + 31) / 32;
  const int nwp = nw <= 2 ? nw : (nw <= 4 ? 4 : 8);
  uint32_t *cols = reinterpret_cast<uint32_t *>(base + kOffCols);
  int *colw = reinterpret_cast<int *>(base + kOffColw);
  uint32_t *hcol = reinterpret_cast<uint32_t *>(base + kOffHcol);
  DevCode *code = reinterpret_cast<DevCode *>(base + kOffCode);

  DevCode t;
  memset(&t, 0, sizeof(t));
  t.R = n;
  t.m = m;
  t.nw = nw;
  t.nwp = nwp;
  t.mw = (m + 31) / 32;
  t.family = kCss;
  t.variant = kUniform;
  t.input_kind = kInSyndromes;
  t.W = W;
  t.Wc = W < kMaxW ? W : kMaxW;
  t.mode = config->mode_of_search;
  t.thr = config->threshold_for_hybrid;
  t.cap = config->max_size_active_positions;
  t.rec_len = n;
  t.cols = cols;
  t.colw = colw;
  t.hcol = hcol;

  noalloc_pack_kernel<<<(m + 127) / 128, 128, 0, s>>>(d_H, n, m, nwp, cols, colw, hcol);
  noalloc_code_kernel<<<1, 256, 0, s>>>(t, colw, m, code);
  e = cudaGetLastError();

  const Tuning &tn = tuning();
  // the decode kernel's CTAs per SM as the regular entry points choose them
  const int per_sm = decode_blocks_per_sm(g_bps[dev], tn);
  int *map = reinterpret_cast<int *>(base + kOffMap);
  int *map_count = reinterpret_cast<int *>(base + kOffMapCount);
  unsigned st = 0;       // status bits of every round of every chunk
  long long unsearched = 0;  // shots whose staging alone exceeds the arena
  for (int lo = 0; lo < num_shots && e == cudaSuccess; lo += kNaChunk) {
    const int cnt = num_shots - lo < kNaChunk ? num_shots - lo : kNaChunk;
    DevBatch b;
    memset(&b, 0, sizeof(b));
    b.num_codes = 1;
    b.codes = code;
    b.in = d_syndromes + (size_t)lo * n;
    b.results = d_results + lo;
    b.ncr = reinterpret_cast<const unsigned long long *>(base + kOffNcr);
    b.jobs = reinterpret_cast<Job *>(base + kOffJobs);
    b.max_jobs = kNaChunk;
    b.counters = reinterpret_cast<unsigned long long *>(base + kOffSmall);
    b.status = reinterpret_cast<unsigned *>(base + kOffSmall + kStatusByteOffset);
    b.scratch = reinterpret_cast<uint32_t *>(base + kOffArena);
    b.scratch_words = kNaArenaWords;
    b.deferred = reinterpret_cast<int *>(base + kOffDeferred);
    b.queue = reinterpret_cast<unsigned long long *>(base + kOffQueue);
    b.epoch = reinterpret_cast<unsigned *>(base + kOffSmall + kCtlBytes);
    b.fast = tn.fast;
    b.light_max_log2 = tn.light_max_log2;
    b.tile_k = tn.tile_k;
    // Rounds: all of the chunk's shots, then, while some heavy shots found the
    // arena full, only those (their list built on the device), each round with
    // an empty arena.  A round in which no deferred shot fits means that each of
    // them alone needs more than the arena: those get a zero result.
    int todo = cnt;
    for (int round = 0; e == cudaSuccess; ++round) {
      b.num_shots = todo;
      b.shot_map = round == 0 ? nullptr : map;
      // control words and status restart for every round
      e = cudaMemsetAsync(base + kOffSmall, 0, kCtlBytes, s);
      if (e == cudaSuccess) e = launch_decode(b, g_sms[dev] * per_sm, s);
      unsigned rs = 0;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(&rs, base + kOffSmall + kStatusByteOffset, sizeof(unsigned),
                            cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) break;
      st |= rs & ~(unsigned)(kStatusScratchOverflow | kStatusJobOverflow);
      if (!(rs & (kStatusScratchOverflow | kStatusJobOverflow))) break;
      noalloc_deferred_kernel<<<1, 32, 0, s>>>(b.deferred, cnt, map, map_count);
      int left = 0;
      e = cudaGetLastError();
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(&left, map_count, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess || left == 0) break;
      if (left >= todo) {
        noalloc_clear_kernel<<<(left * 18 + 255) / 256, 256, 0, s>>>(map, left, b.results);
        e = cudaGetLastError();
        unsearched += left;
        break;
      }
      todo = left;
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    fprintf(stderr, "grand_decode_cc_noalloc: CUDA error %s\n", cudaGetErrorString(e));
    return GRAND_ERR_CUDA;
  }
  if (unsearched) {
    fprintf(stderr,
            "grand_decode_cc_noalloc: %lld shot(s) need more than the fixed %llu-word search "
            "arena on their own; their results are zero (found = 0)\n",
            unsearched, kNaArenaWords);
    return GRAND_ERR_LIMIT;
  }
  if (st & kStatusTamLimit) {
    fprintf(stderr, "grand_decode_cc_noalloc: an active-position set exceeded %d\n", kMaxTam);
    return GRAND_ERR_LIMIT;
  }
  if (st & kStatusCasLimit) return GRAND_ERR_CUDA;
  return 0;
}
