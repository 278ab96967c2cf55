// grand_sample.cu -- on-device shot generation for registered codes (sm_103a).
//
// No upstream counterpart: upstream draws its shots in Python (numpy / stim,
// Create_Files/*) and ships them to the decoder as int32 rows.  Here a kernel
// draws i.i.d. flips of every error position (CSS: qubit, DEM: mechanism) with
// per-position probabilities, forms the syndrome / detectors and true logical
// flips, and writes the code's int32 records straight into device memory for
// grand_engine_decode_device: a statistical run never moves shots over PCIe or
// C2C.
//
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011), a counter-based generator: output
// block = Philox(counter, key) with no state, so every (seed, shot, position)
// has its own fixed draw whatever the launch shape.  Key = the 64-bit seed;
// counter = {group, shot low, shot high, 0x47524E44}; lane l of a warp computes
// block (32g + l) and uses word u for position 128g + 32u + l.  A position
// flips when its 32-bit word is below floor(p * 2^32) (p = 1: 2^32 - 1).
#include <cuda_runtime.h>

#include "grand_device.cuh"
#include "grand_host.h"

namespace grand {

__host__ __device__ inline void philox4x32_10(uint32_t (&c)[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned long long p0 = 0xD2511F53ull * c[0];
    const unsigned long long p1 = 0xCD9E8D57ull * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__device__ __forceinline__ uint32_t flip_threshold(float p) {
  // p * 2^32 is exact in FP32 (a power-of-two scale); truncate, clamp p >= 1
  const float s = p * 4294967296.0f;
  return s >= 4294967295.0f ? 0xFFFFFFFFu : (s <= 0.0f ? 0u : (uint32_t)s);
}

// One warp per shot.  The flips are packed into the warp's shared-memory word
// array, then the record entries are written with coalesced int32 stores.
__global__ void __launch_bounds__(256) sample_kernel(DevCode cd, const float *p,
                                                     unsigned long long seed,
                                                     unsigned long long first_shot, int num_shots,
                                                     int *records) {
  __shared__ uint32_t s_flip[8][kMaxCols / 32];
  __shared__ uint32_t s_syn[8][kMaxRows / 32];
  __shared__ uint32_t s_log[8][kMaxLogicals / 32];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  uint32_t *flip = s_flip[wib];
  uint32_t *syn = s_syn[wib];
  uint32_t *lg = s_log[wib];
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  const int nwarps = gridDim.x * 8;
  for (int i = blockIdx.x * 8 + wib; i < num_shots; i += nwarps) {
    const unsigned long long shot = first_shot + (unsigned long long)i;
    // flips: 128 positions per group, four words of one block per lane
    for (int g = 0; g * 128 < cd.m; ++g) {
      uint32_t c[4] = {(uint32_t)(g * 32 + lane), (uint32_t)shot, (uint32_t)(shot >> 32),
                       0x47524E44u};
      philox4x32_10(c, k0, k1);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = g * 128 + u * 32 + lane;
        const bool f = j < cd.m && c[u] < flip_threshold(__ldg(p + j));
        const uint32_t bits = __ballot_sync(kFull, f);
        if (lane == 0 && g * 4 + u < cd.mw) flip[g * 4 + u] = bits;
      }
    }
    __syncwarp();
    // syndrome / detectors: XOR of the flipped columns (lane w: word w)
    uint32_t s_lane = 0u;
    for (int q = 0; q < cd.mw; ++q) {
      uint32_t word = flip[q];
      while (word) {
        const int col = q * 32 + __ffs(word) - 1;
        word &= word - 1u;
        if (lane < cd.nw) s_lane ^= __ldg(cd.cols + (size_t)col * cd.nwp + lane);
      }
    }
    if (lane < cd.nw) syn[lane] = s_lane;
    // DEM: true logical flips, XOR of the flipped mechanisms' rows of L
    if (cd.family == kDem) {
      for (int q = lane; q < cd.nlw; q += 32) {
        uint32_t acc = 0u;
        for (int qq = 0; qq < cd.mw; ++qq) {
          uint32_t word = flip[qq];
          while (word) {
            const int col = qq * 32 + __ffs(word) - 1;
            word &= word - 1u;
            acc ^= __ldg(cd.lcols + (size_t)col * cd.nlw + q);
          }
        }
        lg[q] = acc;
      }
    }
    __syncwarp();
    int *rec = records + (size_t)i * cd.rec_len;
    if (cd.input_kind == kInErrors) {
      for (int j = lane; j < cd.m; j += 32) rec[j] = (flip[j >> 5] >> (j & 31)) & 1u;
    } else {
      for (int r = lane; r < cd.R; r += 32) rec[r] = (syn[r >> 5] >> (r & 31)) & 1u;
      if (cd.family == kDem)
        for (int j = lane; j < cd.n_logicos; j += 32) rec[cd.R + j] = (lg[j >> 5] >> (j & 31)) & 1u;
    }
    __syncwarp();
  }
}

cudaError_t launch_sample(const DevCode &cd, const float *d_p, unsigned long long seed,
                          unsigned long long first_shot, int num_shots, int *d_records,
                          int sm_count, cudaStream_t s) {
  if (num_shots <= 0) return cudaSuccess;
  int grid = (num_shots + 7) / 8;
  if (grid > sm_count * 8) grid = sm_count * 8;
  sample_kernel<<<grid, 256, 0, s>>>(cd, d_p, seed, first_shot, num_shots, d_records);
  return cudaGetLastError();
}

}  // namespace grand
