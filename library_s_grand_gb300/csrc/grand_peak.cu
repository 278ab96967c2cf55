// grand_peak.cu -- integer-ALU throughput probe (the denominator of the search's roofline).
//
// The search is bound by 32-bit logic-op issue (LOP3 XOR/OR chains and IMNMX
// minima), not by HBM or tensor cores.  This kernel issues independent lop3.b32
// chains (8 per thread, inline PTX so the compiler cannot fold them) on every
// SM and reports the sustained rate in 32-bit ops per second, the denominator
// the decoder's integer roofline is quoted against.
#include <cuda_runtime.h>
#include <stdint.h>

namespace grand {

__global__ void __launch_bounds__(256) lop3_peak_kernel(uint32_t *sink, int iters, uint32_t seed) {
  uint32_t a[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) a[i] = seed ^ (threadIdx.x * 2654435761u + i * 40503u);
  const uint32_t b = seed * 747796405u + 1u, c = ~seed;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int r = 0; r < 16; ++r) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
        asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[i]) : "r"(b), "r"(c));
    }
  }
  uint32_t x = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) x ^= a[i];
  if (x == 0x12345678u) sink[blockIdx.x] = x;  // keeps the chains live
}

// Returns ops/s (one lop3 = one 32-bit op per lane) or a negative value.
double measure_lop3_peak(int sm_count) {
  uint32_t *sink = nullptr;
  if (cudaMalloc(&sink, sizeof(uint32_t) * 65536) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int bps = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, lop3_peak_kernel, 256, 0);
  if (bps < 1) bps = 1;
  const int grid = sm_count * bps;
  const int iters = 4096;
  lop3_peak_kernel<<<grid, 256>>>(sink, 64, 1u);  // warm-up
  double best = 0.0;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    lop3_peak_kernel<<<grid, 256>>>(sink, iters, 7u + rep);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double ops = (double)grid * 256.0 * iters * 16.0 * 8.0;
    if (ms > 0 && ops / (ms * 1e-3) > best) best = ops / (ms * 1e-3);
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  return err == cudaSuccess ? best : -1.0;
}

}  // namespace grand
