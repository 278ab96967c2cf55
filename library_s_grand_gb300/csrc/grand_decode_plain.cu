// grand_decode_plain.cu -- the decode kernel built without the ML paths (smaller
// code, fewer registers), for batches without an ML code; and the launcher that
// picks the build.
#include "grand_decode.cuh"
#include "grand_host.h"

namespace grand {

#ifndef GRAND_HOST_EMULATION
cudaError_t launch_decode_ml(const DevBatch &b, int grid, cudaStream_t s);
cudaError_t decode_occupancy_ml(int *blocks_per_sm);

cudaError_t launch_decode(const DevBatch &b, int grid, cudaStream_t s) {
  if (b.has_ml) return launch_decode_ml(b, grid, s);
  decode_kernel<false><<<grid, kDecodeWarps * 32, 0, s>>>(b);
  return cudaGetLastError();
}

// Resident blocks per SM both builds reach (the grid is sized for the smaller).
cudaError_t decode_occupancy(int *blocks_per_sm) {
  int a = 0, c = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, decode_kernel<false>,
                                                                kDecodeWarps * 32, 0);
  if (e == cudaSuccess) e = decode_occupancy_ml(&c);
  *blocks_per_sm = a < c ? a : c;
  return e;
}
#endif

}  // namespace grand
