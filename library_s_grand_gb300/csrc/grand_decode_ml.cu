// grand_decode_ml.cu -- the decode kernel built with the ML (cost-ordered)
// search paths, for batches with an ML code.
#include "grand_decode.cuh"
#include "grand_host.h"

namespace grand {

#ifndef GRAND_HOST_EMULATION
cudaError_t launch_decode_ml(const DevBatch &b, int grid, cudaStream_t s) {
  decode_kernel<true><<<grid, kDecodeWarps * 32, 0, s>>>(b);
  return cudaGetLastError();
}

cudaError_t decode_occupancy_ml(int *blocks_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, decode_kernel<true>,
                                                       kDecodeWarps * 32, 0);
}
#endif

}  // namespace grand
