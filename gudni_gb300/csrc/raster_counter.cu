// The per-lane raster kernels with the counter-based stochastic jitter
// (gudni_set_random_source(GUDNI_RANDOM_COUNTER)), compiled apart from raster.cu so
// that the default kernels keep the reference scan's code and registers.

#include <cuda_runtime.h>

#include "column_kernels.cuh"

namespace gudni {

template <int S>
static cudaError_t launch_counter_s(const TileLaunch& a, bool list, int grid, cudaStream_t stream) {
  if (list) {
    raster_list_kernel<S, true><<<grid, kRasterBlock, 0, stream>>>(a);
  } else {
    raster_tiles_kernel<S, true><<<grid, kRasterBlock, 0, stream>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_raster_counter(const TileLaunch& a, bool list, int sections, int grid, cudaStream_t stream) {
  switch (sections) {
    case 1: return launch_counter_s<1>(a, list, grid, stream);
    case 2: return launch_counter_s<2>(a, list, grid, stream);
    case 4: return launch_counter_s<4>(a, list, grid, stream);
    case 8: return launch_counter_s<8>(a, list, grid, stream);
    case 16: return launch_counter_s<16>(a, list, grid, stream);
    case 32: return launch_counter_s<32>(a, list, grid, stream);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gudni
