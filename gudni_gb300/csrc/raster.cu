// Raster kernels (sm_103a).
//
// raster_columns_kernel fuses the reference's three launches (generateThresholds,
// sortThresholds, renderThresholds; OpenCL/CallKernels.hs:124-174) into one: each
// thread runs whole columns start to finish, so the threshold queue never makes the
// generate -> sort -> render round trips through global memory that the reference's
// three kernels make.
//
// Launch shape: a persistent grid (SMs x resident blocks) strides over the job's
// work items (tile x column, the reference's NDRange), consecutive threads taking
// consecutive columns of one tile so a warp walks the same strands together.  Each
// resident thread owns a scratch slot: a threshold queue of `capacity` entries and
// the shape-index table of its column.
//
// Capacity: the fast pass uses a small working capacity.  A column that needs more
// is recorded in an overflow list and re-run by a second launch of the same kernel
// with the spec's full max_thresholds; the second launch reads the list's length on
// the device, so the pair is enqueued without a host round trip (and can be captured
// in a CUDA graph).  The result does not depend on the capacity, only on whether it
// suffices.  A column that exceeds max_thresholds raises
// kStatusOverflow (the reference silently writes past its slab there,
// Kernels.cl:375-380, 1096-1103).

#include <cuda_runtime.h>

#include "raster_device.cuh"
#include "raster_kernels.h"

namespace gudni {

__device__ __forceinline__ bool tileOk(const gudni_tile_info& ti, uint32_t n_shapes) {
  return ti.hdepth >= 0 && ti.hdepth <= 24 && ti.vdepth >= 0 && ti.vdepth <= 24 && ti.left >= 0 &&
         ti.top >= 0 && ti.right >= ti.left && ti.bottom >= ti.top &&
         (uint64_t)ti.shapes.start + (uint64_t)ti.shapes.length <= (uint64_t)n_shapes;
}

template <int SECTIONS>
__global__ void __launch_bounds__(kRasterBlock) raster_columns_kernel(ColumnLaunch a) {
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nslots = gridDim.x * blockDim.x;
  float4* thr = a.scratch.thr + (size_t)slot * (size_t)a.scratch.capacity;
  uint32_t* hdr = a.scratch.hdr + (size_t)slot * (size_t)a.scratch.capacity;
  uint32_t* idx = a.scratch.idx + (size_t)slot * (size_t)a.scratch.idx_stride;
  const uint32_t tmask = (1u << a.in.log2_tpt) - 1u;
  int status = 0;
  uint32_t n_items = a.n_items;
  if (a.n_items_dev) n_items = min(n_items, *a.n_items_dev);
  for (uint32_t w = slot; w < n_items; w += nslots) {
    const uint32_t item = a.items ? a.items[w] : w;
    const int tile = (int)(item >> a.in.log2_tpt);
    const int column = (int)(item & tmask);
    const gudni_tile_info ti = a.in.tiles[tile];
    if (!tileOk(ti, a.in.n_shapes)) {
      status |= kStatusBadInput;
      continue;
    }
    const ColumnState c = initColumn(a.in, ti, column, a.in.tile_jobs ? a.in.tile_jobs[tile] : a.in.job_index);
    if (!c.active) continue;
    Queue q{thr, hdr, a.scratch.capacity, a.scratch.capacity, false};
    ShapeStack<SECTIONS> stack;
    stack.clear();
    const uint32_t bits = buildThresholds<SECTIONS>(a.in, c, q, stack, idx, status);
    if (a.in.counters && !q.overflow) {
      atomicAdd(reinterpret_cast<unsigned long long*>(&a.in.counters[2]), (unsigned long long)q.length());
      atomicMax(reinterpret_cast<unsigned long long*>(&a.in.counters[3]), (unsigned long long)bits);
    }
    if (!q.overflow) renderColumn<SECTIONS>(a.in, c, q, stack, idx, status);
    if (q.overflow) {
      if (a.overflow_items) {
        const uint32_t k = atomicAdd(a.overflow_count, 1u);
        if (k < a.overflow_cap) {
          a.overflow_items[k] = item;
        } else {
          status |= kStatusOverflow;
        }
      } else {
        status |= kStatusOverflow;
      }
    }
  }
  if (status) atomicOr(a.status, status);
}

template <int S>
static cudaError_t launch_s(const ColumnLaunch& a, int grid, cudaStream_t stream) {
  raster_columns_kernel<S><<<grid, kRasterBlock, 0, stream>>>(a);
  return cudaGetLastError();
}

int sections_for(int max_shape) {
  int need = (max_shape + 1 + 63) / 64;
  int s = 1;
  while (s < need) s *= 2;
  return s;
}

cudaError_t launch_columns(const ColumnLaunch& a, int sections, int grid, cudaStream_t stream) {
  switch (sections) {
    case 1: return launch_s<1>(a, grid, stream);
    case 2: return launch_s<2>(a, grid, stream);
    case 4: return launch_s<4>(a, grid, stream);
    case 8: return launch_s<8>(a, grid, stream);
    case 16: return launch_s<16>(a, grid, stream);
    case 32: return launch_s<32>(a, grid, stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t columns_occupancy(int sections, int* blocks_per_sm) {
  const void* fn = nullptr;
  switch (sections) {
    case 1: fn = (const void*)raster_columns_kernel<1>; break;
    case 2: fn = (const void*)raster_columns_kernel<2>; break;
    case 4: fn = (const void*)raster_columns_kernel<4>; break;
    case 8: fn = (const void*)raster_columns_kernel<8>; break;
    case 16: fn = (const void*)raster_columns_kernel<16>; break;
    case 32: fn = (const void*)raster_columns_kernel<32>; break;
    default: return cudaErrorInvalidValue;
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kRasterBlock, 0);
}

}  // namespace gudni
