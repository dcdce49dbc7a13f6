// Raster kernels (sm_103a).
//
// The reference makes three launches per job (generateThresholds, sortThresholds,
// renderThresholds; OpenCL/CallKernels.hs:124-174) and round-trips every column's
// threshold queue and shape state through global memory between them.  Here one
// thread runs a whole column start to finish (raster_device.cuh), and two kernels
// schedule the columns:
//
// raster_tiles_kernel -- the fast pass.  A persistent grid of warps pulls work units
//   -- 32 consecutive columns of one tile -- from a work counter (one atomicAdd per
//   unit, lane 0), optionally from a cost-descending unit list, and runs the unit's
//   columns on its lanes (the lanes walk the same strands and write one row segment
//   per pixel row).  A tile of more than 32 columns is spread over several warps.
//   Tiles may belong to different scenes of a batch, each with its own canvas,
//   output, background and threads per tile.  Every thread owns a scratch slot (a
//   queue of `capacity` entries and the shape-index table of its column).
//
// raster_tiles_warp_kernel -- the fast pass with warp-cooperative dense columns
//   (warp_column.cuh): the same units, but a unit's columns whose queues hold at least
//   `dense_min` thresholds are scanned by the whole warp, one after another, instead
//   of each by its own lane.  Chosen by gudni_set_dense_columns; the output is the
//   same bit for bit.
//
// raster_list_kernel -- the full-capacity pass.  Columns that overflowed the fast
//   pass's small working capacity were appended to a list (work unit and lane); this kernel, launched
//   right after on the same stream, reads the list's length on the device and re-runs
//   them with the spec's max_thresholds.  The result does not depend on the capacity,
//   only on whether it suffices, and no host round trip separates the two launches
//   (the pair can be captured in a CUDA graph).  A column that exceeds max_thresholds
//   raises kStatusOverflow (the reference silently writes past its slab there,
//   Kernels.cl:375-380, 1096-1103).

#include <cuda_runtime.h>

#include <algorithm>

#include "column_kernels.cuh"
#include "raster_device.cuh"
#include "raster_kernels.h"
#include "tile_coop.cuh"
#include "warp_column.cuh"

namespace gudni {

// The fast pass with warp-cooperative units (tile_coop.cuh): a unit's thresholds are
// generated by all 32 lanes over (strand, column) pairs and binned to the columns by
// ballots, the tile's shape records are staged by a bulk copy, each lane sorts and
// scans its column as in raster_tiles_kernel, and the pixels leave through a
// shared-memory tile by whole rows.  Units that do not qualify run the per-column code
// on their lanes.  The image is raster_tiles_kernel's bit for bit.
template <int SECTIONS>
__global__ void __launch_bounds__(kRasterBlock) raster_tiles_coop_kernel(TileLaunch a) {
  __shared__ __align__(16) CoopShared sh[kRasterBlock / 32];
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  CoopShared& cs = sh[threadIdx.x >> 5];
  const size_t cap = (size_t)a.scratch.capacity;
  const size_t istride = (size_t)a.scratch.idx_stride;
  float4* thr = a.scratch.thr + (size_t)slot * cap;
  uint32_t* hdr = a.scratch.hdr + (size_t)slot * cap;
  uint32_t* idx = a.scratch.idx + (size_t)slot * istride;
  float4* thrWarp = thr - (size_t)lane * cap;
  uint32_t* hdrWarp = hdr - (size_t)lane * cap;
  if (lane == 0) mbarInit(&cs.mbar);
  __syncwarp();
  uint32_t phase = 0u;
  int status = 0;
  for (;;) {
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(a.next_tile, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= a.n_units) break;
    int tile, chunk;
    unitOf(a.units, a.chunk_log2, k, tile, chunk);
    bool ok;
    const RasterInputs in = sceneInputs(a.in, a.scenes, a.tile_scene, a.n_scenes, tile, status, ok);
    if (!ok) continue;
    const gudni_tile_info ti = in.tiles[tile];
    if (!tileOk(ti, in.n_shapes) || in.log2_tpt < 0 || in.log2_tpt > kMaxLog2Tpt) {
      status |= kStatusBadInput;
      continue;
    }
    const int tpt = 1 << in.log2_tpt;
    const int column = chunk * 32 + lane;
    const int flags = runUnitCoop(in, ti, chunk, lane, thrWarp, hdrWarp, (int)cap, status, cs, phase);
    bool overflow = (flags & kCoopOverflow) != 0;
    if (flags & kCoopNotTaken)
      overflow = column < tpt && runColumn<SECTIONS, false>(in, ti, column, thr, hdr, (int)cap, idx, status);
    if (overflow) {
      if (a.overflow_items) {
        const uint32_t n = atomicAdd(a.overflow_count, 1u);
        if (n < a.overflow_cap) {
          a.overflow_items[n] = (k << kLaneBits) | (uint32_t)lane;
        } else {
          status |= kStatusOverflow;
        }
      } else {
        status |= kStatusOverflow;
      }
    }
  }
  bulkStoreDrain();
  if (status) atomicOr(a.status, status);
}

template <int SECTIONS>
__global__ void __launch_bounds__(kRasterBlock) raster_tiles_warp_kernel(TileLaunch a) {
  __shared__ float4 sProd[kRasterBlock];
  __shared__ uint32_t sBit[kRasterBlock];
  __shared__ uint32_t sFlips[kRasterBlock / 32 * kWarpFlipWords];
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const WarpScratch ws{sProd + (threadIdx.x & ~31u), sBit + (threadIdx.x & ~31u),
                       sFlips + (threadIdx.x >> 5) * kWarpFlipWords};
  float4* thr = a.scratch.thr + (size_t)slot * (size_t)a.scratch.capacity;
  uint32_t* hdr = a.scratch.hdr + (size_t)slot * (size_t)a.scratch.capacity;
  uint32_t* idx = a.scratch.idx + (size_t)slot * (size_t)a.scratch.idx_stride;
  int status = 0;
  for (;;) {
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(a.next_tile, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= a.n_units) break;
    int tile, chunk;
    unitOf(a.units, a.chunk_log2, k, tile, chunk);
    bool ok;
    const RasterInputs in = sceneInputs(a.in, a.scenes, a.tile_scene, a.n_scenes, tile, status, ok);
    if (!ok) continue;
    const gudni_tile_info ti = in.tiles[tile];
    if (!tileOk(ti, in.n_shapes) || in.log2_tpt < 0 || in.log2_tpt > kMaxLog2Tpt) {
      status |= kStatusBadInput;
      continue;
    }
    const int tpt = 1 << in.log2_tpt;
    const int column = chunk * 32 + lane;
    const int flags = runUnitWarp<SECTIONS>(in, ti, column, column < tpt, thr, hdr, a.scratch.capacity, idx, status,
                                            lane, a.dense_min, ws);
    if (flags & kUnitOverflow) {
      if (a.overflow_items) {
        const uint32_t n = atomicAdd(a.overflow_count, 1u);
        if (n < a.overflow_cap) {
          a.overflow_items[n] = (k << kLaneBits) | (uint32_t)lane;
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

// ------------------------------------------------------------------ tile order
// A frame's tiles differ in cost by orders of magnitude (a tile crossed by a large
// shape against an empty one), and the persistent grid pulls units in list order, so
// the expensive tiles should start first.  Three small kernels build a cost-descending
// unit list on the device: a histogram of log2(cost) over the tiles, a prefix over the
// 32 buckets in descending order, and a scatter of every tile's units to its bucket's
// next slots (order within a bucket is arbitrary; the output does not depend on it).
// Cost: the strands of the tile's shapes plus its shape count, plus one.

__device__ __forceinline__ int tileBucket(const gudni_tile_info& ti, const gudni_shape* shapes, uint32_t n_shapes) {
  uint64_t cost = 1;
  if ((uint64_t)ti.shapes.start + ti.shapes.length <= n_shapes) {
    for (uint32_t i = 0; i < ti.shapes.length; ++i) cost += 1 + shapes[ti.shapes.start + i].num_strands;
  }
  return 63 - __clzll((long long)cost);  // 0..63
}

__global__ void tile_cost_hist_kernel(const gudni_tile_info* tiles, uint32_t n_tiles, const gudni_shape* shapes,
                                      uint32_t n_shapes, uint32_t* hist) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_tiles; t += gridDim.x * blockDim.x)
    atomicAdd(&hist[tileBucket(tiles[t], shapes, n_shapes)], 1u);
}

__global__ void tile_bucket_prefix_kernel(const uint32_t* hist, uint32_t* cursor) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    uint32_t acc = 0;
    for (int b = 63; b >= 0; --b) {  // most expensive bucket first
      cursor[b] = acc;
      acc += hist[b];
    }
  }
}

__global__ void tile_order_scatter_kernel(const gudni_tile_info* tiles, uint32_t n_tiles, const gudni_shape* shapes,
                                          uint32_t n_shapes, int chunk_log2, uint32_t* cursor, uint32_t* units) {
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_tiles; t += gridDim.x * blockDim.x) {
    const uint32_t pos = atomicAdd(&cursor[tileBucket(tiles[t], shapes, n_shapes)], 1u);
    for (uint32_t c = 0; c < (1u << chunk_log2); ++c)
      units[((size_t)pos << chunk_log2) + c] = (t << kChunkBits) | c;
  }
}

cudaError_t launch_tile_order(const gudni_tile_info* tiles, uint32_t n_tiles, const gudni_shape* shapes,
                              uint32_t n_shapes, int chunk_log2, uint32_t* words128, uint32_t* units,
                              cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(words128, 0, 128 * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  const int grid = (int)std::min<uint32_t>((n_tiles + 255) / 256, 1024u);
  tile_cost_hist_kernel<<<grid, 256, 0, stream>>>(tiles, n_tiles, shapes, n_shapes, words128);
  tile_bucket_prefix_kernel<<<1, 32, 0, stream>>>(words128, words128 + 64);
  tile_order_scatter_kernel<<<grid, 256, 0, stream>>>(tiles, n_tiles, shapes, n_shapes, chunk_log2, words128 + 64,
                                                       units);
  return cudaGetLastError();
}

int sections_for(int max_shape) {
  int need = (max_shape + 1 + 63) / 64;
  int s = 1;
  while (s < need) s *= 2;
  return s;
}

template <int S>
static cudaError_t launch_s(const TileLaunch& a, bool list, int grid, cudaStream_t stream) {
  if (list) {
    raster_list_kernel<S, false><<<grid, kRasterBlock, 0, stream>>>(a);
  } else if (a.dense_min > 0) {
    raster_tiles_warp_kernel<S><<<grid, kRasterBlock, 0, stream>>>(a);
  } else if (a.coop) {
    raster_tiles_coop_kernel<S><<<grid, kRasterBlock, 0, stream>>>(a);
  } else {
    raster_tiles_kernel<S, false><<<grid, kRasterBlock, 0, stream>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_raster(const TileLaunch& a, bool list, int sections, int grid, cudaStream_t stream) {
  // the counter-based jitter runs on its own instantiation of the per-lane kernels
  // (raster_counter.cu; the warp-cooperative scan of dense columns is not used then)
  if (a.in.random_mode == kRandomCounter && a.in.stochastic != 0.0f)
    return launch_raster_counter(a, list, sections, grid, stream);
  switch (sections) {
    case 1: return launch_s<1>(a, list, grid, stream);
    case 2: return launch_s<2>(a, list, grid, stream);
    case 4: return launch_s<4>(a, list, grid, stream);
    case 8: return launch_s<8>(a, list, grid, stream);
    case 16: return launch_s<16>(a, list, grid, stream);
    case 32: return launch_s<32>(a, list, grid, stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t raster_coop_occupancy(int sections, int* blocks_per_sm) {
  const void* fn = nullptr;
  switch (sections) {
    case 1: fn = (const void*)raster_tiles_coop_kernel<1>; break;
    case 2: fn = (const void*)raster_tiles_coop_kernel<2>; break;
    case 4: fn = (const void*)raster_tiles_coop_kernel<4>; break;
    case 8: fn = (const void*)raster_tiles_coop_kernel<8>; break;
    case 16: fn = (const void*)raster_tiles_coop_kernel<16>; break;
    case 32: fn = (const void*)raster_tiles_coop_kernel<32>; break;
    default: return cudaErrorInvalidValue;
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kRasterBlock, 0);
}

cudaError_t raster_occupancy(int sections, int* blocks_per_sm) {
  const void* fn = nullptr;
  switch (sections) {
    case 1: fn = (const void*)raster_tiles_kernel<1, false>; break;
    case 2: fn = (const void*)raster_tiles_kernel<2, false>; break;
    case 4: fn = (const void*)raster_tiles_kernel<4, false>; break;
    case 8: fn = (const void*)raster_tiles_kernel<8, false>; break;
    case 16: fn = (const void*)raster_tiles_kernel<16, false>; break;
    case 32: fn = (const void*)raster_tiles_kernel<32, false>; break;
    default: return cudaErrorInvalidValue;
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kRasterBlock, 0);
}

}  // namespace gudni
