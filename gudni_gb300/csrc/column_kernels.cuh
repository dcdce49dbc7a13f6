// The per-lane raster kernels (the fast pass and the full-capacity pass), shared by
// raster.cu, which instantiates them with the reference's random-field jitter, and
// raster_counter.cu, which instantiates them with the counter-based jitter
// (kCounterJitter, gudni_set_random_source); the two sets are compiled apart so that
// the default kernels are exactly the reference scan's.
#pragma once

#include <cuda_runtime.h>

#include "raster_device.cuh"
#include "raster_kernels.h"

namespace gudni {

// With a stack of at most two words the kernel is held to 72 registers (7 blocks of
// 128 threads per SM): the scan is latency-bound, and on the 4K page the extra resident
// warps outweigh the few spills (23.3 ms a frame against 24.8 ms at the 80 registers
// ptxas picks).  Wider stacks (hundreds of shapes per column) spill heavily at that
// bound (4x slower on 500 canvas-wide shapes) and keep ptxas's choice.
template <int SECTIONS>
constexpr int rasterMinBlocks() { return SECTIONS <= 2 ? 7 : 1; }

template <int SECTIONS, bool kCounterJitter>
__global__ void __launch_bounds__(kRasterBlock, rasterMinBlocks<SECTIONS>()) raster_tiles_kernel(TileLaunch a) {
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
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
    if (column < tpt) {
      if (runColumn<SECTIONS, kCounterJitter>(in, ti, column, thr, hdr, a.scratch.capacity, idx, status)) {
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
  }
  if (status) atomicOr(a.status, status);
}

template <int SECTIONS, bool kCounterJitter>
__global__ void __launch_bounds__(kRasterBlock) raster_list_kernel(TileLaunch a) {
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nslots = gridDim.x * blockDim.x;
  float4* thr = a.scratch.thr + (size_t)slot * (size_t)a.scratch.capacity;
  uint32_t* hdr = a.scratch.hdr + (size_t)slot * (size_t)a.scratch.capacity;
  uint32_t* idx = a.scratch.idx + (size_t)slot * (size_t)a.scratch.idx_stride;
  int status = 0;
  const uint32_t n_items = min(*a.list_count, a.list_cap);
  for (uint32_t w = slot; w < n_items; w += nslots) {
    const uint32_t item = a.list[w];
    int tile, chunk;
    unitOf(a.units, a.chunk_log2, item >> kLaneBits, tile, chunk);
    const int column = chunk * 32 + (int)(item & ((1u << kLaneBits) - 1u));
    bool ok;
    const RasterInputs in = sceneInputs(a.in, a.scenes, a.tile_scene, a.n_scenes, tile, status, ok);
    if (!ok) continue;
    const gudni_tile_info ti = in.tiles[tile];
    if (runColumn<SECTIONS, kCounterJitter>(in, ti, column, thr, hdr, a.scratch.capacity, idx, status)) status |= kStatusOverflow;
  }
  if (status) atomicOr(a.status, status);
}

}  // namespace gudni
