// Host-visible launch interface of the raster kernels (raster.cu).
#pragma once

#include <cuda_runtime.h>

#include "raster_device.cuh"

namespace gudni {

constexpr int kRasterBlock = 128;
constexpr int kColumnBits = 11;   // overflow-list items are (tile << 11) | column
constexpr int kMaxLog2Tpt = 10;   // up to 1024 threads per tile

struct ColumnScratch {
  float4* thr;       // slots * capacity threshold geometries
  uint32_t* hdr;     // slots * capacity headers
  uint32_t* idx;     // slots * idx_stride shape indices
  int capacity;      // queue entries per column in this launch
  int idx_stride;    // >= max_shape
};

// Per-scene part of the inputs when one launch renders several scenes.
struct SceneInfo {
  int32_t bitmap_w, bitmap_h;
  int32_t log2_tpt;       // threads per tile of this scene's spec
  int32_t job_index;
  uint64_t out_offset;    // first pixel of this scene in the output buffer
  float background[4];
};

struct TileLaunch {
  RasterInputs in;              // shared piles (+ the single scene when scenes == null)
  const SceneInfo* scenes;      // optional per-scene table
  const int32_t* tile_scene;    // scene of each tile (with scenes)
  uint32_t n_scenes;
  ColumnScratch scratch;
  // fast pass
  const uint32_t* order;        // optional tile order (cost-descending)
  uint32_t n_tiles;
  uint32_t* next_tile;          // work counter, zero at launch
  uint32_t* overflow_items;     // where columns that overflow `capacity` go
  uint32_t overflow_cap;
  uint32_t* overflow_count;
  // full-capacity pass
  const uint32_t* list;         // overflowed columns
  const uint32_t* list_count;   // their number (device)
  uint32_t list_cap;
  int* status;                  // kStatus* bits
};

int sections_for(int max_shape);
cudaError_t launch_raster(const TileLaunch& a, bool list, int sections, int grid, cudaStream_t stream);
cudaError_t raster_occupancy(int sections, int* blocks_per_sm);

}  // namespace gudni
