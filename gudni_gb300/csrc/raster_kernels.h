// Host-visible launch interface of the raster kernels (raster.cu).
#pragma once

#include <cuda_runtime.h>

#include "raster_device.cuh"

namespace gudni {

constexpr int kRasterBlock = 128;
constexpr int kLaneBits = 5;      // overflow-list items are (work unit << 5) | lane
constexpr uint64_t kMaxUnits = 1ull << 27;  // work units per launch (items fit 32 bits)
constexpr int kMaxLog2Tpt = 10;   // up to 1024 threads per tile
constexpr int kChunkBits = 5;     // work units are (tile << 5) | chunk of 32 columns

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
  // fast pass: work units of 32 columns of one tile, pulled from a counter
  const uint32_t* units;        // optional unit list ((tile << kChunkBits) | chunk), cost-descending
  uint32_t n_units;             // units in the launch
  int chunk_log2;               // without a list: unit k is tile k >> chunk_log2, chunk k & mask
  uint32_t* next_tile;          // work counter, zero at launch
  uint32_t* overflow_items;     // where columns that overflow `capacity` go
  uint32_t overflow_cap;
  uint32_t* overflow_count;
  int dense_min;                // > 0: columns with at least this many thresholds are
                                // scanned by the whole warp (raster_tiles_warp_kernel)
  int coop;                     // != 0: warp-cooperative units (raster_tiles_coop_kernel)
  // full-capacity pass
  const uint32_t* list;         // overflowed columns
  const uint32_t* list_count;   // their number (device)
  uint32_t list_cap;
  int* status;                  // kStatus* bits
};

// Work unit k of a launch: its tile and its chunk of 32 columns.
__device__ __forceinline__ void unitOf(const uint32_t* units, int chunk_log2, uint32_t k, int& tile, int& chunk) {
  if (units) {
    const uint32_t u = units[k];
    tile = (int)(u >> kChunkBits);
    chunk = (int)(u & ((1u << kChunkBits) - 1u));
  } else {
    tile = (int)(k >> chunk_log2);
    chunk = (int)(k & ((1u << chunk_log2) - 1u));
  }
}

// log2 of the 32-column chunks of a tile with 2^log2_tpt columns
__host__ __device__ __forceinline__ int chunkLog2(int log2_tpt) { return log2_tpt > 5 ? log2_tpt - 5 : 0; }

__device__ __forceinline__ bool tileOk(const gudni_tile_info& ti, uint32_t n_shapes) {
  return ti.hdepth >= 0 && ti.hdepth <= 24 && ti.vdepth >= 0 && ti.vdepth <= 24 && ti.left >= 0 &&
         ti.top >= 0 && ti.right >= ti.left && ti.bottom >= ti.top &&
         (uint64_t)ti.shapes.start + (uint64_t)ti.shapes.length <= (uint64_t)n_shapes;
}

// The inputs of tile `tile`: the shared piles plus its scene's canvas, output,
// background, threads per tile and job index.
__device__ __forceinline__ RasterInputs sceneInputs(const RasterInputs& base, const SceneInfo* scenes,
                                                    const int32_t* tile_scene, uint32_t n_scenes, int tile,
                                                    int& status, bool& ok) {
  RasterInputs in = base;
  ok = true;
  if (scenes) {
    const uint32_t s = (uint32_t)tile_scene[tile];
    if (s >= n_scenes) {
      status |= kStatusBadInput;
      ok = false;
      return in;
    }
    const SceneInfo sc = scenes[s];
    in.bitmap_w = sc.bitmap_w;
    in.bitmap_h = sc.bitmap_h;
    in.log2_tpt = sc.log2_tpt;
    in.job_index = sc.job_index;
    in.out = base.out + sc.out_offset;
    in.background = make_float4(sc.background[0], sc.background[1], sc.background[2], sc.background[3]);
  } else if (base.tile_jobs) {
    in.job_index = base.tile_jobs[tile];
  }
  return in;
}

int sections_for(int max_shape);
cudaError_t launch_raster(const TileLaunch& a, bool list, int sections, int grid, cudaStream_t stream);
// the same kernels with the counter-based jitter (raster_counter.cu)
cudaError_t launch_raster_counter(const TileLaunch& a, bool list, int sections, int grid, cudaStream_t stream);
// Cost-descending work units of a frame's tiles (3 launches); words128: 128 words of
// scratch (bucket counts and cursors), units: n_tiles << chunk_log2 entries.
cudaError_t launch_tile_order(const gudni_tile_info* tiles, uint32_t n_tiles, const gudni_shape* shapes,
                              uint32_t n_shapes, int chunk_log2, uint32_t* words128, uint32_t* units,
                              cudaStream_t stream);
cudaError_t raster_occupancy(int sections, int* blocks_per_sm);
cudaError_t raster_coop_occupancy(int sections, int* blocks_per_sm);

}  // namespace gudni
