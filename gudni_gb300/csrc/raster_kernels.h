// Host-visible launch interface of the raster kernels (raster.cu).
#pragma once

#include <cuda_runtime.h>

#include "raster_device.cuh"

namespace gudni {

constexpr int kRasterBlock = 128;

struct ColumnScratch {
  float4* thr;       // slots * capacity threshold geometries
  uint32_t* hdr;     // slots * capacity headers
  uint32_t* idx;     // slots * idx_stride shape indices
  int capacity;      // queue entries per column in this launch
  int idx_stride;    // >= max_shape
};

struct ColumnLaunch {
  RasterInputs in;
  ColumnScratch scratch;
  const uint32_t* items;      // optional explicit work-item list
  uint32_t n_items;           // tiles * threads_per_tile, or the list's capacity
  const uint32_t* n_items_dev;  // optional: the list's length, read on the device
  uint32_t* overflow_items;   // where columns that overflow `capacity` are recorded
  uint32_t overflow_cap;
  uint32_t* overflow_count;
  int* status;                // kStatus* bits
};

int sections_for(int max_shape);
cudaError_t launch_columns(const ColumnLaunch& a, int sections, int grid, cudaStream_t stream);
cudaError_t columns_occupancy(int sections, int* blocks_per_sm);

}  // namespace gudni
