// Host-visible launch interface of the adjoint kernel (adjoint.cu).
#pragma once

#include <cuda_runtime.h>

#include "raster_kernels.h"

namespace gudni {

constexpr int kAdjointBlock = 128;

struct AdjointLaunch {
  RasterInputs in;
  const SceneInfo* scenes;
  const int32_t* tile_scene;
  uint32_t n_scenes;
  const uint32_t* units;  // optional unit list, as for the raster fast pass
  uint32_t n_units;
  int chunk_log2;
  uint32_t* next_tile;
  int capacity;           // thresholds (and lines) per column
  float4* thr;            // slots * capacity
  uint32_t* hdr;          // slots * capacity
  float4* thr_fwd;        // slots * capacity: the forward scan's copy of the sorted queue
  uint32_t* hdr_fwd;      // slots * capacity
  int regenerate;         // 1: the forward generates its own thresholds, the backward regenerates them
  int4* prov;             // slots * capacity
  void* lines;            // slots * capacity line records
  float4* line_grad;      // slots * capacity
  uint32_t* idx;          // slots * max_shape
  float4* bit_grad;       // slots * max_shape
  float4* layers;         // slots * 2 * (max_shape + 1): layer colours, composites in front
  int32_t* layer_bits;    // slots * (max_shape + 1)
  float4* image;          // per pixel: I rgb, section area sum
  const float4* target;   // per pixel: target rgb
  float* grad_geometry;   // per pile float (accumulated)
  float* grad_substances; // 4 per substance (accumulated)
  int* status;
};

cudaError_t launch_adjoint(const AdjointLaunch& a, int sections, int grid, cudaStream_t stream);
cudaError_t adjoint_occupancy(int sections, int* blocks_per_sm);
size_t adjoint_line_bytes();

}  // namespace gudni
