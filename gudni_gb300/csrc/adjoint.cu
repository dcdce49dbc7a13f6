// Adjoint of the raster path (sm_103a): gradients of the per-pixel L2 loss
//   L = sum_p sum_{c in RGB} (I_c(p) - T_c(p))^2,   I(p) = sum_s col_s a_s / sum_s a_s
// (the pixel colour before the byte conversion, Kernels.cl:1897-1904, 2017) with respect
// to every float of the geometry pile and every solid substance colour.
//
// Each column runs twice, start to finish, in one thread:
//   pass 1  the raster kernel's own generate / order / render, writing I(p) and the
//           pixel's section area sum A(p) instead of bytes;
//   pass 2  the thresholds are generated again (recomputed, not stored), now with
//           provenance -- every threshold remembers the line it lies on, whose two end
//           points are either strand points of the pile or intercepts of a de
//           Casteljau sub-curve with a column border (K:1226-1333), and every section
//           y-bound remembers the line end point it came from -- and the same scan
//           accumulates dL/d(line end points) through the boundary terms of the
//           coverage integral,
//             a_s = (x1 - x0)(y1 - y0),  x = X_line((y0 + y1)/2)  (K:916-926),
//           and dL/d(colours) back through the front-to-back composite chain
//           (K:878-887, 1447-1513).
// At the column's end, line end-point gradients are carried to pile floats (strand
// points directly; intercepts through the sub-curve's Bernstein weights and the
// intercept's partials) and colour gradients per shape bit to their substances, with
// one atomicAdd each.  Discrete choices (which shapes cover a section, bifurcation
// branches, threshold keep/drop) are those of the forward pass and carry no gradient.
//
// The forward decisions of both passes are bit-identical to raster_tiles_kernel's.

#include <cuda_runtime.h>

#include "adjoint_device.cuh"
#include "adjoint_kernels.h"
#include "raster_device.cuh"
#include "raster_kernels.h"

namespace gudni {

namespace {

// Add v to base[idx] for every lane of the (converged, full) warp, one atomic per
// distinct index: neighbouring columns carry gradient to the same curve points, and
// aggregating first removes most of the contention on them.  idx < 0: nothing.
__device__ __forceinline__ void warpAdd(float* base, int32_t idx, float v) {
  const unsigned peers = __match_any_sync(0xffffffffu, idx);
  if (idx < 0) return;
  float sum = 0.0f;
  for (unsigned p = peers; p != 0u; p &= p - 1u) sum += __shfl_sync(peers, v, __ffs((int)p) - 1);
  if ((int)(threadIdx.x & 31u) == __ffs((int)peers) - 1 && sum != 0.0f) atomicAdd(&base[idx], sum);
}

// Carry every lane's line and colour gradients to the pile and substance gradients;
// called by the whole warp together.
__device__ void warpChain(const RasterInputs& in, const AdjSlot& s, int nLines, int nBits, float2 delta,
                          float* gGeo, float* gSub) {
  const float* pile = reinterpret_cast<const float*>(in.geometry);
  const int maxLines = (int)__reduce_max_sync(0xffffffffu, (unsigned)nLines);
  for (int i = 0; i < maxLines; ++i) {
    int32_t idx[2 * kEpTargets];
    float val[2 * kEpTargets];
    if (i < nLines) {
      const float4 lg = s.lineGrad[i];
      epTargets(s.lines[i].a, lg.x, lg.y, pile, delta, idx, val);
      epTargets(s.lines[i].b, lg.z, lg.w, pile, delta, idx + kEpTargets, val + kEpTargets);
    } else {
#pragma unroll
      for (int k = 0; k < 2 * kEpTargets; ++k) {
        idx[k] = -1;
        val[k] = 0.0f;
      }
    }
#pragma unroll
    for (int k = 0; k < 2 * kEpTargets; ++k) warpAdd(gGeo, idx[k], val[k]);
  }
  const int maxBits = (int)__reduce_max_sync(0xffffffffu, (unsigned)nBits);
  for (int b = 0; b < maxBits; ++b) {
    int32_t sub = -1;
    float4 bg = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (b < nBits) {
      bg = s.bitGrad[b];
      const uint64_t sid = in.shapes[s.idx[b]].tag & GUDNI_TAG_ID_MASK;
      if ((bg.x != 0.0f || bg.y != 0.0f || bg.z != 0.0f || bg.w != 0.0f) && sid < in.n_substances) sub = (int32_t)sid;
    }
    warpAdd(gSub, sub < 0 ? -1 : 4 * sub + 0, bg.x);
    warpAdd(gSub, sub < 0 ? -1 : 4 * sub + 1, bg.y);
    warpAdd(gSub, sub < 0 ? -1 : 4 * sub + 2, bg.z);
    warpAdd(gSub, sub < 0 ? -1 : 4 * sub + 3, bg.w);
  }
}

}  // namespace

template <int SECTIONS>
__global__ void __launch_bounds__(kAdjointBlock) adjoint_tiles_kernel(AdjointLaunch a) {
  const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const size_t cap = (size_t)a.capacity;
  AdjSlot s;
  s.cap = a.capacity;
  s.thr = a.thr + slot * cap;
  s.hdr = a.hdr + slot * cap;
  s.thrFwd = a.thr_fwd + slot * cap;
  s.hdrFwd = a.hdr_fwd + slot * cap;
  s.prov = a.prov + slot * cap;
  s.lines = reinterpret_cast<LineRec*>(a.lines) + slot * cap;
  s.lineGrad = a.line_grad + slot * cap;
  s.idx = a.idx + (size_t)slot * (size_t)a.in.max_shape;
  s.bitGrad = a.bit_grad + (size_t)slot * (size_t)a.in.max_shape;
  s.layerCap = a.in.max_shape + 1;
  // layer records interleaved across the warp's lanes: lane l's k-th at [k * 32 + l]
  s.ls = 32;
  const size_t warpBase = (size_t)(slot & ~31u);
  s.layer = a.layers + warpBase * 2 * (size_t)s.layerCap + lane;
  s.front = s.layer + 32 * (size_t)s.layerCap;
  s.layerBit = a.layer_bits + warpBase * (size_t)s.layerCap + lane;
  int status = 0;
  for (;;) {
    uint32_t k = 0;
    if (lane == 0) k = atomicAdd(a.next_tile, 1u);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= a.n_units) break;
    int tile, chunk;
    unitOf(a.units, a.chunk_log2, k, tile, chunk);
    bool ok;
    RasterInputs in = sceneInputs(a.in, a.scenes, a.tile_scene, a.n_scenes, tile, status, ok);
    if (!ok) continue;
    const gudni_tile_info ti = in.tiles[tile];
    if (!tileOk(ti, in.n_shapes) || in.log2_tpt < 0 || in.log2_tpt > kMaxLog2Tpt) {
      status |= kStatusBadInput;
      continue;
    }
    // image and target of this tile's scene (float4 per pixel, same offsets as out)
    const size_t base = a.scenes ? (size_t)a.scenes[a.tile_scene[tile]].out_offset : 0;
    const int tpt = 1 << in.log2_tpt;
    const int column = chunk * 32 + lane;
    int nLines = 0, nBits = 0;
    float2 delta = make_float2(0.0f, 0.0f);
    if (column < tpt) {
      if (adjointColumn<SECTIONS>(in, ti, column, s, a.image + base, a.target + base, a.regenerate != 0, nLines,
                                  nBits, delta, status))
        status |= kStatusOverflow;
    }
    warpChain(in, s, nLines, nBits, delta, a.grad_geometry, a.grad_substances);  // all 32 lanes
  }
  if (status) atomicOr(a.status, status);
}

template <int S>
static cudaError_t adj_launch_s(const AdjointLaunch& a, int grid, cudaStream_t stream) {
  adjoint_tiles_kernel<S><<<grid, kAdjointBlock, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_adjoint(const AdjointLaunch& a, int sections, int grid, cudaStream_t stream) {
  switch (sections) {
    case 1: return adj_launch_s<1>(a, grid, stream);
    case 2: return adj_launch_s<2>(a, grid, stream);
    case 4: return adj_launch_s<4>(a, grid, stream);
    case 8: return adj_launch_s<8>(a, grid, stream);
    case 16: return adj_launch_s<16>(a, grid, stream);
    case 32: return adj_launch_s<32>(a, grid, stream);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t adjoint_occupancy(int sections, int* blocks_per_sm) {
  const void* fn = nullptr;
  switch (sections) {
    case 1: fn = (const void*)adjoint_tiles_kernel<1>; break;
    case 2: fn = (const void*)adjoint_tiles_kernel<2>; break;
    case 4: fn = (const void*)adjoint_tiles_kernel<4>; break;
    case 8: fn = (const void*)adjoint_tiles_kernel<8>; break;
    case 16: fn = (const void*)adjoint_tiles_kernel<16>; break;
    case 32: fn = (const void*)adjoint_tiles_kernel<32>; break;
    default: return cudaErrorInvalidValue;
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, kAdjointBlock, 0);
}

size_t adjoint_line_bytes() { return sizeof(LineRec); }

}  // namespace gudni
