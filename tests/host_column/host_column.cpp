// TEST INFRASTRUCTURE -- not part of the product and never loaded by it.
//
// The product's device column machine (gudni_gb300/csrc/raster_device.cuh) compiled
// for the host CPU, so that its exact-arithmetic transformations (strand-table range
// test and y culling, batched insertion and merge of split parts, opaque-cut colour
// memo, one-word stack) can be checked against the oracle without a GPU.  The CUDA
// qualifiers and the few intrinsics the header uses get host definitions below; the
// floating-point expressions are compiled with IEEE single precision and no
// contraction, as the CUDA build is.  Columns run one after another on one thread.

#include <cuda_runtime.h>  // vector types and make_* (host-usable)

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

using std::isnan;

static inline int __clzll(long long x) { return x ? __builtin_clzll((unsigned long long)x) : 64; }
static inline int __clz(int x) { return x ? __builtin_clz((unsigned)x) : 32; }
static inline unsigned __float_as_uint(float f) {
  unsigned u;
  std::memcpy(&u, &f, 4);
  return u;
}
static inline float __uint_as_float(unsigned u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
static inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) {
  const unsigned long long o = *p;
  *p = o + v;
  return o;
}
static inline int max(int a, int b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline unsigned long long atomicMax(unsigned long long* p, unsigned long long v) {
  const unsigned long long o = *p;
  if (v > o) *p = v;
  return o;
}

#include "../../gudni_gb300/csrc/raster_device.cuh"
#include "../../gudni_gb300/csrc/strand_table.h"

namespace {

template <int SECTIONS>
int run_all(const gudni::RasterInputs& in, const gudni_tile_info* tiles, int n_tiles, int tpt, int cap,
            int* overflow) {
  std::vector<float4> thr((size_t)cap);
  std::vector<uint32_t> hdr((size_t)cap);
  std::vector<uint32_t> idx((size_t)in.max_shape + 1);
  int status = 0;
  for (int t = 0; t < n_tiles; ++t) {
    for (int column = 0; column < tpt; ++column) {
      if (gudni::runColumn<SECTIONS>(in, tiles[t], column, thr.data(), hdr.data(), cap, idx.data(), status))
        *overflow = 1;
    }
  }
  return status;
}

}  // namespace

// One job, as gudni_raster_job does it, on the host.  Returns the kernel status bits
// (0 when clean); *overflow is set when a column needed more than max_thresholds.
extern "C" int host_column_raster_job(const uint8_t* geometry, size_t geometry_bytes, const float* substances,
                                      size_t n_substances, const uint8_t* pictures, size_t picture_bytes,
                                      const gudni_picture_use* uses, size_t n_uses, const gudni_radial* radials,
                                      size_t n_radials, const gudni_shape* shapes, size_t n_shapes,
                                      const gudni_tile_info* tiles, int n_tiles, int compute_depth, int bitmap_w,
                                      int bitmap_h, int job_index, const float* background, int max_thresholds,
                                      int max_shape, uint32_t* out, int* overflow) {
  std::vector<uint4> table;
  std::vector<float2> ys;
  std::vector<uint32_t> first;
  gudni::build_strand_table(geometry, geometry_bytes, table, ys, first);
  gudni::RasterInputs in;
  std::memset(&in, 0, sizeof(in));
  in.geometry = geometry;
  in.geometry_bytes = geometry_bytes;
  in.substances = reinterpret_cast<const float4*>(substances);
  in.n_substances = (uint32_t)n_substances;
  in.pictures = pictures;
  in.picture_bytes = picture_bytes;
  in.uses = uses;
  in.n_uses = (uint32_t)n_uses;
  in.radials = radials;
  in.n_radials = (uint32_t)n_radials;
  in.random_field = nullptr;
  in.stochastic = 0.0f;
  in.shapes = shapes;
  in.n_shapes = (uint32_t)n_shapes;
  in.tiles = tiles;
  in.n_tiles = n_tiles;
  in.log2_tpt = compute_depth;
  in.bitmap_w = bitmap_w;
  in.bitmap_h = bitmap_h;
  in.job_index = job_index;
  in.background = make_float4(background[0], background[1], background[2], background[3]);
  in.max_shape = max_shape;
  in.out = out;
  in.tile_jobs = nullptr;
  in.counters = nullptr;
  in.strand_table = table.empty() ? nullptr : table.data();
  in.strand_y = ys.empty() ? nullptr : ys.data();
  in.n_strands = (uint32_t)table.size();
  in.strand_first = first.data();
  in.n_units = (uint32_t)first.size();
  *overflow = 0;
  const int tpt = 1 << compute_depth;
  int sections = 1;  // stack words for max_shape, a power of two (as the CUDA launch picks them)
  while (64 * sections < max_shape + 1) sections *= 2;
  switch (sections) {
    case 1: return run_all<1>(in, tiles, n_tiles, tpt, max_thresholds, overflow);
    case 2: return run_all<2>(in, tiles, n_tiles, tpt, max_thresholds, overflow);
    case 4: return run_all<4>(in, tiles, n_tiles, tpt, max_thresholds, overflow);
    case 8: return run_all<8>(in, tiles, n_tiles, tpt, max_thresholds, overflow);
    case 16: return run_all<16>(in, tiles, n_tiles, tpt, max_thresholds, overflow);
    case 32: return run_all<32>(in, tiles, n_tiles, tpt, max_thresholds, overflow);
    default: return -1;
  }
}
