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

#include "warp_emu.h"

// how often each path of the warp-cooperative band step ran (GUDNI_WARP_TRACE)
static long long g_warp_trace[8];
#define GUDNI_WARP_TRACE(event) (g_warp_trace[(event)] += 1)

// warp collectives on the emulated warp
static inline void __syncwarp(unsigned = 0xffffffffu) { warp_emu::collective(warp_emu::kSync, 0u, 0); }
static inline unsigned __shfl_sync(unsigned, unsigned v, int src) {
  return warp_emu::collective(warp_emu::kShfl, v, src);
}
static inline int __shfl_sync(unsigned, int v, int src) {
  return (int)warp_emu::collective(warp_emu::kShfl, (unsigned)v, src);
}
static inline float __shfl_sync(unsigned, float v, int src) {
  return __uint_as_float(warp_emu::collective(warp_emu::kShfl, __float_as_uint(v), src));
}
static inline float __shfl_up_sync(unsigned, float v, unsigned delta) {
  return __uint_as_float(warp_emu::collective(warp_emu::kShflUp, __float_as_uint(v), (int)delta));
}
static inline unsigned __ballot_sync(unsigned, int pred) {
  return warp_emu::collective(warp_emu::kBallot, pred ? 1u : 0u, 0);
}
static inline float __shfl_xor_sync(unsigned, float v, int mask) {
  return __uint_as_float(warp_emu::collective(warp_emu::kShflXor, __float_as_uint(v), mask));
}
static inline int __shfl_xor_sync(unsigned, int v, int mask) {
  return (int)warp_emu::collective(warp_emu::kShflXor, (unsigned)v, mask);
}
static inline int __ffs(int x) { return __builtin_ffs(x); }
static inline int __ffsll(long long x) { return __builtin_ffsll(x); }
static inline int __popcll(unsigned long long x) { return __builtin_popcountll(x); }
static inline unsigned __match_any_sync(unsigned, unsigned v) {
  return warp_emu::collective(warp_emu::kMatch, v, 0);
}
static inline bool __all_sync(unsigned, int pred) {
  return warp_emu::collective(warp_emu::kBallot, pred ? 1u : 0u, 0) == 0xffffffffu;
}
static inline bool __any_sync(unsigned, int pred) {
  return warp_emu::collective(warp_emu::kBallot, pred ? 1u : 0u, 0) != 0u;
}
static inline unsigned __shfl_up_sync(unsigned, unsigned v, unsigned delta) {
  return warp_emu::collective(warp_emu::kShflUp, v, (int)delta);
}
static inline unsigned long long atomicOr(unsigned long long* p, unsigned long long v) {
  const unsigned long long o = *p;
  *p = o | v;
  return o;
}
static inline unsigned long long atomicXor(unsigned long long* p, unsigned long long v) {
  const unsigned long long o = *p;
  *p = o ^ v;
  return o;
}
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
// shared-memory atomics: lanes run one at a time between collectives
static inline unsigned atomicXor(unsigned* p, unsigned v) {
  const unsigned o = *p;
  *p = o ^ v;
  return o;
}

#include "../../gudni_gb300/csrc/raster_device.cuh"
#include "../../gudni_gb300/csrc/adjoint_device.cuh"
#include "../../gudni_gb300/csrc/strand_table.h"
#include "../../gudni_gb300/csrc/warp_column.cuh"
#include "../../gudni_gb300/csrc/tile_coop.cuh"

namespace {

// jitter source of the following host_column_* calls (host_set_random_source)
uint32_t g_random_mode = gudni::kRandomField;
uint64_t g_random_seed = 0;

template <int SECTIONS>
int run_all(const gudni::RasterInputs& in, const gudni_tile_info* tiles, int n_tiles, int tpt, int cap,
            int* overflow) {
  std::vector<float4> thr((size_t)cap);
  std::vector<uint32_t> hdr((size_t)cap);
  std::vector<uint32_t> idx((size_t)in.max_shape + 1);
  int status = 0;
  for (int t = 0; t < n_tiles; ++t) {
    for (int column = 0; column < tpt; ++column) {
      const bool over = in.random_mode == gudni::kRandomCounter && in.stochastic != 0.0f
                            ? gudni::runColumn<SECTIONS, true>(in, tiles[t], column, thr.data(), hdr.data(), cap,
                                                               idx.data(), status)
                            : gudni::runColumn<SECTIONS>(in, tiles[t], column, thr.data(), hdr.data(), cap,
                                                         idx.data(), status);
      if (over) *overflow = 1;
    }
  }
  return status;
}

// The warp-cooperative form: every work unit (32 columns of a tile) on an emulated
// warp, the lanes resuming in a seeded random order at each collective; columns that
// overflow the working capacity `cap` are re-run by the per-lane path with
// `full_cap`, as the full-capacity pass does.
template <int SECTIONS>
int run_all_warp(const gudni::RasterInputs& in, const gudni_tile_info* tiles, int n_tiles, int tpt, int cap,
                 int full_cap, int dense_min, uint64_t seed, int* overflow, int* by_warp) {
  const size_t idxStride = (size_t)in.max_shape + 1;
  std::vector<float4> thr(32 * (size_t)cap), big((size_t)full_cap);
  std::vector<uint32_t> hdr(32 * (size_t)cap), bigH((size_t)full_cap);
  std::vector<uint32_t> idx(32 * idxStride);
  float4 prod[32];
  uint32_t bits[32];
  uint32_t flips[gudni::kWarpFlipWords];
  const gudni::WarpScratch ws{prod, bits, flips};
  int status = 0;
  for (int t = 0; t < n_tiles; ++t) {
    for (int chunk = 0; chunk * 32 < tpt; ++chunk) {
      int flags[32] = {0};
      int laneStatus[32] = {0};
      const std::function<void(int)> body = [&](int lane) {
        const int column = chunk * 32 + lane;
        int st = 0;
        flags[lane] = gudni::runUnitWarp<SECTIONS>(in, tiles[t], column, column < tpt,
                                                   thr.data() + (size_t)lane * cap, hdr.data() + (size_t)lane * cap,
                                                   cap, idx.data() + (size_t)lane * idxStride, st, lane, dense_min,
                                                   ws);
        laneStatus[lane] = st;
      };
      if (!warp_emu::run(body, seed * 1000003ull + (uint64_t)t * 64u + (uint64_t)chunk)) return -100;
      for (int lane = 0; lane < 32; ++lane) {
        status |= laneStatus[lane];
        if (flags[lane] & gudni::kUnitByWarp) *by_warp += 1;
        if (flags[lane] & gudni::kUnitOverflow) {
          if (gudni::runColumn<SECTIONS>(in, tiles[t], chunk * 32 + lane, big.data(), bigH.data(), full_cap,
                                         idx.data(), status))
            *overflow = 1;
        }
      }
    }
  }
  return status;
}

// The warp-cooperative units (tile_coop.cuh): every work unit on an emulated warp,
// the lanes resuming in a seeded random order at each collective; units that do not
// qualify run the per-column code on their lanes, and columns that overflow the
// working capacity `cap` are re-run by the per-column code with `full_cap`, as the
// kernel and the full-capacity pass do.  *taken counts the units run cooperatively.
template <int SECTIONS>
int run_all_coop(const gudni::RasterInputs& in, const gudni_tile_info* tiles, int n_tiles, int tpt, int cap,
                 int full_cap, uint64_t seed, int* overflow, int* taken) {
  const size_t idxStride = (size_t)in.max_shape + 1;
  std::vector<float4> thr(32 * (size_t)cap, make_float4(-7.0f, -7.0f, -7.0f, -7.0f)), big((size_t)full_cap);
  std::vector<uint32_t> hdr(32 * (size_t)cap, 0xDEADBEEFu), bigH((size_t)full_cap);
  std::vector<uint32_t> idx(32 * idxStride);
  gudni::CoopShared* sh = new gudni::CoopShared;
  std::memset(sh, 0x5A, sizeof(*sh));
  int status = 0;
  for (int t = 0; t < n_tiles; ++t) {
    for (int chunk = 0; chunk * 32 < tpt; ++chunk) {
      int flags[32] = {0};
      int laneStatus[32] = {0};
      uint32_t phases[32] = {0};
      const std::function<void(int)> body = [&](int lane) {
        int st = 0;
        flags[lane] = gudni::runUnitCoop(in, tiles[t], chunk, lane, thr.data(), hdr.data(), cap, st, *sh,
                                         phases[lane]);
        laneStatus[lane] = st;
      };
      if (!warp_emu::run(body, seed * 1000003ull + (uint64_t)t * 64u + (uint64_t)chunk)) {
        delete sh;
        return -100;
      }
      if (!(flags[0] & gudni::kCoopNotTaken)) *taken += 1;
      for (int lane = 0; lane < 32; ++lane) {
        status |= laneStatus[lane];
        const int column = chunk * 32 + lane;
        if (column >= tpt) continue;
        if (flags[lane] & gudni::kCoopNotTaken) {
          if (gudni::runColumn<SECTIONS>(in, tiles[t], column, thr.data() + (size_t)lane * cap,
                                         hdr.data() + (size_t)lane * cap, cap, idx.data() + (size_t)lane * idxStride,
                                         status)) {
            if (gudni::runColumn<SECTIONS>(in, tiles[t], column, big.data(), bigH.data(), full_cap, idx.data(),
                                           status))
              *overflow = 1;
          }
        } else if (flags[lane] & gudni::kCoopOverflow) {
          if (gudni::runColumn<SECTIONS>(in, tiles[t], column, big.data(), bigH.data(), full_cap, idx.data(),
                                         status))
            *overflow = 1;
        }
      }
    }
  }
  delete sh;
  return status;
}

}  // namespace

struct HostTables {
  std::vector<uint4> table;
  std::vector<float2> ys;
  std::vector<uint32_t> first;
};

static gudni::RasterInputs host_inputs(HostTables& t, const uint8_t* geometry, size_t geometry_bytes,
                                       const float* substances, size_t n_substances, const uint8_t* pictures,
                                       size_t picture_bytes, const gudni_picture_use* uses, size_t n_uses,
                                       const gudni_radial* radials, size_t n_radials, const gudni_shape* shapes,
                                       size_t n_shapes, const gudni_tile_info* tiles, int n_tiles, int compute_depth,
                                       int bitmap_w, int bitmap_h, int job_index, const float* background,
                                       int max_shape, uint32_t* out) {
  gudni::build_strand_table(geometry, geometry_bytes, t.table, t.ys, t.first);
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
  in.strand_table = t.table.empty() ? nullptr : t.table.data();
  in.strand_y = t.ys.empty() ? nullptr : t.ys.data();
  in.n_strands = (uint32_t)t.table.size();
  in.strand_first = t.first.data();
  in.n_units = (uint32_t)t.first.size();
  in.random_mode = g_random_mode;
  in.random_seed = g_random_seed;
  return in;
}

static int stack_words(int max_shape) {
  int sections = 1;  // stack words for max_shape, a power of two (as the CUDA launch picks them)
  while (64 * sections < max_shape + 1) sections *= 2;
  return sections;
}

static int g_adjoint_regenerate = 0;  // host_column_set_adjoint_regenerate

extern "C" void host_column_set_adjoint_regenerate(int on) { g_adjoint_regenerate = on ? 1 : 0; }

template <int SECTIONS>
static int adjoint_all(const gudni::RasterInputs& in, const gudni_tile_info* tiles, int n_tiles, int tpt, int cap,
                       float4* image, const float4* target, float* gGeo, float* gSub, int* overflow) {
  const int layerCap = in.max_shape + 1;
  std::vector<float4> thr((size_t)cap), thrFwd((size_t)cap), lineGrad((size_t)cap), bitGrad((size_t)in.max_shape + 1);
  std::vector<uint32_t> hdr((size_t)cap), hdrFwd((size_t)cap), idx((size_t)in.max_shape + 1);
  std::vector<int4> prov((size_t)cap);
  std::vector<gudni::LineRec> lines((size_t)cap);
  std::vector<float4> layers(2 * (size_t)layerCap);
  std::vector<int32_t> layerBits((size_t)layerCap);
  gudni::AdjSlot s;
  s.thr = thr.data();
  s.hdr = hdr.data();
  s.thrFwd = thrFwd.data();
  s.hdrFwd = hdrFwd.data();
  s.prov = prov.data();
  s.lines = lines.data();
  s.lineGrad = lineGrad.data();
  s.idx = idx.data();
  s.bitGrad = bitGrad.data();
  s.layer = layers.data();
  s.front = layers.data() + layerCap;
  s.layerBit = layerBits.data();
  s.cap = cap;
  s.layerCap = layerCap;
  s.ls = 1;
  const float* pile = reinterpret_cast<const float*>(in.geometry);
  int status = 0;
  for (int t = 0; t < n_tiles; ++t) {
    for (int column = 0; column < tpt; ++column) {
      int nLines = 0, nBits = 0;
      float2 delta = make_float2(0.0f, 0.0f);
      if (gudni::adjointColumn<SECTIONS>(in, tiles[t], column, s, image, target, g_adjoint_regenerate != 0, nLines,
                                         nBits, delta, status))
        *overflow = 1;
      // the kernel's warp gathering, one lane at a time
      for (int i = 0; i < nLines; ++i) {
        int32_t ix[2 * gudni::kEpTargets];
        float v[2 * gudni::kEpTargets];
        gudni::epTargets(lines[i].a, lineGrad[i].x, lineGrad[i].y, pile, delta, ix, v);
        gudni::epTargets(lines[i].b, lineGrad[i].z, lineGrad[i].w, pile, delta, ix + gudni::kEpTargets,
                         v + gudni::kEpTargets);
        for (int k = 0; k < 2 * gudni::kEpTargets; ++k)
          if (ix[k] >= 0) gGeo[ix[k]] += v[k];
      }
      for (int b = 0; b < nBits; ++b) {
        const uint64_t sid = in.shapes[idx[b]].tag & GUDNI_TAG_ID_MASK;
        if (sid >= in.n_substances) continue;
        gSub[4 * sid + 0] += bitGrad[b].x;
        gSub[4 * sid + 1] += bitGrad[b].y;
        gSub[4 * sid + 2] += bitGrad[b].z;
        gSub[4 * sid + 3] += bitGrad[b].w;
      }
    }
  }
  return status;
}

// One job's adjoint, as gudni_adjoint_tiles_device computes it, on the host: image
// (W*H float4: I rgb, section-area sum), gradients ADDED to gGeo / gSub.
extern "C" int host_column_adjoint_job(const uint8_t* geometry, size_t geometry_bytes, const float* substances,
                                       size_t n_substances, const uint8_t* pictures, size_t picture_bytes,
                                       const gudni_picture_use* uses, size_t n_uses, const gudni_radial* radials,
                                       size_t n_radials, const gudni_shape* shapes, size_t n_shapes,
                                       const gudni_tile_info* tiles, int n_tiles, int compute_depth, int bitmap_w,
                                       int bitmap_h, int job_index, const float* background, int capacity,
                                       int max_shape, const float* target, float* image, float* grad_geometry,
                                       float* grad_substances, int* overflow) {
  HostTables t;
  gudni::RasterInputs in = host_inputs(t, geometry, geometry_bytes, substances, n_substances, pictures,
                                       picture_bytes, uses, n_uses, radials, n_radials, shapes, n_shapes, tiles,
                                       n_tiles, compute_depth, bitmap_w, bitmap_h, job_index, background, max_shape,
                                       nullptr);
  *overflow = 0;
  const int tpt = 1 << compute_depth;
  float4* img = reinterpret_cast<float4*>(image);
  const float4* tg = reinterpret_cast<const float4*>(target);
  switch (stack_words(max_shape)) {
    case 1: return adjoint_all<1>(in, tiles, n_tiles, tpt, capacity, img, tg, grad_geometry, grad_substances, overflow);
    case 2: return adjoint_all<2>(in, tiles, n_tiles, tpt, capacity, img, tg, grad_geometry, grad_substances, overflow);
    case 4: return adjoint_all<4>(in, tiles, n_tiles, tpt, capacity, img, tg, grad_geometry, grad_substances, overflow);
    case 8: return adjoint_all<8>(in, tiles, n_tiles, tpt, capacity, img, tg, grad_geometry, grad_substances, overflow);
    default: return -1;
  }
}

// One job, as gudni_raster_job does it, on the host.  Returns the kernel status bits
// (0 when clean); *overflow is set when a column needed more than max_thresholds.
extern "C" int host_column_raster_job(const uint8_t* geometry, size_t geometry_bytes, const float* substances,
                                      size_t n_substances, const uint8_t* pictures, size_t picture_bytes,
                                      const gudni_picture_use* uses, size_t n_uses, const gudni_radial* radials,
                                      size_t n_radials, const gudni_shape* shapes, size_t n_shapes,
                                      const gudni_tile_info* tiles, int n_tiles, int compute_depth, int bitmap_w,
                                      int bitmap_h, int job_index, const float* background,
                                      const float* random_field, float stochastic, int max_thresholds,
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
  in.random_field = random_field;
  in.stochastic = stochastic;
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
  in.random_mode = g_random_mode;
  in.random_seed = g_random_seed;
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

// The strand table of a pile built with `threads` host threads, copied out (at most
// `cap` strands); returns the strand count.
extern "C" size_t host_strand_table(const uint8_t* geometry, size_t bytes, unsigned threads, uint4* table_out,
                                    float2* ys_out, uint32_t* first_out, size_t cap) {
  std::vector<uint4> table;
  std::vector<float2> ys;
  std::vector<uint32_t> first;
  gudni::build_strand_table(geometry, bytes, table, ys, first, threads);
  const size_t n = std::min(cap, table.size());
  std::memcpy(table_out, table.data(), n * sizeof(uint4));
  std::memcpy(ys_out, ys.data(), n * sizeof(float2));
  std::memcpy(first_out, first.data(), first.size() * sizeof(uint32_t));
  return table.size();
}

// One job by the warp-cooperative form (see run_all_warp).  Returns the status bits;
// *by_warp receives the number of columns the whole warp scanned, *overflow is set
// when a column needed more than full_cap.
extern "C" int host_column_raster_job_warp(const uint8_t* geometry, size_t geometry_bytes, const float* substances,
                                           size_t n_substances, const uint8_t* pictures, size_t picture_bytes,
                                           const gudni_picture_use* uses, size_t n_uses, const gudni_radial* radials,
                                           size_t n_radials, const gudni_shape* shapes, size_t n_shapes,
                                           const gudni_tile_info* tiles, int n_tiles, int compute_depth,
                                           int bitmap_w, int bitmap_h, int job_index, const float* background,
                                           const float* random_field, float stochastic, int cap, int full_cap,
                                           int max_shape, int dense_min, uint64_t seed, uint32_t* out,
                                           int* overflow, int* by_warp) {
  HostTables t;
  gudni::RasterInputs in = host_inputs(t, geometry, geometry_bytes, substances, n_substances, pictures,
                                       picture_bytes, uses, n_uses, radials, n_radials, shapes, n_shapes, tiles,
                                       n_tiles, compute_depth, bitmap_w, bitmap_h, job_index, background, max_shape,
                                       out);
  in.random_field = random_field;
  in.stochastic = stochastic;
  *overflow = 0;
  *by_warp = 0;
  const int tpt = 1 << compute_depth;
  switch (stack_words(max_shape)) {
    case 1: return run_all_warp<1>(in, tiles, n_tiles, tpt, cap, full_cap, dense_min, seed, overflow, by_warp);
    case 2: return run_all_warp<2>(in, tiles, n_tiles, tpt, cap, full_cap, dense_min, seed, overflow, by_warp);
    case 4: return run_all_warp<4>(in, tiles, n_tiles, tpt, cap, full_cap, dense_min, seed, overflow, by_warp);
    case 8: return run_all_warp<8>(in, tiles, n_tiles, tpt, cap, full_cap, dense_min, seed, overflow, by_warp);
    case 16: return run_all_warp<16>(in, tiles, n_tiles, tpt, cap, full_cap, dense_min, seed, overflow, by_warp);
    case 32: return run_all_warp<32>(in, tiles, n_tiles, tpt, cap, full_cap, dense_min, seed, overflow, by_warp);
    default: return -1;
  }
}

// Path counts of the warp-cooperative band step since the last call, by
// gudni::WarpTraceEvent (GUDNI_WARP_TRACE).
extern "C" void host_warp_trace(long long out[gudni::kTraceEvents]) {
  for (int i = 0; i < gudni::kTraceEvents; ++i) {
    out[i] = g_warp_trace[i];
    g_warp_trace[i] = 0;
  }
}

extern "C" void host_set_random_source(int mode, uint64_t seed) {
  g_random_mode = mode == 1 ? gudni::kRandomCounter : gudni::kRandomField;
  g_random_seed = seed;
}

// One job through the warp-cooperative units on the host (see run_all_coop).
extern "C" int host_column_raster_job_coop(const uint8_t* geometry, size_t geometry_bytes, const float* substances,
                                           size_t n_substances, const uint8_t* pictures, size_t picture_bytes,
                                           const gudni_picture_use* uses, size_t n_uses, const gudni_radial* radials,
                                           size_t n_radials, const gudni_shape* shapes, size_t n_shapes,
                                           const gudni_tile_info* tiles, int n_tiles, int compute_depth,
                                           int bitmap_w, int bitmap_h, int job_index, const float* background,
                                           const float* random_field, float stochastic, int capacity,
                                           int max_thresholds, int max_shape, uint64_t seed, uint32_t* out,
                                           int* overflow, int* taken) {
  HostTables t;
  gudni::RasterInputs in = host_inputs(t, geometry, geometry_bytes, substances, n_substances, pictures,
                                       picture_bytes, uses, n_uses, radials, n_radials, shapes, n_shapes, tiles,
                                       n_tiles, compute_depth, bitmap_w, bitmap_h, job_index, background, max_shape,
                                       out);
  in.random_field = random_field;
  in.stochastic = stochastic;
  in.random_mode = gudni::kRandomField;
  *overflow = 0;
  *taken = 0;
  const int tpt = 1 << compute_depth;
  switch (stack_words(max_shape)) {
    case 1: return run_all_coop<1>(in, tiles, n_tiles, tpt, capacity, max_thresholds, seed, overflow, taken);
    case 2: return run_all_coop<2>(in, tiles, n_tiles, tpt, capacity, max_thresholds, seed, overflow, taken);
    case 4: return run_all_coop<4>(in, tiles, n_tiles, tpt, capacity, max_thresholds, seed, overflow, taken);
    case 8: return run_all_coop<8>(in, tiles, n_tiles, tpt, capacity, max_thresholds, seed, overflow, taken);
    case 16: return run_all_coop<16>(in, tiles, n_tiles, tpt, capacity, max_thresholds, seed, overflow, taken);
    case 32: return run_all_coop<32>(in, tiles, n_tiles, tpt, capacity, max_thresholds, seed, overflow, taken);
    default: return -1;
  }
}
