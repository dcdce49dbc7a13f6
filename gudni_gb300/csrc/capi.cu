// C ABI of the raster path (include/gudni_cuda.h).
//
// A context owns its device, stream, the uploaded common buffers, per-job staging
// buffers and the threshold scratch.  Scratch is sized for the resident grid
// (SMs x resident blocks x 128 threads), not for the job: each resident thread reuses
// one slot for every column it runs.  This replaces the reference's per-job
// allocation of columns x MAXTHRESHOLDS thresholds (OpenCL/CallKernels.hs:124-127).
//
// Every launch is a pair on one stream: the fast pass over the tiles and the
// full-capacity pass over the columns that overflowed it (raster.cu).  Nothing
// between them, or after them, waits on the host until the caller asks for the
// output or the status.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "adjoint_kernels.h"
#include "gudni_cuda.h"
#include "gudni_serialize.h"
#include "raster_kernels.h"
#include "serialize_device.cuh"
#include "strand_table.h"

using gudni::TileLaunch;

// Work units per resident cooperative warp below which a launch takes the cooperative
// units when the choice is automatic (gudni_set_cooperative_units(ctx, -1)).
#define GUDNI_COOP_UNITS_PER_WARP 2

namespace {

std::mutex g_create_mutex;
std::string g_create_error;

template <class T>
struct DevBuf {
  T* ptr = nullptr;
  size_t cap = 0;  // elements
  cudaError_t reserve(size_t n) {
    if (n <= cap && ptr) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(n, 1);
    if (want > SIZE_MAX / sizeof(T)) return cudaErrorMemoryAllocation;  // the byte count would wrap
    cudaError_t e = cudaMalloc(&ptr, want * sizeof(T));
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
};

}  // namespace

namespace gudni {
// Error text reported by gudni_last_error(NULL) for calls made without a context.
void set_global_error(const std::string& msg) {
  std::lock_guard<std::mutex> lock(g_create_mutex);
  g_create_error = msg;
}
}  // namespace gudni

struct gudni_ctx {
  gudni_spec spec;
  int device = 0;
  int sm_count = 0;
  int sections = 1;
  int blocks_per_sm = 1;
  int coop_blocks_per_sm = 1;  // resident blocks of the cooperative-unit kernel
  int grid = 1;
  int working_capacity = 256;
  cudaStream_t stream = nullptr;
  std::string error;

  // common buffers (BuffersInCommon)
  bool common_ready = false;
  DevBuf<uint8_t> geometry;
  size_t geometry_bytes = 0;
  DevBuf<float4> substances;
  size_t n_substances = 0;
  DevBuf<uint8_t> pictures;
  size_t picture_bytes = 0;
  DevBuf<gudni_picture_use> uses;
  size_t n_uses = 0;
  uint64_t uses_extent = 0;           // furthest picture-pile byte the uploaded usages read
  DevBuf<gudni_radial> radials;
  size_t n_radials = 0;
  DevBuf<float> random_field;
  bool has_random = false;
  DevBuf<uint4> strand_table;
  DevBuf<float2> strand_y;            // per strand: lowest and highest point y
  DevBuf<uint32_t> strand_first;
  size_t n_strands = 0;
  size_t n_units = 0;
  std::vector<uint4> h_strand_table;
  std::vector<float2> h_strand_y;
  std::vector<uint32_t> h_strand_first;

  // per-job / per-frame staging
  DevBuf<gudni_shape> shapes;
  DevBuf<gudni_tile_info> tiles;
  DevBuf<int32_t> tile_jobs;
  DevBuf<uint32_t> out;
  std::vector<gudni_shape> h_shapes;
  std::vector<gudni_tile_info> h_tiles;
  std::vector<int32_t> h_tile_jobs;

  // batch
  bool batch_ready = false;
  size_t batch_tiles = 0;
  size_t batch_shapes = 0;
  size_t batch_scenes = 0;
  size_t batch_pixels = 0;
  size_t batch_units = 0;
  int batch_chunk_log2 = 0;           // largest over the batch's scenes
  DevBuf<gudni_shape> b_shapes;
  DevBuf<gudni_tile_info> b_tiles;
  DevBuf<int32_t> b_tile_scene;
  DevBuf<uint32_t> b_order;           // work units, cost-descending
  DevBuf<uint32_t> f_units;           // a frame's cost-ordered work units (device-built)
  DevBuf<uint32_t> f_order_words;     // their bucket counts and cursors
  DevBuf<gudni::SceneInfo> b_scenes;
  DevBuf<uint32_t> b_out;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;

  // scratch: fast pass (grid slots x working capacity), full-capacity pool
  DevBuf<float4> thr;
  DevBuf<uint32_t> hdr;
  DevBuf<uint32_t> idx;
  DevBuf<float4> big_thr;
  DevBuf<uint32_t> big_hdr;
  DevBuf<uint32_t> big_idx;
  size_t fallback_slots = 0;
  DevBuf<uint32_t> overflow_items;
  DevBuf<uint32_t> words;   // [0] overflow count, [1] next tile
  DevBuf<int> status;
  DevBuf<int64_t> counters;
  bool counters_on = false;
  int dense_min = 0;  // gudni_set_dense_columns (0: per-lane scan only)
  int coop = 0;       // gudni_set_cooperative_units: 1 on, 0 off (default), -1 chosen per launch
  uint32_t random_mode = gudni::kRandomField;  // gudni_set_random_source
  uint64_t random_seed = 0;
  bool device_strands = false;  // gudni_set_device_strand_table

  // adjoint scratch: slots x capacity thresholds, provenance and line records
  int adj_grid = 0;
  int adj_capacity = 0;
  DevBuf<float4> a_thr;
  DevBuf<uint32_t> a_hdr;
  DevBuf<float4> a_thr_fwd;  // the forward scan's copy of each column's sorted queue
  DevBuf<uint32_t> a_hdr_fwd;
  int adj_regenerate = 0;  // gudni_set_adjoint_regenerate
  DevBuf<int4> a_prov;
  DevBuf<uint8_t> a_lines;
  DevBuf<float4> a_line_grad;
  DevBuf<uint32_t> a_idx;
  DevBuf<float4> a_bit_grad;
  DevBuf<float4> a_layers;
  DevBuf<int32_t> a_layer_bits;
  // serializer on the device: the scene's arrays, pass temporaries, the frame's piles
  DevBuf<int32_t> ser_sub_start, ser_compound, ser_outline_start, ser_pair_start;
  DevBuf<float> ser_pairs;
  DevBuf<uint64_t> ser_sub_tag;
  DevBuf<uint8_t> ser_tmp[gudni::ser::kSlots];
  DevBuf<gudni_shape> ds_shapes;
  DevBuf<gudni_tile_info> ds_tiles;
  DevBuf<int32_t> ds_tile_jobs;
  DevBuf<uint32_t> ds_point_offsets;
  DevBuf<int32_t> ds_point_sources;
  DevBuf<float> ds_point_weights;
  uint64_t launches = 0;
  cudaStream_t last_stream = nullptr;
};

namespace {

int fail(gudni_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->error = msg;
  return code;
}

int cuda_fail(gudni_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? GUDNI_ERR_OUT_OF_MEMORY : GUDNI_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

int status_to_code(int bits) {
  if (bits & gudni::kStatusBadInput) return GUDNI_ERR_BAD_INPUT;
  if (bits & gudni::kStatusOverflow) return GUDNI_ERR_THRESHOLD_OVERFLOW;
  if (bits & gudni::kStatusIterLimit) return GUDNI_ERR_ITER_LIMIT;
  return GUDNI_OK;
}

const char* status_message(int bits) {
  if (bits & gudni::kStatusBadInput) return "a shape, strand, substance, picture or tile record points outside its buffer";
  if (bits & gudni::kStatusOverflow) return "a column needed more thresholds than max_thresholds";
  if (bits & gudni::kStatusIterLimit) return "a device loop hit its iteration cap";
  return "";
}

bool valid_spec(const gudni_spec* s, std::string& why) {
  auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
  if (!s) { why = "null spec"; return false; }
  if (!pow2(s->threads_per_tile) || s->threads_per_tile > (1 << gudni::kMaxLog2Tpt)) {
    why = "threads_per_tile must be a power of two <= 1024";
    return false;
  }
  if (s->max_thresholds < 4) { why = "max_thresholds must be >= 4"; return false; }
  if (s->max_shape < 1 || s->max_shape > 64 * 32 - 1) { why = "max_shape must be in [1, 2047]"; return false; }
  if (s->stack_sections < 1 || s->max_shape > 64 * s->stack_sections - 1) {
    why = "max_shape must be <= 64*stack_sections-1";
    return false;
  }
  if (!(s->stochastic_factor == s->stochastic_factor)) { why = "stochastic_factor is NaN"; return false; }
  return true;
}

int ensure_scratch(gudni_ctx* ctx) {
  const size_t slots = (size_t)ctx->grid * gudni::kRasterBlock;
  const size_t cap = (size_t)ctx->working_capacity;
  cudaError_t e;
  if ((e = ctx->thr.reserve(slots * cap)) != cudaSuccess) return cuda_fail(ctx, e, "scratch thresholds");
  if ((e = ctx->hdr.reserve(slots * cap)) != cudaSuccess) return cuda_fail(ctx, e, "scratch headers");
  if ((e = ctx->idx.reserve(slots * (size_t)ctx->spec.max_shape)) != cudaSuccess) return cuda_fail(ctx, e, "scratch shape indices");
  if (!ctx->status.ptr) {  // device memory starts undefined: clear the words once
    if ((e = ctx->status.reserve(1)) != cudaSuccess) return cuda_fail(ctx, e, "status word");
    if ((e = cudaMemset(ctx->status.ptr, 0, sizeof(int))) != cudaSuccess) return cuda_fail(ctx, e, "status word");
  }
  if (!ctx->words.ptr) {
    if ((e = ctx->words.reserve(2)) != cudaSuccess) return cuda_fail(ctx, e, "work counters");
    if ((e = cudaMemset(ctx->words.ptr, 0, 2 * sizeof(uint32_t))) != cudaSuccess) return cuda_fail(ctx, e, "work counters");
  }
  if (!ctx->counters.ptr) {
    if ((e = ctx->counters.reserve(4)) != cudaSuccess) return cuda_fail(ctx, e, "counters");
    if ((e = cudaMemset(ctx->counters.ptr, 0, 4 * sizeof(int64_t))) != cudaSuccess) return cuda_fail(ctx, e, "counters");
  }
  return GUDNI_OK;
}

// Scratch for the full-capacity pass: a fixed pool of slots (at most ~2 GB).
int ensure_fallback_pool(gudni_ctx* ctx) {
  if (ctx->fallback_slots) return GUDNI_OK;
  const size_t per_slot = (size_t)ctx->spec.max_thresholds * 20 + (size_t)ctx->spec.max_shape * 4;
  size_t slots = ((size_t)2 << 30) / per_slot;
  slots = std::min<size_t>(slots, (size_t)ctx->grid * gudni::kRasterBlock);
  slots = std::max<size_t>(gudni::kRasterBlock, (slots / gudni::kRasterBlock) * gudni::kRasterBlock);
  cudaError_t e;
  if ((e = ctx->big_thr.reserve(slots * ctx->spec.max_thresholds)) != cudaSuccess) return cuda_fail(ctx, e, "fallback scratch");
  if ((e = ctx->big_hdr.reserve(slots * ctx->spec.max_thresholds)) != cudaSuccess) return cuda_fail(ctx, e, "fallback scratch");
  if ((e = ctx->big_idx.reserve(slots * ctx->spec.max_shape)) != cudaSuccess) return cuda_fail(ctx, e, "fallback scratch");
  ctx->fallback_slots = slots;
  return GUDNI_OK;
}

int validate_tiles_host(gudni_ctx* ctx, const gudni_tile_info* tiles, size_t n_tiles, size_t n_shapes) {
  for (size_t i = 0; i < n_tiles; ++i) {
    const gudni_tile_info& t = tiles[i];
    if ((uint64_t)t.shapes.start + t.shapes.length > n_shapes || t.hdepth < 0 || t.hdepth > 24 || t.vdepth < 0 ||
        t.vdepth > 24 || t.left < 0 || t.top < 0)
      return fail(ctx, GUDNI_ERR_BAD_INPUT, "tile " + std::to_string(i) + " is malformed");
  }
  return GUDNI_OK;
}

int validate_job(gudni_ctx* ctx, const gudni_shape* shapes, size_t n_shapes, const gudni_tile_info* tiles,
                 size_t n_tiles, int32_t bitmap_w, int32_t bitmap_h, int32_t compute_depth, bool host) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if (!ctx->common_ready) return fail(ctx, GUDNI_ERR_NOT_READY, "gudni_upload_common has not been called");
  if (bitmap_w <= 0 || bitmap_h <= 0) return fail(ctx, GUDNI_ERR_BAD_INPUT, "bitmap size must be positive");
  if ((int64_t)bitmap_w * bitmap_h > (int64_t)1 << 31) return fail(ctx, GUDNI_ERR_BAD_INPUT, "bitmap too large");
  if (compute_depth < 0 || compute_depth > gudni::kMaxLog2Tpt || (1 << compute_depth) != ctx->spec.threads_per_tile)
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "compute_depth must be log2(threads_per_tile)");
  if (n_tiles > 0 && !tiles) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null tiles");
  if (n_shapes > 0 && !shapes) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null shapes");
  if (((uint64_t)n_tiles << gudni::chunkLog2(compute_depth)) >= gudni::kMaxUnits)
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "too many tiles in one launch");
  if (n_shapes > 0xFFFFFFFFull) return fail(ctx, GUDNI_ERR_BAD_INPUT, "too many shapes");
  if (host) return validate_tiles_host(ctx, tiles, n_tiles, n_shapes);
  return GUDNI_OK;
}

gudni::RasterInputs inputs(gudni_ctx* ctx, const gudni_shape* d_shapes, size_t n_shapes,
                           const gudni_tile_info* d_tiles, size_t n_tiles, int32_t bitmap_w, int32_t bitmap_h,
                           int32_t compute_depth, int32_t job_index, const float background[4], uint32_t* d_out) {
  gudni::RasterInputs in;
  in.geometry = ctx->geometry.ptr;
  in.geometry_bytes = ctx->geometry_bytes;
  in.substances = ctx->substances.ptr;
  in.n_substances = (uint32_t)ctx->n_substances;
  in.pictures = ctx->pictures.ptr;
  in.picture_bytes = ctx->picture_bytes;
  in.uses = ctx->uses.ptr;
  in.n_uses = (uint32_t)ctx->n_uses;
  in.radials = ctx->radials.ptr;
  in.n_radials = (uint32_t)ctx->n_radials;
  in.random_field = ctx->has_random ? ctx->random_field.ptr : nullptr;
  in.stochastic = ctx->spec.stochastic_factor;
  in.shapes = d_shapes;
  in.n_shapes = (uint32_t)n_shapes;
  in.tiles = d_tiles;
  in.n_tiles = (int)n_tiles;
  in.log2_tpt = compute_depth;
  in.bitmap_w = bitmap_w;
  in.bitmap_h = bitmap_h;
  in.job_index = job_index;
  in.background = background ? make_float4(background[0], background[1], background[2], background[3])
                             : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  in.max_shape = ctx->spec.max_shape;
  in.out = d_out;
  in.tile_jobs = nullptr;
  in.counters = ctx->counters_on ? ctx->counters.ptr : nullptr;
  in.strand_table = ctx->n_strands ? ctx->strand_table.ptr : nullptr;
  in.strand_y = ctx->n_strands ? ctx->strand_y.ptr : nullptr;
  in.n_strands = (uint32_t)ctx->n_strands;
  in.strand_first = ctx->strand_first.ptr;
  in.n_units = (uint32_t)ctx->n_units;
  in.random_mode = ctx->random_mode;
  in.random_seed = ctx->random_seed;
  return in;
}

// Enqueue the fast pass over `n_tiles` tiles and the full-capacity pass over the
// columns that overflowed it.  `max_tpt` is the largest threads-per-tile in the
// launch (sizes the overflow list).  Work units: the `units` list (n_units entries),
// or without one every tile's 32-column chunks in tile order (chunk_log2 per tile).
int enqueue(gudni_ctx* ctx, const gudni::RasterInputs& in, const gudni::SceneInfo* scenes,
            const int32_t* tile_scene, size_t n_scenes, const uint32_t* units, size_t n_units, int chunk_log2,
            size_t n_tiles, int max_tpt, cudaStream_t stream) {
  int rc = ensure_scratch(ctx);
  if (rc) return rc;
  if (n_tiles == 0) return GUDNI_OK;
  cudaError_t e;
  if (!units && n_tiles >= 64) {
    // no unit list given: schedule the tiles most expensive first, ordered on the device
    n_units = n_tiles << chunk_log2;
    if ((e = ctx->f_units.reserve(n_units)) != cudaSuccess || (e = ctx->f_order_words.reserve(128)) != cudaSuccess)
      return cuda_fail(ctx, e, "tile order scratch");
    if ((e = gudni::launch_tile_order(in.tiles, (uint32_t)n_tiles, in.shapes, in.n_shapes, chunk_log2,
                                      ctx->f_order_words.ptr, ctx->f_units.ptr, stream)) != cudaSuccess)
      return cuda_fail(ctx, e, "tile order");
    ctx->launches += 3;
    units = ctx->f_units.ptr;
  }
  if (!units) n_units = n_tiles << chunk_log2;
  const size_t max_items = n_tiles * (size_t)max_tpt;
  const bool need_fallback = ctx->working_capacity < ctx->spec.max_thresholds;
  if (need_fallback) {
    if ((e = ctx->overflow_items.reserve(max_items)) != cudaSuccess) return cuda_fail(ctx, e, "overflow list");
    if ((rc = ensure_fallback_pool(ctx))) return rc;
  }
  if ((e = cudaMemsetAsync(ctx->words.ptr, 0, 2 * sizeof(uint32_t), stream)) != cudaSuccess)
    return cuda_fail(ctx, e, "memset");
  TileLaunch a;
  std::memset(&a, 0, sizeof(a));
  a.in = in;
  a.scenes = scenes;
  a.tile_scene = tile_scene;
  a.n_scenes = (uint32_t)n_scenes;
  a.scratch = gudni::ColumnScratch{ctx->thr.ptr, ctx->hdr.ptr, ctx->idx.ptr, ctx->working_capacity,
                                   ctx->spec.max_shape};
  a.units = units;
  a.n_units = (uint32_t)n_units;
  a.chunk_log2 = chunk_log2;
  a.next_tile = ctx->words.ptr + 1;
  a.overflow_items = need_fallback ? ctx->overflow_items.ptr : nullptr;
  a.overflow_cap = (uint32_t)std::min<size_t>(max_items, 0xFFFFFFFFull);
  a.overflow_count = ctx->words.ptr;
  a.dense_min = ctx->dense_min;
  // Cooperative units shorten each unit (its generation is shared by the warp) but
  // hold more registers per thread, so fewer warps are resident.  A launch with few
  // units per resident warp is bound by its longest units and takes them; one with
  // many is bound by throughput and runs the per-column kernel, which keeps more warps
  // in flight (GUDNI_COOP_UNITS_PER_WARP units per resident cooperative warp is the
  // crossover measured on GB300).
  const size_t coop_warps = (size_t)ctx->sm_count * (size_t)ctx->coop_blocks_per_sm * (gudni::kRasterBlock / 32);
  a.coop = ctx->coop > 0 || (ctx->coop < 0 && n_units <= coop_warps * GUDNI_COOP_UNITS_PER_WARP) ? 1 : 0;
  a.status = ctx->status.ptr;
  const size_t warps_per_block = gudni::kRasterBlock / 32;
  const int grid = (int)std::min<size_t>((n_units + warps_per_block - 1) / warps_per_block, (size_t)ctx->grid);
  if ((e = gudni::launch_raster(a, false, ctx->sections, grid, stream)) != cudaSuccess)
    return cuda_fail(ctx, e, "raster launch");
  ctx->launches += 1;
  if (!need_fallback) return GUDNI_OK;
  TileLaunch f = a;
  f.scratch = gudni::ColumnScratch{ctx->big_thr.ptr, ctx->big_hdr.ptr, ctx->big_idx.ptr, ctx->spec.max_thresholds,
                                   ctx->spec.max_shape};
  f.overflow_items = nullptr;
  f.list = ctx->overflow_items.ptr;
  f.list_count = ctx->words.ptr;
  f.list_cap = a.overflow_cap;
  const int fgrid = (int)std::max<size_t>(1, std::min<size_t>(ctx->fallback_slots / gudni::kRasterBlock,
                                                              (max_items + gudni::kRasterBlock - 1) / gudni::kRasterBlock));
  if ((e = gudni::launch_raster(f, true, ctx->sections, fgrid, stream)) != cudaSuccess)
    return cuda_fail(ctx, e, "fallback launch");
  ctx->launches += 1;
  return GUDNI_OK;
}

int read_status(gudni_ctx* ctx, cudaStream_t stream) {
  int bits = 0;
  if (ctx->status.ptr) {
    cudaError_t e = cudaMemcpyAsync(&bits, ctx->status.ptr, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->status.ptr, 0, sizeof(int), stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "status read");
  }
  if (bits) return fail(ctx, status_to_code(bits), status_message(bits));
  return GUDNI_OK;
}

template <class T>
int upload(gudni_ctx* ctx, DevBuf<T>& buf, const void* src, size_t count, const char* what) {
  cudaError_t e = buf.reserve(count);
  if (e == cudaSuccess && count) e = cudaMemcpyAsync(buf.ptr, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, what);
  return GUDNI_OK;
}

int build_strand_table(gudni_ctx* ctx, const uint8_t* geo, size_t bytes);
int build_strand_table_device(gudni_ctx* ctx, size_t bytes);

// The strand table of the pile just uploaded: on the host from the caller's copy, or
// (gudni_set_device_strand_table) on the device from the uploaded one.
int strand_table_of(gudni_ctx* ctx, const void* geometry, size_t bytes) {
  if (ctx->device_strands) return build_strand_table_device(ctx, bytes);
  return build_strand_table(ctx, static_cast<const uint8_t*>(geometry), bytes);
}

// Every picture usage must read inside a picture pile of `picture_bytes` bytes, from a
// 4-byte aligned offset; *extent receives the furthest byte any of them reads.
int check_picture_uses(gudni_ctx* ctx, const gudni_picture_use* uses, size_t n, size_t picture_bytes,
                       uint64_t* extent) {
  uint64_t far = 0;
  for (size_t i = 0; i < n; ++i) {
    const gudni_picture_use& u = uses[i];
    const uint64_t end = (uint64_t)u.mem_offset + 4ull * (uint64_t)u.size_x * (uint64_t)u.size_y;
    if (u.size_x < 0 || u.size_y < 0 || u.mem_offset < 0 || (u.mem_offset & 3) != 0 || end > picture_bytes)
      return fail(ctx, GUDNI_ERR_BAD_INPUT, "picture use " + std::to_string(i) + " points outside the picture pile");
    far = std::max(far, end);
  }
  *extent = far;
  return GUDNI_OK;
}

int upload_common_buffers(gudni_ctx* ctx, const void* geometry, size_t geometry_bytes, const float* substances,
                          size_t n_substances, const uint8_t* pictures, size_t picture_bytes,
                          const gudni_picture_use* picture_uses, size_t n_picture_uses,
                          const gudni_radial* radials, size_t n_radials, const float* random_field) {
  if ((geometry_bytes && !geometry) || (n_substances && !substances) || (picture_bytes && !pictures) ||
      (n_picture_uses && !picture_uses) || (n_radials && !radials))
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "null buffer with non-zero size");
  if (geometry_bytes % 16 != 0) return fail(ctx, GUDNI_ERR_BAD_INPUT, "geometry pile must be a multiple of 16 bytes");
  uint64_t extent = 0;
  int rc = check_picture_uses(ctx, picture_uses, n_picture_uses, picture_bytes, &extent);
  if (rc) return rc;
  ctx->common_ready = false;
  if ((rc = upload(ctx, ctx->geometry, geometry, geometry_bytes, "geometry upload"))) return rc;
  if ((rc = upload(ctx, ctx->substances, substances, n_substances, "substance upload"))) return rc;
  if ((rc = upload(ctx, ctx->pictures, pictures, picture_bytes, "picture upload"))) return rc;
  if ((rc = upload(ctx, ctx->uses, picture_uses, n_picture_uses, "picture use upload"))) return rc;
  if ((rc = upload(ctx, ctx->radials, radials, n_radials, "radial upload"))) return rc;
  ctx->has_random = random_field != nullptr;
  if (random_field && (rc = upload(ctx, ctx->random_field, random_field, GUDNI_RANDOM_FIELD_SIZE, "random field upload")))
    return rc;
  if ((rc = strand_table_of(ctx, geometry, geometry_bytes))) return rc;
  ctx->geometry_bytes = geometry_bytes;
  ctx->n_substances = n_substances;
  ctx->picture_bytes = picture_bytes;
  ctx->n_uses = n_picture_uses;
  ctx->uses_extent = extent;
  ctx->n_radials = n_radials;
  return GUDNI_OK;
}

// The strand table of the uploaded pile (strand_table.h), uploaded beside it.
int build_strand_table(gudni_ctx* ctx, const uint8_t* geo, size_t bytes) {
  static_assert(gudni::kNoStrandIndex == gudni::kNoStrand, "one marker for units without a strand");
  ctx->n_strands = 0;
  ctx->n_units = bytes / 16;
  const unsigned cores = std::thread::hardware_concurrency();
  gudni::build_strand_table(geo, bytes, ctx->h_strand_table, ctx->h_strand_y, ctx->h_strand_first,
                            std::min(16u, cores ? cores : 1u));
  int rc;
  if ((rc = upload(ctx, ctx->strand_table, ctx->h_strand_table.data(), ctx->h_strand_table.size(), "strand table")))
    return rc;
  if ((rc = upload(ctx, ctx->strand_y, ctx->h_strand_y.data(), ctx->h_strand_y.size(), "strand y ranges")))
    return rc;
  if ((rc = upload(ctx, ctx->strand_first, ctx->h_strand_first.data(), ctx->h_strand_first.size(), "strand map")))
    return rc;
  ctx->n_strands = ctx->h_strand_table.size();
  return GUDNI_OK;
}

void drop_graph(gudni_ctx* ctx) {
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  if (ctx->graph) cudaGraphDestroy(ctx->graph);
  ctx->graph_exec = nullptr;
  ctx->graph = nullptr;
}

// Adjoint scratch, sized once: one slot per resident thread (capped so the whole
// stays within ~16 GB), each holding `capacity` thresholds with their provenance and
// line records, per-shape-bit index and colour-gradient words, and the composited
// layers of one section (at most max_shape + 1).
int ensure_adjoint_scratch(gudni_ctx* ctx) {
  if (ctx->adj_grid) return GUDNI_OK;
  int rc = ensure_scratch(ctx);  // status word
  if (rc) return rc;
  int cap = std::min(ctx->spec.max_thresholds, 1024);
  if (const char* env = std::getenv("GUDNI_ADJOINT_CAPACITY")) {
    const int v = std::atoi(env);
    if (v >= 4) cap = std::min(ctx->spec.max_thresholds, v);
  }
  int bps = 1;
  if (gudni::adjoint_occupancy(ctx->sections, &bps) != cudaSuccess || bps < 1) bps = 1;
  const size_t per_slot = (size_t)cap * (2 * (sizeof(float4) + 4) + sizeof(int4) + gudni::adjoint_line_bytes() +
                                         sizeof(float4)) +
                          (size_t)ctx->spec.max_shape * (4 + sizeof(float4)) +
                          (size_t)(ctx->spec.max_shape + 1) * (2 * sizeof(float4) + 4);
  size_t slots = (size_t)ctx->sm_count * (size_t)bps * gudni::kAdjointBlock;
  slots = std::min(slots, ((size_t)16 << 30) / per_slot);
  slots = std::max<size_t>(gudni::kAdjointBlock, (slots / gudni::kAdjointBlock) * gudni::kAdjointBlock);
  cudaError_t e;
  if ((e = ctx->a_thr.reserve(slots * cap)) != cudaSuccess ||
      (e = ctx->a_hdr.reserve(slots * cap)) != cudaSuccess ||
      (e = ctx->a_thr_fwd.reserve(slots * cap)) != cudaSuccess ||
      (e = ctx->a_hdr_fwd.reserve(slots * cap)) != cudaSuccess ||
      (e = ctx->a_prov.reserve(slots * cap)) != cudaSuccess ||
      (e = ctx->a_lines.reserve(slots * cap * gudni::adjoint_line_bytes())) != cudaSuccess ||
      (e = ctx->a_line_grad.reserve(slots * cap)) != cudaSuccess ||
      (e = ctx->a_idx.reserve(slots * (size_t)ctx->spec.max_shape)) != cudaSuccess ||
      (e = ctx->a_bit_grad.reserve(slots * (size_t)ctx->spec.max_shape)) != cudaSuccess ||
      (e = ctx->a_layers.reserve(slots * 2 * (size_t)(ctx->spec.max_shape + 1))) != cudaSuccess ||
      (e = ctx->a_layer_bits.reserve(slots * (size_t)(ctx->spec.max_shape + 1))) != cudaSuccess)
    return cuda_fail(ctx, e, "adjoint scratch");
  ctx->adj_capacity = cap;
  ctx->adj_grid = (int)(slots / gudni::kAdjointBlock);
  return GUDNI_OK;
}

int enqueue_adjoint(gudni_ctx* ctx, const gudni::RasterInputs& in, const gudni::SceneInfo* scenes,
                    const int32_t* tile_scene, size_t n_scenes, const uint32_t* units, size_t n_units,
                    int chunk_log2, size_t n_tiles, const float* target, float* image, float* grad_geometry,
                    float* grad_substances, cudaStream_t stream) {
  int rc = ensure_adjoint_scratch(ctx);
  if (rc) return rc;
  if (n_tiles == 0) return GUDNI_OK;
  cudaError_t e;
  if (!units && n_tiles >= 64) {  // most expensive tiles first, as for the raster pass
    n_units = n_tiles << chunk_log2;
    if ((e = ctx->f_units.reserve(n_units)) != cudaSuccess || (e = ctx->f_order_words.reserve(128)) != cudaSuccess)
      return cuda_fail(ctx, e, "tile order scratch");
    if ((e = gudni::launch_tile_order(in.tiles, (uint32_t)n_tiles, in.shapes, in.n_shapes, chunk_log2,
                                      ctx->f_order_words.ptr, ctx->f_units.ptr, stream)) != cudaSuccess)
      return cuda_fail(ctx, e, "tile order");
    ctx->launches += 3;
    units = ctx->f_units.ptr;
  }
  if (!units) n_units = n_tiles << chunk_log2;
  e = cudaMemsetAsync(ctx->words.ptr, 0, 2 * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "memset");
  gudni::AdjointLaunch a;
  std::memset(&a, 0, sizeof(a));
  a.in = in;
  a.in.counters = nullptr;
  a.in.stochastic = 0.0f;  // the loss is defined on the deterministic render
  a.in.random_field = nullptr;
  a.scenes = scenes;
  a.tile_scene = tile_scene;
  a.n_scenes = (uint32_t)n_scenes;
  a.units = units;
  a.n_units = (uint32_t)n_units;
  a.chunk_log2 = chunk_log2;
  a.next_tile = ctx->words.ptr + 1;
  a.capacity = ctx->adj_capacity;
  a.thr = ctx->a_thr.ptr;
  a.thr_fwd = ctx->a_thr_fwd.ptr;
  a.hdr_fwd = ctx->a_hdr_fwd.ptr;
  a.regenerate = ctx->adj_regenerate;
  a.hdr = ctx->a_hdr.ptr;
  a.prov = ctx->a_prov.ptr;
  a.lines = ctx->a_lines.ptr;
  a.line_grad = ctx->a_line_grad.ptr;
  a.idx = ctx->a_idx.ptr;
  a.bit_grad = ctx->a_bit_grad.ptr;
  a.layers = ctx->a_layers.ptr;
  a.layer_bits = ctx->a_layer_bits.ptr;
  a.image = reinterpret_cast<float4*>(image);
  a.target = reinterpret_cast<const float4*>(target);
  a.grad_geometry = grad_geometry;
  a.grad_substances = grad_substances;
  a.status = ctx->status.ptr;
  const size_t warps_per_block = gudni::kAdjointBlock / 32;
  const int grid = (int)std::min<size_t>((n_units + warps_per_block - 1) / warps_per_block, (size_t)ctx->adj_grid);
  if ((e = gudni::launch_adjoint(a, ctx->sections, grid, stream)) != cudaSuccess)
    return cuda_fail(ctx, e, "adjoint launch");
  ctx->launches += 1;
  return GUDNI_OK;
}

bool adjoint_pointers_ok(const float* target, const float* image, const float* grad_geometry,
                         const float* grad_substances) {
  return target && image && grad_geometry && grad_substances && ((uintptr_t)target & 15) == 0 &&
         ((uintptr_t)image & 15) == 0 && ((uintptr_t)grad_geometry & 3) == 0 && ((uintptr_t)grad_substances & 3) == 0;
}

// ---------------------------------------------------------------- device serializer
// The executor that runs the serializer's passes (serialize_device.cuh) as kernels on
// the context's stream; results land in the context's frame buffers.

struct SerExec {
  gudni_ctx* ctx;
  cudaStream_t stream;
  cudaError_t err = cudaSuccess;

  int check(cudaError_t e) {
    if (e == cudaSuccess) return 0;
    err = e;
    return -1;
  }
  template <class U>
  void* grow(DevBuf<U>& b, uint64_t bytes) {
    if (check(b.reserve((size_t)((bytes + sizeof(U) - 1) / sizeof(U))))) return nullptr;
    return b.ptr;
  }
  template <class T>
  T* alloc(gudni::ser::Slot slot, uint64_t n) {
    if (n > UINT64_MAX / sizeof(T)) return nullptr;  // the byte count would wrap: a storage error
    const uint64_t bytes = n * sizeof(T);
    void* p;
    switch (slot) {
      case gudni::ser::kGeometry: p = grow(ctx->geometry, bytes); break;
      case gudni::ser::kStrandTable: p = grow(ctx->strand_table, bytes); break;
      case gudni::ser::kStrandY: p = grow(ctx->strand_y, bytes); break;
      case gudni::ser::kStrandFirst: p = grow(ctx->strand_first, bytes); break;
      case gudni::ser::kShapes: p = grow(ctx->ds_shapes, bytes); break;
      case gudni::ser::kTiles: p = grow(ctx->ds_tiles, bytes); break;
      case gudni::ser::kTileJobs: p = grow(ctx->ds_tile_jobs, bytes); break;
      case gudni::ser::kPointOffsets: p = grow(ctx->ds_point_offsets, bytes); break;
      case gudni::ser::kPointSources: p = grow(ctx->ds_point_sources, bytes); break;
      case gudni::ser::kPointWeights: p = grow(ctx->ds_point_weights, bytes); break;
      default: p = grow(ctx->ser_tmp[slot], bytes); break;
    }
    return static_cast<T*>(p);
  }
  template <class Pass>
  int forEach(uint64_t n, const Pass& pass) {
    if (n == 0) return 0;
    const int grid = (int)std::min<uint64_t>((n + gudni::ser::kPassBlock - 1) / gudni::ser::kPassBlock,
                                              (uint64_t)ctx->sm_count * 8);
    gudni::ser::pass_kernel<Pass><<<grid, gudni::ser::kPassBlock, 0, stream>>>(pass, n);
    ctx->launches += 1;
    return check(cudaGetLastError());
  }
  int scan(const uint64_t* in, uint64_t* out, uint64_t n) {
    gudni::ser::scan_kernel<<<1, gudni::ser::kScanBlock, 0, stream>>>(in, out, n);
    ctx->launches += 1;
    return check(cudaGetLastError());
  }
  int read(void* dst, const void* src, size_t bytes) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return check(e);
  }
  int copy(void* dst, const void* src, size_t bytes) {
    return check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, stream));
  }
  int upload(void* dst, const void* src, size_t bytes) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);  // src may be a temporary
    return check(e);
  }
};

// The strand table of the uploaded pile by the device passes (serialize_device.cuh
// strandTable) on the context's stream; one read of the strand count.
int build_strand_table_device(gudni_ctx* ctx, size_t bytes) {
  SerExec ex{ctx, ctx->stream};
  gudni::ser::StrandTableOut t;
  const int rc = gudni::ser::strandTable(ex, bytes ? ctx->geometry.ptr : nullptr, bytes, t);
  if (rc == -2) return fail(ctx, GUDNI_ERR_BAD_INPUT, "too many strands");
  if (rc) return cuda_fail(ctx, ex.err, "strand table");
  ctx->n_strands = t.n_strands;
  ctx->n_units = bytes / 16;
  return GUDNI_OK;
}

}  // namespace

extern "C" {

gudni_ctx* gudni_create(const gudni_spec* spec, int device) {
  std::lock_guard<std::mutex> lock(g_create_mutex);
  std::string why;
  if (!valid_spec(spec, why)) {
    g_create_error = "invalid spec: " + why;
    return nullptr;
  }
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    g_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
    return nullptr;
  }
  if (device < 0 || device >= n) {
    g_create_error = "device index out of range";
    return nullptr;
  }
  gudni_ctx* ctx = new gudni_ctx();
  ctx->spec = *spec;
  ctx->device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    g_create_error = std::string("CUDA setup failed: ") + cudaGetErrorString(e);
    delete ctx;
    return nullptr;
  }
  ctx->sections = gudni::sections_for(spec->max_shape);
  if ((e = gudni::raster_occupancy(ctx->sections, &ctx->blocks_per_sm)) != cudaSuccess || ctx->blocks_per_sm < 1)
    ctx->blocks_per_sm = 1;
  if ((e = gudni::raster_coop_occupancy(ctx->sections, &ctx->coop_blocks_per_sm)) != cudaSuccess ||
      ctx->coop_blocks_per_sm < 1)
    ctx->coop_blocks_per_sm = 1;
  ctx->grid = ctx->sm_count * ctx->blocks_per_sm;
  // fast-pass capacity: as much of max_thresholds as ~8 GB of slots allow (at most
  // 4096); only columns that need more go through the full-capacity pass
  {
    const size_t slots = (size_t)ctx->grid * gudni::kRasterBlock;
    const size_t budget = ((size_t)8 << 30) / (slots * (sizeof(float4) + 4));
    ctx->working_capacity = (int)std::max<size_t>(64, std::min<size_t>({(size_t)spec->max_thresholds, budget, 4096}));
  }
  if (const char* env = std::getenv("GUDNI_WORKING_CAPACITY")) {
    int v = std::atoi(env);
    if (v >= 4) ctx->working_capacity = std::min(spec->max_thresholds, v);
  }
  return ctx;
}

void gudni_destroy(gudni_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  drop_graph(ctx);
  ctx->geometry.release(); ctx->substances.release(); ctx->pictures.release(); ctx->uses.release();
  ctx->radials.release(); ctx->random_field.release(); ctx->shapes.release(); ctx->tiles.release();
  ctx->strand_table.release(); ctx->strand_y.release(); ctx->strand_first.release();
  ctx->tile_jobs.release(); ctx->out.release();
  ctx->b_shapes.release(); ctx->b_tiles.release(); ctx->b_tile_scene.release(); ctx->b_order.release();
  ctx->b_scenes.release(); ctx->b_out.release(); ctx->f_units.release(); ctx->f_order_words.release();
  ctx->thr.release(); ctx->hdr.release(); ctx->idx.release(); ctx->big_thr.release(); ctx->big_hdr.release();
  ctx->big_idx.release(); ctx->overflow_items.release(); ctx->words.release(); ctx->status.release();
  ctx->counters.release();
  ctx->a_thr.release(); ctx->a_hdr.release(); ctx->a_prov.release(); ctx->a_lines.release();
  ctx->a_line_grad.release(); ctx->a_idx.release(); ctx->a_bit_grad.release(); ctx->a_layers.release();
  ctx->a_layer_bits.release();
  ctx->ser_sub_start.release(); ctx->ser_compound.release(); ctx->ser_outline_start.release();
  ctx->ser_pair_start.release(); ctx->ser_pairs.release(); ctx->ser_sub_tag.release();
  for (auto& b : ctx->ser_tmp) b.release();
  ctx->ds_shapes.release(); ctx->ds_tiles.release(); ctx->ds_tile_jobs.release();
  ctx->ds_point_offsets.release(); ctx->ds_point_sources.release(); ctx->ds_point_weights.release();
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* gudni_last_error(const gudni_ctx* ctx) {
  if (!ctx) return g_create_error.c_str();
  return ctx->error.c_str();
}

int gudni_upload_common(gudni_ctx* ctx, const void* geometry, size_t geometry_bytes, const float* substances,
                        size_t n_substances, const uint8_t* pictures, size_t picture_bytes,
                        const gudni_picture_use* picture_uses, size_t n_picture_uses, const gudni_radial* radials,
                        size_t n_radials, const float* random_field) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  cudaSetDevice(ctx->device);
  ctx->batch_ready = false;
  drop_graph(ctx);
  int rc = upload_common_buffers(ctx, geometry, geometry_bytes, substances, n_substances, pictures, picture_bytes,
                                 picture_uses, n_picture_uses, radials, n_radials, random_field);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "upload");
  ctx->common_ready = true;
  return GUDNI_OK;
}

int gudni_upload_pictures(gudni_ctx* ctx, const uint8_t* pictures, size_t picture_bytes) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if (picture_bytes && !pictures) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null picture pile with non-zero size");
  cudaSetDevice(ctx->device);
  ctx->batch_ready = false;  // a batch's usages index the pile its own upload brought
  drop_graph(ctx);
  // the uploaded frame stays usable only while its usages still read inside the pile
  const bool keep_frame = ctx->common_ready && ctx->uses_extent <= picture_bytes;
  ctx->common_ready = false;
  ctx->picture_bytes = 0;
  int rc = upload(ctx, ctx->pictures, pictures, picture_bytes, "picture upload");
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "picture upload");
  ctx->picture_bytes = picture_bytes;
  ctx->common_ready = keep_frame;
  return GUDNI_OK;
}

int gudni_upload_random_field(gudni_ctx* ctx, const float* random_field) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  cudaSetDevice(ctx->device);
  drop_graph(ctx);
  ctx->has_random = false;
  if (!random_field) return GUDNI_OK;
  int rc = upload(ctx, ctx->random_field, random_field, GUDNI_RANDOM_FIELD_SIZE, "random field upload");
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "random field upload");
  ctx->has_random = true;
  return GUDNI_OK;
}

int gudni_upload_frame(gudni_ctx* ctx, const void* geometry, size_t geometry_bytes, const float* substances,
                       size_t n_substances, const gudni_picture_use* picture_uses, size_t n_picture_uses,
                       const gudni_radial* radials, size_t n_radials) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  cudaSetDevice(ctx->device);
  ctx->batch_ready = false;
  drop_graph(ctx);
  if ((geometry_bytes && !geometry) || (n_substances && !substances) || (n_picture_uses && !picture_uses) ||
      (n_radials && !radials))
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "null buffer with non-zero size");
  if (geometry_bytes % 16 != 0) return fail(ctx, GUDNI_ERR_BAD_INPUT, "geometry pile must be a multiple of 16 bytes");
  uint64_t extent = 0;
  int rc = check_picture_uses(ctx, picture_uses, n_picture_uses, ctx->picture_bytes, &extent);
  if (rc) return rc;
  ctx->common_ready = false;
  if ((rc = upload(ctx, ctx->geometry, geometry, geometry_bytes, "geometry upload"))) return rc;
  if ((rc = upload(ctx, ctx->substances, substances, n_substances, "substance upload"))) return rc;
  if ((rc = upload(ctx, ctx->uses, picture_uses, n_picture_uses, "picture use upload"))) return rc;
  if ((rc = upload(ctx, ctx->radials, radials, n_radials, "radial upload"))) return rc;
  cudaError_t e;
  if (!ctx->pictures.ptr && (e = ctx->pictures.reserve(0)) != cudaSuccess)  // never hand the kernels a null pile
    return cuda_fail(ctx, e, "picture pile");
  if ((rc = strand_table_of(ctx, geometry, geometry_bytes))) return rc;
  ctx->geometry_bytes = geometry_bytes;
  ctx->n_substances = n_substances;
  ctx->n_uses = n_picture_uses;
  ctx->uses_extent = extent;
  ctx->n_radials = n_radials;
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "upload");
  ctx->common_ready = true;
  return GUDNI_OK;
}

int gudni_serialize_device(gudni_ctx* ctx, const struct gudni_scene_desc* s, int flags, gudni_device_frame* frame) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if (!s || !frame) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null scene or frame");
  gudni::ser::Scene sc;
  int64_t n_pairs = 0;
  std::vector<float4> subs;
  std::vector<gudni_picture_use> uses;
  std::vector<gudni_radial> rads;
  std::vector<uint64_t> tags;
  const char* why = gudni::ser::checkScene(s, ctx->spec, sc, n_pairs);
  if (!why) why = gudni::ser::buildSubstances(s, subs, uses, rads, tags);
  if (why) return fail(ctx, GUDNI_ERR_BAD_INPUT, why);
  uint64_t extent = 0;
  int rc = check_picture_uses(ctx, uses.data(), uses.size(), ctx->picture_bytes, &extent);
  if (rc) return rc;
  cudaSetDevice(ctx->device);
  ctx->batch_ready = false;
  drop_graph(ctx);
  ctx->common_ready = false;
  const size_t n_sub = (size_t)s->n_substances;
  if ((rc = upload(ctx, ctx->substances, subs.data(), subs.size(), "substance upload"))) return rc;
  if ((rc = upload(ctx, ctx->uses, uses.data(), uses.size(), "picture use upload"))) return rc;
  if ((rc = upload(ctx, ctx->radials, rads.data(), rads.size(), "radial upload"))) return rc;
  if ((rc = upload(ctx, ctx->ser_sub_tag, tags.data(), tags.size(), "scene upload"))) return rc;
  if ((rc = upload(ctx, ctx->ser_sub_start, s->substance_shape_start, n_sub ? n_sub + 1 : 0, "scene upload"))) return rc;
  const size_t shapes_end = (size_t)sc.shape1, outlines_end = (size_t)sc.outline1;
  const bool any_shape = sc.shape1 > sc.shape0, any_outline = sc.outline1 > sc.outline0;
  if ((rc = upload(ctx, ctx->ser_compound, s->shape_compound, any_shape ? shapes_end : 0, "scene upload"))) return rc;
  if ((rc = upload(ctx, ctx->ser_outline_start, s->shape_outline_start, any_shape ? shapes_end + 1 : 0, "scene upload")))
    return rc;
  if ((rc = upload(ctx, ctx->ser_pair_start, s->outline_pair_start, any_outline ? outlines_end + 1 : 0, "scene upload")))
    return rc;
  if ((rc = upload(ctx, ctx->ser_pairs, s->pairs, any_outline ? 4 * (size_t)n_pairs : 0, "scene upload"))) return rc;
  cudaError_t e;
  if (!ctx->pictures.ptr && (e = ctx->pictures.reserve(0)) != cudaSuccess) return cuda_fail(ctx, e, "picture pile");
  sc.substance_shape_start = ctx->ser_sub_start.ptr;
  sc.substance_tag = ctx->ser_sub_tag.ptr;
  sc.shape_compound = ctx->ser_compound.ptr;
  sc.shape_outline_start = ctx->ser_outline_start.ptr;
  sc.outline_pair_start = ctx->ser_pair_start.ptr;
  sc.pairs = ctx->ser_pairs.ptr;
  gudni::ser::Limits lim{ctx->spec.max_tile_size, ctx->spec.threads_per_tile, ctx->spec.max_tiles_per_call,
                         ctx->spec.max_shape, (int64_t)ctx->spec.max_strands_per_tile};
  SerExec ex{ctx, ctx->stream};
  gudni::ser::Result res;
  rc = gudni::ser::serialize(ex, sc, lim, res, (flags & GUDNI_SERIALIZE_PROVENANCE) != 0);
  if (rc == -2) return fail(ctx, GUDNI_ERR_BAD_INPUT, "scene too large for the device serializer");
  if (rc) return cuda_fail(ctx, ex.err, "device serializer");
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(ctx, e, "device serializer");
  ctx->geometry_bytes = res.geometry_bytes;
  ctx->n_strands = res.n_strands;
  ctx->n_units = res.geometry_bytes / 16;
  ctx->n_substances = subs.size();
  ctx->n_uses = uses.size();
  ctx->uses_extent = extent;
  ctx->n_radials = rads.size();
  ctx->common_ready = true;
  frame->geometry_bytes = res.geometry_bytes;
  frame->n_strands = res.n_strands;
  frame->n_shapes = res.n_shapes;
  frame->n_tiles = res.n_tiles;
  frame->n_jobs = res.n_jobs;
  std::memcpy(frame->stats, res.stats, sizeof(frame->stats));
  frame->geometry = res.geometry;
  frame->shapes = res.shapes;
  frame->tiles = res.tiles;
  frame->tile_jobs = res.tile_jobs;
  frame->n_points = res.n_points;
  frame->point_offsets = res.point_offsets;
  frame->point_sources = res.point_sources;
  frame->point_weights = res.point_weights;
  return GUDNI_OK;
}

int gudni_device_frame_download(gudni_ctx* ctx, const gudni_device_frame* frame, uint8_t* geometry,
                                gudni_shape* shapes, gudni_tile_info* tiles, int32_t* tile_jobs,
                                uint32_t* point_offsets, int32_t* point_sources, float* point_weights) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if (!frame) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null frame");
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaSuccess;
  auto get = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && dst && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
  };
  get(geometry, frame->geometry, frame->geometry_bytes);
  get(shapes, frame->shapes, frame->n_shapes * sizeof(gudni_shape));
  get(tiles, frame->tiles, frame->n_tiles * sizeof(gudni_tile_info));
  get(tile_jobs, frame->tile_jobs, frame->n_tiles * sizeof(int32_t));
  if (frame->n_points && !frame->point_offsets) return fail(ctx, GUDNI_ERR_BAD_INPUT, "frame has no provenance");
  get(point_offsets, frame->point_offsets, frame->n_points * sizeof(uint32_t));
  get(point_sources, frame->point_sources, frame->n_points * 3 * sizeof(int32_t));
  get(point_weights, frame->point_weights, frame->n_points * 3 * sizeof(float));
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "device frame download");
  return GUDNI_OK;
}

int gudni_raster_job(gudni_ctx* ctx, const gudni_shape* shapes, size_t n_shapes, const gudni_tile_info* tiles,
                     size_t n_tiles, int32_t columns_to_alloc, int32_t bitmap_w, int32_t bitmap_h,
                     int32_t compute_depth, int32_t frame_number, int32_t job_index, const float background[4],
                     uint32_t* out) {
  (void)columns_to_alloc;
  (void)frame_number;
  int rc = validate_job(ctx, shapes, n_shapes, tiles, n_tiles, bitmap_w, bitmap_h, compute_depth, true);
  if (rc) return rc;
  if (!out || !background) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null out or background");
  cudaSetDevice(ctx->device);
  const size_t pixels = (size_t)bitmap_w * (size_t)bitmap_h;
  if ((rc = upload(ctx, ctx->shapes, shapes, n_shapes, "shape upload"))) return rc;
  if ((rc = upload(ctx, ctx->tiles, tiles, n_tiles, "tile upload"))) return rc;
  // pixels outside this job's tiles keep the caller's values (the reference reads
  // the whole target back through a host-pointer buffer, Instances.hs:60-75)
  if ((rc = upload(ctx, ctx->out, out, pixels, "bitmap upload"))) return rc;
  gudni::RasterInputs in = inputs(ctx, ctx->shapes.ptr, n_shapes, ctx->tiles.ptr, n_tiles, bitmap_w, bitmap_h,
                                  compute_depth, job_index, background, ctx->out.ptr);
  if ((rc = enqueue(ctx, in, nullptr, nullptr, 0, nullptr, 0, gudni::chunkLog2(compute_depth), n_tiles,
                    ctx->spec.threads_per_tile, ctx->stream)))
    return rc;
  cudaError_t e = cudaMemcpyAsync(out, ctx->out.ptr, pixels * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "bitmap read-back");
  return read_status(ctx, ctx->stream);
}

int gudni_raster_job_device(gudni_ctx* ctx, const gudni_shape* shapes, size_t n_shapes, const gudni_tile_info* tiles,
                            size_t n_tiles, int32_t columns_to_alloc, int32_t bitmap_w, int32_t bitmap_h,
                            int32_t compute_depth, int32_t frame_number, int32_t job_index,
                            const float background[4], uint32_t* out, void* stream) {
  (void)columns_to_alloc;
  (void)frame_number;
  int rc = validate_job(ctx, shapes, n_shapes, tiles, n_tiles, bitmap_w, bitmap_h, compute_depth, false);
  if (rc) return rc;
  if (!out || !background) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null out or background");
  if (((uintptr_t)shapes & 7) != 0 || ((uintptr_t)tiles & 3) != 0 || ((uintptr_t)out & 3) != 0)
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "misaligned device pointer");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  ctx->last_stream = s;
  gudni::RasterInputs in = inputs(ctx, shapes, n_shapes, tiles, n_tiles, bitmap_w, bitmap_h, compute_depth,
                                  job_index, background, out);
  return enqueue(ctx, in, nullptr, nullptr, 0, nullptr, 0, gudni::chunkLog2(compute_depth), n_tiles,
                 ctx->spec.threads_per_tile, s);
}

int gudni_raster_frame(gudni_ctx* ctx, const gudni_job_desc* jobs, size_t n_jobs, int32_t bitmap_w,
                       int32_t bitmap_h, int32_t compute_depth, int32_t frame_number, const float background[4],
                       uint32_t* out) {
  (void)frame_number;
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if ((n_jobs && !jobs) || !out || !background) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null argument");
  // concatenate the jobs' piles; each tile's shape slice is offset into the whole
  ctx->h_shapes.clear();
  ctx->h_tiles.clear();
  ctx->h_tile_jobs.clear();
  for (size_t j = 0; j < n_jobs; ++j) {
    const gudni_job_desc& d = jobs[j];
    int rc = validate_job(ctx, d.shapes, d.n_shapes, d.tiles, d.n_tiles, bitmap_w, bitmap_h, compute_depth, true);
    if (rc) return rc;
    const uint32_t base = (uint32_t)ctx->h_shapes.size();
    ctx->h_shapes.insert(ctx->h_shapes.end(), d.shapes, d.shapes + d.n_shapes);
    for (size_t t = 0; t < d.n_tiles; ++t) {
      gudni_tile_info ti = d.tiles[t];
      ti.shapes.start += base;
      ctx->h_tiles.push_back(ti);
      ctx->h_tile_jobs.push_back((int32_t)j);
    }
  }
  if (((uint64_t)ctx->h_tiles.size() << gudni::chunkLog2(compute_depth)) >= gudni::kMaxUnits)
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "too many tiles in one frame");
  cudaSetDevice(ctx->device);
  int rc;
  const size_t pixels = (size_t)bitmap_w * (size_t)bitmap_h;
  if ((rc = upload(ctx, ctx->shapes, ctx->h_shapes.data(), ctx->h_shapes.size(), "shape upload"))) return rc;
  if ((rc = upload(ctx, ctx->tiles, ctx->h_tiles.data(), ctx->h_tiles.size(), "tile upload"))) return rc;
  if ((rc = upload(ctx, ctx->tile_jobs, ctx->h_tile_jobs.data(), ctx->h_tile_jobs.size(), "tile job upload"))) return rc;
  cudaError_t e = ctx->out.reserve(pixels);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "bitmap");
  gudni::RasterInputs in = inputs(ctx, ctx->shapes.ptr, ctx->h_shapes.size(), ctx->tiles.ptr, ctx->h_tiles.size(),
                                  bitmap_w, bitmap_h, compute_depth, 0, background, ctx->out.ptr);
  in.tile_jobs = ctx->tile_jobs.ptr;
  if ((rc = enqueue(ctx, in, nullptr, nullptr, 0, nullptr, 0, gudni::chunkLog2(compute_depth), ctx->h_tiles.size(),
                    ctx->spec.threads_per_tile, ctx->stream)))
    return rc;
  e = cudaMemcpyAsync(out, ctx->out.ptr, pixels * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "bitmap read-back");
  return read_status(ctx, ctx->stream);
}

int gudni_raster_tiles_device(gudni_ctx* ctx, const gudni_shape* shapes, size_t n_shapes,
                              const gudni_tile_info* tiles, const int32_t* tile_jobs, size_t n_tiles,
                              int32_t bitmap_w, int32_t bitmap_h, int32_t compute_depth, int32_t frame_number,
                              const float background[4], uint32_t* out, void* stream) {
  (void)frame_number;
  int rc = validate_job(ctx, shapes, n_shapes, tiles, n_tiles, bitmap_w, bitmap_h, compute_depth, false);
  if (rc) return rc;
  if (!out || !background) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null out or background");
  if (((uintptr_t)shapes & 7) != 0 || ((uintptr_t)tiles & 3) != 0 || ((uintptr_t)out & 3) != 0 ||
      ((uintptr_t)tile_jobs & 3) != 0)
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "misaligned device pointer");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  ctx->last_stream = s;
  gudni::RasterInputs in = inputs(ctx, shapes, n_shapes, tiles, n_tiles, bitmap_w, bitmap_h, compute_depth, 0,
                                  background, out);
  in.tile_jobs = tile_jobs;
  return enqueue(ctx, in, nullptr, nullptr, 0, nullptr, 0, gudni::chunkLog2(compute_depth), n_tiles,
                 ctx->spec.threads_per_tile, s);
}

int gudni_batch_upload(gudni_ctx* ctx, const void* geometry, size_t geometry_bytes, const float* substances,
                       size_t n_substances, const uint8_t* pictures, size_t picture_bytes,
                       const gudni_picture_use* picture_uses, size_t n_picture_uses, const gudni_radial* radials,
                       size_t n_radials, const gudni_shape* shapes, size_t n_shapes, const gudni_tile_info* tiles,
                       const int32_t* tile_scene, const float* tile_cost, size_t n_tiles,
                       const gudni_batch_scene* scenes, size_t n_scenes, size_t out_pixels) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  cudaSetDevice(ctx->device);
  ctx->batch_ready = false;
  drop_graph(ctx);
  if ((n_tiles && (!tiles || !tile_scene)) || (n_scenes && !scenes) || (n_shapes && !shapes))
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "null batch array");
  if ((uint64_t)n_tiles * 32 >= gudni::kMaxUnits) return fail(ctx, GUDNI_ERR_BAD_INPUT, "too many tiles");
  int rc = validate_tiles_host(ctx, tiles, n_tiles, n_shapes);
  if (rc) return rc;
  int max_tpt = 1;
  std::vector<gudni::SceneInfo> sc(n_scenes);
  for (size_t i = 0; i < n_scenes; ++i) {
    const gudni_batch_scene& b = scenes[i];
    if (b.bitmap_w <= 0 || b.bitmap_h <= 0 || b.compute_depth < 0 || b.compute_depth > gudni::kMaxLog2Tpt ||
        b.out_offset + (uint64_t)b.bitmap_w * (uint64_t)b.bitmap_h > out_pixels)
      return fail(ctx, GUDNI_ERR_BAD_INPUT, "batch scene " + std::to_string(i) + " is malformed");
    sc[i].bitmap_w = b.bitmap_w;
    sc[i].bitmap_h = b.bitmap_h;
    sc[i].log2_tpt = b.compute_depth;
    sc[i].job_index = b.job_index;
    sc[i].out_offset = b.out_offset;
    std::memcpy(sc[i].background, b.background, sizeof(sc[i].background));
    max_tpt = std::max(max_tpt, 1 << b.compute_depth);
  }
  for (size_t t = 0; t < n_tiles; ++t)
    if (tile_scene[t] < 0 || (size_t)tile_scene[t] >= n_scenes)
      return fail(ctx, GUDNI_ERR_BAD_INPUT, "tile " + std::to_string(t) + " names no scene");
  // work units: every tile's 32-column chunks; scheduled most expensive first
  // (longest-processing-time order, a tile's cost shared by its chunks)
  std::vector<uint32_t> order;
  std::vector<float> unit_cost;
  int chunk_log2_max = 0;
  for (size_t t = 0; t < n_tiles; ++t) {
    const int cl = gudni::chunkLog2(scenes[tile_scene[t]].compute_depth);
    chunk_log2_max = std::max(chunk_log2_max, cl);
    for (int c = 0; c < (1 << cl); ++c) {
      order.push_back(((uint32_t)t << gudni::kChunkBits) | (uint32_t)c);
      unit_cost.push_back(tile_cost ? tile_cost[t] / (float)(1 << cl) : 0.0f);
    }
  }
  if (tile_cost) {
    std::vector<uint32_t> idx(order.size());
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return unit_cost[a] > unit_cost[b]; });
    std::vector<uint32_t> sorted(order.size());
    for (size_t i = 0; i < idx.size(); ++i) sorted[i] = order[idx[i]];
    order.swap(sorted);
  }
  if ((rc = upload_common_buffers(ctx, geometry, geometry_bytes, substances, n_substances, pictures, picture_bytes,
                                  picture_uses, n_picture_uses, radials, n_radials, nullptr)))
    return rc;
  if ((rc = upload(ctx, ctx->b_shapes, shapes, n_shapes, "batch shapes"))) return rc;
  if ((rc = upload(ctx, ctx->b_tiles, tiles, n_tiles, "batch tiles"))) return rc;
  if ((rc = upload(ctx, ctx->b_tile_scene, tile_scene, n_tiles, "batch tile scenes"))) return rc;
  if ((rc = upload(ctx, ctx->b_order, order.data(), order.size(), "batch work units"))) return rc;
  if ((rc = upload(ctx, ctx->b_scenes, sc.data(), n_scenes, "batch scenes"))) return rc;
  cudaError_t e = ctx->b_out.reserve(out_pixels);
  if (e == cudaSuccess) e = cudaMemsetAsync(ctx->b_out.ptr, 0, out_pixels * 4, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batch upload");
  if ((rc = ensure_scratch(ctx))) return rc;
  if (ctx->working_capacity < ctx->spec.max_thresholds) {
    if ((e = ctx->overflow_items.reserve(n_tiles * (size_t)max_tpt)) != cudaSuccess) return cuda_fail(ctx, e, "overflow list");
    if ((rc = ensure_fallback_pool(ctx))) return rc;
  }
  ctx->common_ready = true;
  ctx->batch_tiles = n_tiles;
  ctx->batch_shapes = n_shapes;
  ctx->batch_scenes = n_scenes;
  ctx->batch_pixels = out_pixels;
  ctx->batch_units = order.size();
  ctx->batch_chunk_log2 = chunk_log2_max;
  ctx->batch_ready = true;
  return GUDNI_OK;
}

static int batch_enqueue(gudni_ctx* ctx, cudaStream_t s) {
  gudni::RasterInputs in = inputs(ctx, ctx->b_shapes.ptr, ctx->batch_shapes, ctx->b_tiles.ptr, ctx->batch_tiles, 1,
                                  1, 0, 0, nullptr, ctx->b_out.ptr);
  int max_tpt = 1 << gudni::kMaxLog2Tpt;
  if (ctx->overflow_items.cap && ctx->batch_tiles) max_tpt = (int)std::min<size_t>(max_tpt, ctx->overflow_items.cap / ctx->batch_tiles);
  return enqueue(ctx, in, ctx->b_scenes.ptr, ctx->b_tile_scene.ptr, ctx->batch_scenes, ctx->b_order.ptr,
                 ctx->batch_units, 0, ctx->batch_tiles, max_tpt, s);
}

int gudni_batch_render(gudni_ctx* ctx, int use_graph, void* stream) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if (!ctx->batch_ready) return fail(ctx, GUDNI_ERR_NOT_READY, "gudni_batch_upload has not been called");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  ctx->last_stream = s;
  if (!use_graph || ctx->counters_on) return batch_enqueue(ctx, s);
  if (!ctx->graph_exec) {
    // capture the launch sequence once on the context's own stream
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture");
    const uint64_t launches = ctx->launches;
    int rc = batch_enqueue(ctx, ctx->stream);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture");
    ctx->launches = launches;  // counted when replayed
    ctx->graph = g;
    if ((e = cudaGraphInstantiate(&ctx->graph_exec, g, 0)) != cudaSuccess) {
      drop_graph(ctx);
      return cuda_fail(ctx, e, "graph instantiate");
    }
  }
  cudaError_t e = cudaGraphLaunch(ctx->graph_exec, s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "graph launch");
  ctx->launches += ctx->working_capacity < ctx->spec.max_thresholds ? 2 : 1;
  return GUDNI_OK;
}

int gudni_batch_render_tiles(gudni_ctx* ctx, size_t first_tile, size_t n_tiles, void* stream) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if (!ctx->batch_ready) return fail(ctx, GUDNI_ERR_NOT_READY, "gudni_batch_upload has not been called");
  if (first_tile > ctx->batch_tiles || n_tiles > ctx->batch_tiles - first_tile)
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "tile range outside the batch");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  ctx->last_stream = s;
  gudni::RasterInputs in = inputs(ctx, ctx->b_shapes.ptr, ctx->batch_shapes, ctx->b_tiles.ptr + first_tile, n_tiles,
                                  1, 1, 0, 0, nullptr, ctx->b_out.ptr);
  int max_tpt = 1 << gudni::kMaxLog2Tpt;
  if (ctx->overflow_items.cap && ctx->batch_tiles) max_tpt = (int)std::min<size_t>(max_tpt, ctx->overflow_items.cap / ctx->batch_tiles);
  // chunks of the batch's widest scene: units past a tile's own columns do nothing
  return enqueue(ctx, in, ctx->b_scenes.ptr, ctx->b_tile_scene.ptr + first_tile, ctx->batch_scenes, nullptr, 0,
                 ctx->batch_chunk_log2, n_tiles, max_tpt, s);
}

const uint32_t* gudni_batch_output(const gudni_ctx* ctx) { return ctx ? ctx->b_out.ptr : nullptr; }

int gudni_batch_download(gudni_ctx* ctx, uint32_t* out) {
  if (!ctx || !out) return GUDNI_ERR_BAD_INPUT;
  if (!ctx->batch_ready) return fail(ctx, GUDNI_ERR_NOT_READY, "no batch");
  cudaSetDevice(ctx->device);
  if (ctx->last_stream && ctx->last_stream != ctx->stream) {
    cudaError_t e = cudaStreamSynchronize(ctx->last_stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "stream sync");
  }
  cudaError_t e = cudaMemcpyAsync(out, ctx->b_out.ptr, ctx->batch_pixels * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batch read-back");
  return read_status(ctx, ctx->stream);
}

int gudni_sync_status(gudni_ctx* ctx) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  cudaSetDevice(ctx->device);
  if (ctx->last_stream && ctx->last_stream != ctx->stream) {
    cudaError_t e = cudaStreamSynchronize(ctx->last_stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "stream sync");
  }
  return read_status(ctx, ctx->stream);
}

size_t gudni_scratch_bytes(const gudni_ctx* ctx) {
  if (!ctx) return 0;
  return ctx->thr.cap * sizeof(float4) + ctx->hdr.cap * 4 + ctx->idx.cap * 4 + ctx->big_thr.cap * sizeof(float4) +
         ctx->big_hdr.cap * 4 + ctx->big_idx.cap * 4;
}

int gudni_enable_counters(gudni_ctx* ctx, int enable) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  cudaSetDevice(ctx->device);
  int rc = ensure_scratch(ctx);
  if (rc) return rc;
  cudaError_t e = cudaMemsetAsync(ctx->counters.ptr, 0, 4 * sizeof(int64_t), ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "counters");
  ctx->counters_on = enable != 0;
  return GUDNI_OK;
}

int gudni_set_device_strand_table(gudni_ctx* ctx, int enable) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  ctx->device_strands = enable != 0;
  return GUDNI_OK;
}

int gudni_set_random_source(gudni_ctx* ctx, int source, uint64_t seed) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if (source != GUDNI_RANDOM_FIELD && source != GUDNI_RANDOM_COUNTER)
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "unknown random source");
  drop_graph(ctx);  // a captured batch holds the old setting
  ctx->random_mode = source == GUDNI_RANDOM_COUNTER ? gudni::kRandomCounter : gudni::kRandomField;
  ctx->random_seed = seed;
  return GUDNI_OK;
}

int gudni_set_dense_columns(gudni_ctx* ctx, int32_t min_thresholds) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if (min_thresholds < 0) return fail(ctx, GUDNI_ERR_BAD_INPUT, "min_thresholds must be >= 0");
  if (min_thresholds != ctx->dense_min) drop_graph(ctx);  // a captured launch holds the old setting
  ctx->dense_min = min_thresholds;
  return GUDNI_OK;
}

int gudni_set_cooperative_units(gudni_ctx* ctx, int mode) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  const int m = mode > 0 ? 1 : (mode == 0 ? 0 : -1);
  if (m != ctx->coop) drop_graph(ctx);  // a captured launch holds the old setting
  ctx->coop = m;
  return GUDNI_OK;
}

int gudni_set_adjoint_regenerate(gudni_ctx* ctx, int on) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  ctx->adj_regenerate = on ? 1 : 0;
  return GUDNI_OK;
}

int gudni_read_counters(gudni_ctx* ctx, int64_t out[4]) {
  if (!ctx || !out) return GUDNI_ERR_BAD_INPUT;
  cudaSetDevice(ctx->device);
  int rc = ensure_scratch(ctx);
  if (rc) return rc;
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(out, ctx->counters.ptr, 4 * sizeof(int64_t), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(ctx->counters.ptr, 0, 4 * sizeof(int64_t));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "counters");
  return GUDNI_OK;
}

uint64_t gudni_launch_count(const gudni_ctx* ctx) { return ctx ? ctx->launches : 0; }

int gudni_adjoint_tiles_device(gudni_ctx* ctx, const gudni_shape* shapes, size_t n_shapes,
                               const gudni_tile_info* tiles, const int32_t* tile_jobs, size_t n_tiles,
                               int32_t bitmap_w, int32_t bitmap_h, int32_t compute_depth, const float background[4],
                               const float* target, float* image, float* grad_geometry, float* grad_substances,
                               void* stream) {
  int rc = validate_job(ctx, shapes, n_shapes, tiles, n_tiles, bitmap_w, bitmap_h, compute_depth, false);
  if (rc) return rc;
  if (!background) return fail(ctx, GUDNI_ERR_BAD_INPUT, "null background");
  if (!adjoint_pointers_ok(target, image, grad_geometry, grad_substances))
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "null or misaligned target, image or gradient pointer");
  if (((uintptr_t)shapes & 7) != 0 || ((uintptr_t)tiles & 3) != 0 || ((uintptr_t)tile_jobs & 3) != 0)
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "misaligned device pointer");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  ctx->last_stream = s;
  gudni::RasterInputs in = inputs(ctx, shapes, n_shapes, tiles, n_tiles, bitmap_w, bitmap_h, compute_depth, 0,
                                  background, nullptr);
  in.tile_jobs = tile_jobs;
  return enqueue_adjoint(ctx, in, nullptr, nullptr, 0, nullptr, 0, gudni::chunkLog2(compute_depth), n_tiles,
                         target, image, grad_geometry, grad_substances, s);
}

int gudni_batch_adjoint(gudni_ctx* ctx, const float* target, float* image, float* grad_geometry,
                        float* grad_substances, void* stream) {
  if (!ctx) return GUDNI_ERR_BAD_INPUT;
  if (!ctx->batch_ready) return fail(ctx, GUDNI_ERR_NOT_READY, "gudni_batch_upload has not been called");
  if (!adjoint_pointers_ok(target, image, grad_geometry, grad_substances))
    return fail(ctx, GUDNI_ERR_BAD_INPUT, "null or misaligned target, image or gradient pointer");
  cudaSetDevice(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  ctx->last_stream = s;
  gudni::RasterInputs in = inputs(ctx, ctx->b_shapes.ptr, ctx->batch_shapes, ctx->b_tiles.ptr, ctx->batch_tiles, 1,
                                  1, 0, 0, nullptr, nullptr);
  return enqueue_adjoint(ctx, in, ctx->b_scenes.ptr, ctx->b_tile_scene.ptr, ctx->batch_scenes, ctx->b_order.ptr,
                         ctx->batch_units, 0, ctx->batch_tiles, target, image, grad_geometry, grad_substances, s);
}

}  // extern "C"
