// No-allocation entry point: gudni_raster_job_noalloc (include/gudni_cuda.h).
//
// Some callers cannot allocate device memory: a plugin running inside another
// framework's memory pool or allocator, a sandbox without allocation rights, or a
// real-time loop where cudaMalloc's implicit device synchronisation is not allowed.
// For them, the per-column threshold queues and shape-index tables live in one
// fixed array compiled into this library (GUDNI_NOALLOC_SCRATCH_BYTES), and every
// input and output buffer is the caller's.  Nothing here calls cudaMalloc, cudaFree
// or any allocating routine.
//
// The array is a file-scope __device__ symbol.  In host code its name is only a
// host-side stand-in, not a device address, so the first call on each device looks
// the address up with cudaGetSymbolAddress (with that device current) and caches it;
// that first call should come before any stream capture.  The cached address belongs
// to the device's primary context: after cudaDeviceReset the module is loaded again
// and the array may move, so a process that resets a device must not call this entry
// point on it again.  All calls share the array and it keeps the previous call's
// contents: the status word and the work counter are cleared at the start of every
// call, and calls whose launches overlap on the GPU race on it.
//
// Width of the launch: at the default capacity of 512 thresholds per column and a
// max_shape of 127 one slot takes 10,748 bytes, so the array holds 6,144 slots -- 48
// blocks of 128 threads, fewer blocks than the GPU has SMs.  The array trades that
// width for needing no allocation; the context entry points size their scratch to the
// whole GPU.

#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "gudni_cuda.h"
#include "raster_kernels.h"

namespace gudni {
void set_global_error(const std::string& msg);
}

namespace {

constexpr size_t kScratchBytes = GUDNI_NOALLOC_SCRATCH_BYTES;
constexpr size_t kHeaderBytes = 256;   // status word, work counter
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_addr_mutex;
void* g_addr[kMaxDevices] = {nullptr};

int fail(int code, const std::string& msg) {
  gudni::set_global_error("gudni_raster_job_noalloc: " + msg);
  return code;
}

// Device address of the scratch array on the current device (looked up once).
int scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(GUDNI_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(GUDNI_ERR_BAD_INPUT, "device index beyond the address table");
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(GUDNI_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_addr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_addr[dev]);
  return GUDNI_OK;
}

bool aligned(const void* p, uintptr_t a) { return ((uintptr_t)p & (a - 1)) == 0; }

}  // namespace

extern "C" int gudni_raster_job_noalloc(const gudni_spec* spec, const void* geometry, size_t geometry_bytes,
                                        const float* substances, size_t n_substances, const uint8_t* pictures,
                                        size_t picture_bytes, const gudni_picture_use* picture_uses,
                                        size_t n_picture_uses, const gudni_radial* radials, size_t n_radials,
                                        const gudni_shape* shapes, size_t n_shapes, const gudni_tile_info* tiles,
                                        size_t n_tiles, int32_t bitmap_w, int32_t bitmap_h, int32_t compute_depth,
                                        int32_t job_index, const float background[4], uint32_t* out,
                                        void* stream) {
  if (!spec || !background || !out) return fail(GUDNI_ERR_BAD_INPUT, "null spec, background or out");
  if (spec->max_shape < 1 || spec->max_shape > 64 * 32 - 1 || spec->max_thresholds < 4)
    return fail(GUDNI_ERR_BAD_INPUT, "max_shape must be in [1, 2047] and max_thresholds >= 4");
  if (compute_depth < 0 || compute_depth > gudni::kMaxLog2Tpt || (1 << compute_depth) != spec->threads_per_tile)
    return fail(GUDNI_ERR_BAD_INPUT, "compute_depth must be log2(threads_per_tile) <= 10");
  if (bitmap_w <= 0 || bitmap_h <= 0 || (int64_t)bitmap_w * bitmap_h > ((int64_t)1 << 31))
    return fail(GUDNI_ERR_BAD_INPUT, "bitmap size out of range");
  if ((geometry_bytes && !geometry) || (n_substances && !substances) || (picture_bytes && !pictures) ||
      (n_picture_uses && !picture_uses) || (n_radials && !radials) || (n_shapes && !shapes) || (n_tiles && !tiles))
    return fail(GUDNI_ERR_BAD_INPUT, "null buffer with non-zero size");
  if (geometry_bytes % 16 != 0) return fail(GUDNI_ERR_BAD_INPUT, "geometry pile must be a multiple of 16 bytes");
  if (!aligned(geometry, 16) || !aligned(substances, 16) || !aligned(picture_uses, 4) || !aligned(radials, 16) ||
      !aligned(shapes, 8) || !aligned(tiles, 4) || !aligned(out, 4) || !aligned(pictures, 4))
    return fail(GUDNI_ERR_BAD_INPUT, "misaligned device pointer");
  if (compute_depth < 0 || compute_depth > gudni::kMaxLog2Tpt ||
      ((uint64_t)n_tiles << gudni::chunkLog2(compute_depth)) >= gudni::kMaxUnits || n_shapes > 0xFFFFFFFFull)
    return fail(GUDNI_ERR_BAD_INPUT, "too many tiles or shapes");

  if (spec->stochastic_factor != 0.0f)
    return fail(GUDNI_ERR_BAD_INPUT, "stochastic_factor must be 0 on this path (it takes no random field)");

  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  // Nothing is read back before the launch: the records may still be in flight on
  // `stream` (written there by the caller's asynchronous copies), and only work
  // enqueued on that stream is ordered after them.  The kernel checks every record it
  // reads -- each tile against the shape pile and canvas (tileOk), each picture use's
  // offset and texel against the picture pile (readColor) -- and reports a bad one in
  // the status word read below.

  // Carve the fixed scratch: header, then per-slot queues and shape-index tables.
  const int capacity = spec->max_thresholds < GUDNI_NOALLOC_CAPACITY ? spec->max_thresholds : GUDNI_NOALLOC_CAPACITY;
  const size_t per_slot = (size_t)capacity * (sizeof(float4) + sizeof(uint32_t)) + (size_t)spec->max_shape * 4;
  size_t slots = (kScratchBytes - kHeaderBytes) / per_slot;
  slots = (slots / gudni::kRasterBlock) * gudni::kRasterBlock;
  if (slots < (size_t)gudni::kRasterBlock)
    return fail(GUDNI_ERR_BAD_INPUT, "max_shape too large for the fixed no-allocation scratch");
  unsigned char* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  int* status = reinterpret_cast<int*>(base);
  uint32_t* next_tile = reinterpret_cast<uint32_t*>(base + 4);
  float4* thr = reinterpret_cast<float4*>(base + kHeaderBytes);
  uint32_t* hdr = reinterpret_cast<uint32_t*>(base + kHeaderBytes + slots * (size_t)capacity * sizeof(float4));
  uint32_t* idx = hdr + slots * (size_t)capacity;

  // the array keeps the last call's words: clear the status and the work counter
  if ((e = cudaMemsetAsync(base, 0, 8, s)) != cudaSuccess)
    return fail(GUDNI_ERR_CUDA, std::string("clearing the scratch header: ") + cudaGetErrorString(e));
  if (n_tiles > 0) {
    gudni::TileLaunch a;
    std::memset(&a, 0, sizeof(a));
    gudni::RasterInputs& in = a.in;
    in.geometry = static_cast<const uint8_t*>(geometry);
    in.geometry_bytes = geometry_bytes;
    in.substances = reinterpret_cast<const float4*>(substances);
    in.n_substances = (uint32_t)n_substances;
    in.pictures = pictures;
    in.picture_bytes = picture_bytes;
    in.uses = picture_uses;
    in.n_uses = (uint32_t)n_picture_uses;
    in.radials = radials;
    in.n_radials = (uint32_t)n_radials;
    in.random_field = nullptr;  // STOCHASTIC_FACTOR is 0 on this path
    in.stochastic = 0.0f;
    in.shapes = shapes;
    in.n_shapes = (uint32_t)n_shapes;
    in.tiles = tiles;
    in.n_tiles = (int)n_tiles;
    in.log2_tpt = compute_depth;
    in.bitmap_w = bitmap_w;
    in.bitmap_h = bitmap_h;
    in.job_index = job_index;
    in.background = make_float4(background[0], background[1], background[2], background[3]);
    in.max_shape = spec->max_shape;
    in.out = out;
    a.scratch = gudni::ColumnScratch{thr, hdr, idx, capacity, spec->max_shape};
    a.chunk_log2 = gudni::chunkLog2(compute_depth);
    a.n_units = (uint32_t)(n_tiles << a.chunk_log2);
    a.next_tile = next_tile;
    a.status = status;
    const size_t warps_per_block = gudni::kRasterBlock / 32;
    size_t grid = ((size_t)a.n_units + warps_per_block - 1) / warps_per_block;
    if (grid > slots / gudni::kRasterBlock) grid = slots / gudni::kRasterBlock;
    if ((e = gudni::launch_raster(a, false, gudni::sections_for(spec->max_shape), (int)grid, s)) != cudaSuccess)
      return fail(GUDNI_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  }
  int bits = 0;
  if ((e = cudaMemcpyAsync(&bits, status, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return fail(GUDNI_ERR_CUDA, std::string("status read: ") + cudaGetErrorString(e));
  if (bits & gudni::kStatusBadInput) return fail(GUDNI_ERR_BAD_INPUT, "a record points outside its buffer");
  if (bits & gudni::kStatusOverflow)
    return fail(GUDNI_ERR_THRESHOLD_OVERFLOW, "a column needed more than " + std::to_string(capacity) +
                                                  " thresholds (the no-allocation queue capacity)");
  if (bits & gudni::kStatusIterLimit) return fail(GUDNI_ERR_ITER_LIMIT, "a device loop hit its iteration cap");
  return GUDNI_OK;
}
