/*
 * gudni_cuda.h -- C ABI of the GB300 (sm_103a) rasterizer that replaces gudni's
 * OpenCL raster kernels (generateThresholds, sortThresholds, renderThresholds in
 * src/Graphics/Gudni/OpenCL/Kernels.cl).
 *
 * The host keeps the reference's serialized buffer layout.  Every record below is
 * byte-compatible with the pile the Haskell host builds, so a host that today hands
 * those piles to OpenCL hands the same bytes to these entry points.
 *
 * Plain C types only: no CUDA or torch types appear in any signature.  A `stream`
 * argument is a cudaStream_t passed as void* (NULL = the context's own stream).
 */
#ifndef GUDNI_CUDA_H
#define GUDNI_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- records */

/* Slice {start, length}.  Util/Pile.hs:124-143, Kernels.cl:312-315. */
typedef struct gudni_slice {
    uint32_t start;
    uint32_t length;
} gudni_slice;

/* Shape record, 16 bytes.  tag = substance type (bits 63-62), compound type
 * (bits 61-60), substance id (bits 59-0); geo_start is in 16-byte units of the
 * geometry pile; num_strands strands follow back to back.
 * Raster/Types.hs:159-168, Raster/ShapeInfo.hs:89-99, Kernels.cl:318-324. */
typedef struct gudni_shape {
    uint64_t tag;
    uint32_t geo_start;
    uint32_t num_strands;
} gudni_shape;

/* Tile record, 32 bytes.  Raster/Types.hs:176-198, Kernels.cl:335-341. */
typedef struct gudni_tile_info {
    int32_t left, top, right, bottom;   /* tile box in pixels */
    int16_t hdepth, vdepth;             /* log2 width, log2 height */
    int32_t column_allocation;          /* first column slot of the tile in its job */
    gudni_slice shapes;                 /* the tile's shapes in the job's shape pile */
} gudni_tile_info;

/* Picture usage record, 24 bytes.  Figure/Picture.hs:169-205, Kernels.cl:349-354. */
typedef struct gudni_picture_use {
    float translate_x, translate_y;
    int32_t size_x, size_y;
    int32_t mem_offset;                 /* byte offset into the picture pile */
    float scale;
} gudni_picture_use;

/* Radial-gradient record, 48 bytes.  New substance with no counterpart in the
 * reference (which only has solid colours and pictures): colour = inner + (outer -
 * inner) * min(1, |p - centre| / radius), p = the integer pixel position, constant
 * over the pixel like a picture texel.  A substance of this type stores its record
 * index as a uint32 in the .x lane of its substance colour. */
typedef struct gudni_radial {
    float center_x, center_y, radius, pad;
    float inner[4];
    float outer[4];
} gudni_radial;

/* Shape tag bits.  Raster/Constants.hs:74-89. */
#define GUDNI_TAG_SUBSTANCE_MASK  0xC000000000000000ULL
#define GUDNI_TAG_SOLID           0x8000000000000000ULL
#define GUDNI_TAG_PICTURE         0x4000000000000000ULL
#define GUDNI_TAG_RADIAL          0xC000000000000000ULL /* new substance type */
#define GUDNI_TAG_COMPOUND_MASK   0x3000000000000000ULL
#define GUDNI_TAG_CONTINUE        0x1000000000000000ULL
#define GUDNI_TAG_ADD             0x2000000000000000ULL
#define GUDNI_TAG_SUBTRACT        0x3000000000000000ULL
#define GUDNI_TAG_ID_MASK         0x0FFFFFFFFFFFFFFFULL

#define GUDNI_RANDOM_FIELD_SIZE 4096  /* Raster/Constants.hs:68 */

/* Raster specification: the reference's RasterSpec (OpenCL/Rasterizer.hs:37-50) plus
 * the compile-time knobs it injects as #defines (OpenCL/Setup.hs:45-64). */
typedef struct gudni_spec {
    int32_t max_tile_size;          /* specMaxTileSize (power of two) */
    int32_t threads_per_tile;       /* specThreadsPerTile (power of two, >= max_tile_size) */
    int32_t max_strands_per_tile;   /* specMaxStrandsPerTile */
    int32_t max_tiles_per_call;     /* specMaxTilesPerCall */
    int32_t max_thresholds;         /* MAXTHRESHOLDS: threshold queue capacity per column */
    int32_t max_shape;              /* MAXSHAPE: shapes per column (<= 64*stack_sections-1) */
    int32_t stack_sections;         /* SHAPESTACKSECTIONS: 64-bit words of the shape stack */
    float   stochastic_factor;      /* STOCHASTIC_FACTOR (the reference ships 0.0) */
} gudni_spec;

/* ----------------------------------------------------------------- status */

#define GUDNI_OK                      0
#define GUDNI_ERR_BAD_INPUT          -1  /* argument or record out of range */
#define GUDNI_ERR_THRESHOLD_OVERFLOW -2  /* a column needed more than max_thresholds */
#define GUDNI_ERR_ITER_LIMIT         -3  /* a device loop hit its iteration cap */
#define GUDNI_ERR_CUDA               -4  /* a CUDA call failed; see gudni_last_error */
#define GUDNI_ERR_NO_DEVICE          -5
#define GUDNI_ERR_NOT_READY          -6  /* common buffers not uploaded */
#define GUDNI_ERR_OUT_OF_MEMORY      -7

/* ---------------------------------------------------------------- context */

typedef struct gudni_ctx gudni_ctx;

/* Create a rasterizer on CUDA device `device`.  Replaces setupOpenCL
 * (OpenCL/Setup.hs:102-147): there is no JIT step, the spec's knobs are kernel
 * arguments / template parameters.  Returns NULL on failure (gudni_last_error(NULL)
 * then describes why). */
gudni_ctx* gudni_create(const gudni_spec* spec, int device);
void gudni_destroy(gudni_ctx* ctx);

/* Last error message for this context (or the last failed gudni_create when ctx is
 * NULL).  Never NULL. */
const char* gudni_last_error(const gudni_ctx* ctx);

/* Upload the per-frame buffers shared by all jobs: geometry pile, substance pile
 * (4 floats each), picture pile, picture usages, radial gradients and the random
 * field (GUDNI_RANDOM_FIELD_SIZE floats; may be NULL when stochastic_factor is 0).
 * Replaces the BuffersInCommon set-up of queueRasterJobs (OpenCL/CallKernels.hs:
 * 208-240).  Host pointers; copies are made before the call returns. */
int gudni_upload_common(gudni_ctx* ctx,
                        const void* geometry, size_t geometry_bytes,
                        const float* substances, size_t n_substances,
                        const uint8_t* pictures, size_t picture_bytes,
                        const gudni_picture_use* picture_uses, size_t n_picture_uses,
                        const gudni_radial* radials, size_t n_radials,
                        const float* random_field);

/* Buffers that persist across frames.  The reference re-packs every picture of the
 * scene's picture map into a fresh pile and re-uploads it, with the random field, for
 * every frame (makePictData, Figure/Picture.hs:159-167, called from queueRasterJobs,
 * OpenCL/CallKernels.hs:228-240).  Here a picture pile (RGBA8 bytes, pictures at
 * 4-byte aligned offsets) and the random field can be uploaded once and kept on the
 * device; each frame then uploads only its geometry, substances, picture usages and
 * gradients with gudni_upload_frame.  gudni_upload_common replaces all of them.
 *
 * gudni_upload_pictures: the frame already uploaded stays usable when its picture
 * usages still read inside the new pile; otherwise the next raster call returns
 * GUDNI_ERR_NOT_READY until gudni_upload_frame is called.  An uploaded batch is
 * dropped (gudni_batch_upload again).  Like gudni_upload_common, call these when no
 * launch of this context is in flight.  Host pointers; copies are made before the call
 * returns.
 * gudni_upload_random_field: GUDNI_RANDOM_FIELD_SIZE floats; NULL removes the field. */
int gudni_upload_pictures(gudni_ctx* ctx, const uint8_t* pictures, size_t picture_bytes);
int gudni_upload_random_field(gudni_ctx* ctx, const float* random_field);

/* Upload one frame's own buffers (the per-frame part of BuffersInCommon,
 * OpenCL/CallKernels.hs:208-240): geometry pile, substance pile, picture usages --
 * whose offsets point into the resident picture pile and are checked against it --
 * and radial gradients.  The resident picture pile and random field are kept. */
int gudni_upload_frame(gudni_ctx* ctx,
                       const void* geometry, size_t geometry_bytes,
                       const float* substances, size_t n_substances,
                       const gudni_picture_use* picture_uses, size_t n_picture_uses,
                       const gudni_radial* radials, size_t n_radials);

/* The serializer on the device.  gudni_serialize (include/gudni_serialize.h) restates
 * the reference's host path (Raster/Strand.hs, Deknob.hs, ReorderTable.hs,
 * TileTree.hs, Job.hs; OpenCL/CallKernels.hs:244-255) as one walk on the CPU; this
 * entry point computes the same piles on the GPU, byte for byte: the geometry pile
 * (with the strand table the raster kernels read), and the frame's shape and tile
 * piles with the job of every tile, concatenated as gudni_raster_tiles_device takes
 * them (job 0 -- the last job built -- first).  The substance pile, picture usages and
 * radial gradients are built on the host (one record per substance) and uploaded.
 * The result is the context's current frame, as after gudni_upload_frame: picture
 * offsets in `scene` point into the resident picture pile (gudni_upload_pictures) and
 * are checked against it, and the random field is the resident one.  `scene` holds
 * host pointers; its index arrays must be non-decreasing.  Render it with
 * gudni_raster_tiles_device(ctx, frame->shapes, frame->n_shapes, frame->tiles,
 * frame->tile_jobs, frame->n_tiles, ...).  The device pointers in `frame` stay valid
 * until the next upload or serialization on this context.  Blocks until done. */
typedef struct gudni_device_frame {
    size_t geometry_bytes;
    size_t n_strands;
    size_t n_shapes;               /* shape records of all jobs */
    size_t n_tiles;
    size_t n_jobs;
    int64_t stats[8];              /* as gudni_frame_stats */
    const uint8_t* geometry;       /* device */
    const gudni_shape* shapes;     /* device: the jobs' shape piles, job 0 first */
    const gudni_tile_info* tiles;  /* device: shape slices index `shapes` */
    const int32_t* tile_jobs;      /* device: job index of every tile */
    /* with GUDNI_SERIALIZE_PROVENANCE: every point of the geometry pile, in pile order,
     * as gudni_frame_point_* (include/gudni_serialize.h) gives it; else 0 / NULL */
    size_t n_points;
    const uint32_t* point_offsets; /* device: float index of the point's x in the pile */
    const int32_t* point_sources;  /* device: 3 per point */
    const float* point_weights;    /* device: 3 per point */
} gudni_device_frame;

#define GUDNI_SERIALIZE_PROVENANCE 1  /* also record every point's provenance */

struct gudni_scene_desc;  /* include/gudni_serialize.h */
int gudni_serialize_device(gudni_ctx* ctx, const struct gudni_scene_desc* scene, int flags,
                           gudni_device_frame* frame);

/* Copy a device-serialized frame's piles to host memory (any pointer may be NULL to
 * skip that pile): geometry_bytes bytes, n_shapes shapes, n_tiles tiles and job
 * indices, n_points point offsets and 3 * n_points sources and weights.  Blocks until
 * the copies are done. */
int gudni_device_frame_download(gudni_ctx* ctx, const gudni_device_frame* frame, uint8_t* geometry,
                                gudni_shape* shapes, gudni_tile_info* tiles, int32_t* tile_jobs,
                                uint32_t* point_offsets, int32_t* point_sources, float* point_weights);

/* Rasterize one job: the generateThresholds -> sortThresholds -> renderThresholds
 * sequence of generateCall (OpenCL/CallKernels.hs:88-179), fused into one launch.
 * shapes/tiles/out are HOST pointers; `out` receives bitmap_w*bitmap_h BGRA words
 * (only the job's tiles are written).  Blocks until the pixels are in `out`.
 * Arguments follow the kernels' argument lists (Kernels.cl:2030-2040, 2117-2132). */
int gudni_raster_job(gudni_ctx* ctx,
                     const gudni_shape* shapes, size_t n_shapes,
                     const gudni_tile_info* tiles, size_t n_tiles,
                     int32_t columns_to_alloc,
                     int32_t bitmap_w, int32_t bitmap_h,
                     int32_t compute_depth, int32_t frame_number, int32_t job_index,
                     const float background[4],
                     uint32_t* out);

/* Same as gudni_raster_job with DEVICE pointers for shapes, tiles and out, enqueued
 * on `stream` without synchronising.  Errors found on the device are reported by the
 * next gudni_sync_status on this context. */
int gudni_raster_job_device(gudni_ctx* ctx,
                            const gudni_shape* shapes, size_t n_shapes,
                            const gudni_tile_info* tiles, size_t n_tiles,
                            int32_t columns_to_alloc,
                            int32_t bitmap_w, int32_t bitmap_h,
                            int32_t compute_depth, int32_t frame_number, int32_t job_index,
                            const float background[4],
                            uint32_t* out, void* stream);

/* One job of a frame, for gudni_raster_frame (a RasterJob, Raster/Job.hs:72-76). */
typedef struct gudni_job_desc {
    const gudni_shape* shapes;
    size_t n_shapes;
    const gudni_tile_info* tiles;
    size_t n_tiles;
    int32_t columns_to_alloc;
} gudni_job_desc;

/* Rasterize every job of a frame in one launch: the loop of queueRasterJobs
 * (OpenCL/CallKernels.hs:218-242, zipWithM_ raster jobs [0..]) with the job index of
 * jobs[i] equal to i.  Host pointers; the frame's tiles cover the canvas, so every
 * pixel of `out` (bitmap_w*bitmap_h BGRA words) is written.  Blocks until done. */
int gudni_raster_frame(gudni_ctx* ctx, const gudni_job_desc* jobs, size_t n_jobs,
                       int32_t bitmap_w, int32_t bitmap_h, int32_t compute_depth,
                       int32_t frame_number, const float background[4], uint32_t* out);

/* Device-resident form of gudni_raster_frame: the jobs' shape piles concatenated in
 * `shapes`, their tile piles concatenated in `tiles` with each tile's shape slice
 * already offset into the concatenated shapes, and tile_jobs[t] the job index of tile
 * t (may be NULL: all tiles belong to job 0).  Enqueued on `stream`. */
int gudni_raster_tiles_device(gudni_ctx* ctx,
                              const gudni_shape* shapes, size_t n_shapes,
                              const gudni_tile_info* tiles, const int32_t* tile_jobs, size_t n_tiles,
                              int32_t bitmap_w, int32_t bitmap_h, int32_t compute_depth,
                              int32_t frame_number, const float background[4],
                              uint32_t* out, void* stream);

/* ------------------------------------------------------------------ batches */

/* One scene of a batch (40 bytes). */
typedef struct gudni_batch_scene {
    int32_t bitmap_w, bitmap_h;
    int32_t compute_depth;          /* log2 threads per tile of this scene's spec */
    int32_t job_index;
    uint64_t out_offset;            /* first pixel of the scene in the batch output */
    float background[4];
} gudni_batch_scene;

/* Upload a batch of scenes rendered together by gudni_batch_render (no counterpart in
 * the reference, which renders one scene per frame): the scenes' common piles
 * concatenated (geometry, substances, pictures, picture uses, radial gradients, with
 * every shape's geo_start, every tag's substance id and every substance's picture /
 * gradient id rebased into the concatenation), their shape piles concatenated, their
 * tile piles concatenated with each tile's shape slice rebased, the scene of every
 * tile, and the scene table.  Tiles are scheduled in descending `tile_cost` (NULL:
 * input order).  All scenes share the context's max_shape; threads per tile may
 * differ per scene.  Host pointers.  Replaces the context's common buffers. */
int gudni_batch_upload(gudni_ctx* ctx,
                       const void* geometry, size_t geometry_bytes,
                       const float* substances, size_t n_substances,
                       const uint8_t* pictures, size_t picture_bytes,
                       const gudni_picture_use* picture_uses, size_t n_picture_uses,
                       const gudni_radial* radials, size_t n_radials,
                       const gudni_shape* shapes, size_t n_shapes,
                       const gudni_tile_info* tiles, const int32_t* tile_scene,
                       const float* tile_cost, size_t n_tiles,
                       const gudni_batch_scene* scenes, size_t n_scenes,
                       size_t out_pixels);

/* Render the uploaded batch into the context's batch output, in one persistent
 * launch (plus the full-capacity pass for overflowing columns) enqueued on `stream`.
 * With use_graph != 0 the launch sequence is captured into a CUDA graph on first use
 * and replayed afterwards. */
int gudni_batch_render(gudni_ctx* ctx, int use_graph, void* stream);

/* Render only tiles [first_tile, first_tile + n_tiles) of the uploaded batch, in
 * input order, as an ordinary launch pair: the plain one-launch-per-scene path over
 * the same resident piles, for comparison with gudni_batch_render. */
int gudni_batch_render_tiles(gudni_ctx* ctx, size_t first_tile, size_t n_tiles, void* stream);

/* Device address of the batch output (out_pixels BGRA words), and a blocking copy
 * of it to host memory. */
const uint32_t* gudni_batch_output(const gudni_ctx* ctx);
int gudni_batch_download(gudni_ctx* ctx, uint32_t* out);

/* Work counters of the next launches, for measurement: when enabled, kernels add
 * [0] sections scanned, [1] picture texels read, [2] thresholds generated,
 * [3] largest shape-bit count of a column.  gudni_read_counters returns and clears
 * them.  Counting costs a few atomics per column; it is off by default. */
int gudni_enable_counters(gudni_ctx* ctx, int enable);
int gudni_read_counters(gudni_ctx* ctx, int64_t out[4]);

/* Source of the stochastic area jitter (read only when the spec's stochastic_factor
 * is not 0).  GUDNI_RANDOM_FIELD (default) is the reference's: the uploaded random
 * field, walked one step per section from a start the column's position picks
 * (initRandomField / getRandom, Kernels.cl:1597-1613).  GUDNI_RANDOM_COUNTER takes
 * the jitter of pixel (x, y) for the section with ordinal k in its column's scan from
 * a counter-based hash of (seed, x, y, k) instead: no table, no period of 4096
 * sections, no sharing of values between neighbouring columns; a new seed per frame
 * gives independent jitter per frame.  No reference
 * counterpart.  Takes effect from the next launch. */
/* Where the uploads (gudni_upload_common, gudni_upload_frame, gudni_batch_upload)
 * build the strand table the raster kernels read (per strand its offset, size, x
 * extent and y range, and per 16-byte unit of the pile the strand starting there):
 * 0 (default) on the host, by one walk of the caller's pile, then uploaded; 1 on the
 * device from the uploaded pile, by data-parallel passes (the walk's chain found by
 * pointer doubling) -- the same table, no host walk and no table upload.  Takes effect
 * from the next upload. */
int gudni_set_device_strand_table(gudni_ctx* ctx, int enable);

#define GUDNI_RANDOM_FIELD   0
#define GUDNI_RANDOM_COUNTER 1
int gudni_set_random_source(gudni_ctx* ctx, int source, uint64_t seed);

/* Warp-cooperative dense columns for the next launches of this context: a column
 * whose sorted queue holds at least `min_thresholds` thresholds is scanned by all 32
 * lanes of its warp together (sections dealt to the lanes, pixel sums taken in section
 * order), instead of by its own lane.  The output is the same bit for bit; the choice
 * is one of speed.  0 (the default) keeps every column on its own lane.  No
 * counterpart in the reference. */
int gudni_set_dense_columns(gudni_ctx* ctx, int32_t min_thresholds);

/* Warp-cooperative work units: the 32 lanes of a warp generate a unit's thresholds
 * together -- strands dealt to the lanes, their (strand, column) pairs dealt again,
 * the thresholds binned to the columns by warp ballots in the order the per-column
 * generation pushes them -- with the tile's shape records staged in shared memory by
 * a bulk copy (the colour walk reads their tags there) and the pixels written out by
 * rows from a shared tile; each column is then sorted and scanned by its own lane.
 * Replaces the per-column generation of generateThresholds (Kernels.cl:2030-2082,
 * buildThresholdArray K:1540-1595); the output is the same bit for bit.  Units of
 * tiles with more than 64 shapes or more shapes than max_shape run the per-column
 * generation.  mode 1: every launch uses them; 0 (the default): none does; -1: a
 * launch uses them when it has at most two work units per warp the cooperative
 * kernel keeps resident (few, long units: the kernel is bound by its longest units,
 * which the shared generation shortens), and the per-column kernel otherwise (many
 * units: throughput, where the per-column kernel's smaller register footprint keeps
 * more warps in flight).  On GB300 the cooperative kernel renders the 1920x1080 page
 * in 12.3 ms against 13.5 ms, and the 3840x2160 page in 27.1 ms against 23.3 ms; tiles
 * it does not take (more than 64 shapes) run slower inside it than in the per-column
 * kernel.  Not used by the warp-cooperative dense scan
 * (gudni_set_dense_columns), by the counter-based jitter, or by
 * gudni_raster_job_noalloc. */
int gudni_set_cooperative_units(gudni_ctx* ctx, int mode);

/* ------------------------------------------------------------------ adjoint */

/* Gradients of the per-pixel L2 loss L = sum_p sum_{c in RGB} (I_c(p) - T_c(p))^2,
 * where I(p) is the pixel colour before the byte conversion (the reference's
 * accumulated colour / area, Kernels.cl:2017), with respect to every float of the
 * geometry pile and every solid substance colour.  No counterpart in the reference.
 *
 * Frame form, device pointers, enqueued on `stream`: the frame's shape and tile piles
 * as for gudni_raster_tiles_device; `target` and `image` are bitmap_w*bitmap_h float4
 * (image receives I rgb and the pixel's section-area sum in .w); `grad_geometry`
 * (geometry_bytes/4 floats) and `grad_substances` (4 floats per substance) are ADDED
 * to.  Forward and backward run in one launch, one work unit (a tile's 32 columns) at
 * a time, and no threshold outlives its work unit: by default each column's
 * thresholds are generated once, with their sources in the pile, the forward scan
 * runs on a copy of the sorted queue and the gradient scan on the queue itself; with
 * gudni_set_adjoint_regenerate(ctx, 1) the forward generates its own and the
 * backward generates them again.  The image is the same either way.  A column that
 * needs more than the adjoint's working capacity (min(max_thresholds, 1024), or
 * GUDNI_ADJOINT_CAPACITY) raises GUDNI_ERR_THRESHOLD_OVERFLOW.  The stochastic area
 * jitter (STOCHASTIC_FACTOR) is off in the adjoint: the loss is defined on the
 * deterministic render. */
int gudni_adjoint_tiles_device(gudni_ctx* ctx,
                               const gudni_shape* shapes, size_t n_shapes,
                               const gudni_tile_info* tiles, const int32_t* tile_jobs, size_t n_tiles,
                               int32_t bitmap_w, int32_t bitmap_h, int32_t compute_depth,
                               const float background[4],
                               const float* target, float* image,
                               float* grad_geometry, float* grad_substances, void* stream);

/* 1: the adjoint's backward pass regenerates each column's thresholds instead of
 * scanning the forward pass's queue (0, the default).  Returns GUDNI_OK. */
int gudni_set_adjoint_regenerate(gudni_ctx* ctx, int on);

/* Batch form: every scene of the uploaded batch (gudni_batch_upload) in one
 * persistent launch; target and image hold out_pixels float4 at the scenes' output
 * offsets; gradients index the batch's concatenated piles. */
int gudni_batch_adjoint(gudni_ctx* ctx, const float* target, float* image,
                        float* grad_geometry, float* grad_substances, void* stream);

/* ------------------------------------------------- no-allocation entry point */

/* Size of the device scratch that gudni_raster_job_noalloc uses: a fixed array
 * compiled into the library, held by every GPU that loads it until the process
 * exits. */
#define GUDNI_NOALLOC_SCRATCH_BYTES (64u << 20)
/* Threshold queue capacity per column in gudni_raster_job_noalloc. */
#define GUDNI_NOALLOC_CAPACITY 512

/* Rasterize one job without allocating any device memory.  No counterpart in the
 * reference: it is for callers that cannot call cudaMalloc -- code running inside
 * another framework's memory pool or a frame-pacing loop that forbids allocation,
 * a sandboxed plugin without allocation rights, or a real-time path where an
 * allocation's implicit synchronisation is not allowed.  Every buffer is supplied
 * by the caller as a DEVICE pointer: the common piles (geometry, substances,
 * pictures, picture uses, radial gradients), the job's shape and tile piles, and
 * `out` (bitmap_w*bitmap_h BGRA words; only the job's tiles are written).  The
 * per-column threshold queues live in the library's fixed device scratch of
 * GUDNI_NOALLOC_SCRATCH_BYTES, with a queue capacity of GUDNI_NOALLOC_CAPACITY
 * thresholds per column (min with spec->max_thresholds); a column that needs more
 * returns GUDNI_ERR_THRESHOLD_OVERFLOW, and a max_shape too large for the scratch
 * returns GUDNI_ERR_BAD_INPUT.  No context is needed; the spec supplies max_shape
 * and threads per tile.  The path takes no random field: a spec with a non-zero
 * stochastic_factor is refused with GUDNI_ERR_BAD_INPUT.
 *
 * The first call on a device looks up the scratch's device address (with that device
 * current); make that first call before any stream capture.  The address is kept for
 * the life of the process: do not call this entry point again on a device after
 * cudaDeviceReset.  Every call shares the one scratch array, so calls whose launches
 * overlap on the GPU race: issue them on one stream, or serialise them.  The call
 * enqueues its work on `stream` (NULL = the legacy default stream) after whatever the
 * caller enqueued there before -- it reads none of the records from the host, so
 * records still being copied on `stream` are fine -- and then waits for `stream` to
 * read the device status.  Malformed tiles and picture uses are found by the kernel
 * and returned as GUDNI_ERR_BAD_INPUT.  Error messages are read with
 * gudni_last_error(NULL). */
int gudni_raster_job_noalloc(const gudni_spec* spec,
                             const void* geometry, size_t geometry_bytes,
                             const float* substances, size_t n_substances,
                             const uint8_t* pictures, size_t picture_bytes,
                             const gudni_picture_use* picture_uses, size_t n_picture_uses,
                             const gudni_radial* radials, size_t n_radials,
                             const gudni_shape* shapes, size_t n_shapes,
                             const gudni_tile_info* tiles, size_t n_tiles,
                             int32_t bitmap_w, int32_t bitmap_h, int32_t compute_depth,
                             int32_t job_index, const float background[4],
                             uint32_t* out, void* stream);

/* Number of kernel launches this context has issued. */
uint64_t gudni_launch_count(const gudni_ctx* ctx);

/* Wait for the context's stream and return the accumulated device status
 * (GUDNI_OK or the first error raised by a kernel since the last call). */
int gudni_sync_status(gudni_ctx* ctx);

/* Device bytes of threshold scratch the context holds right now. */
size_t gudni_scratch_bytes(const gudni_ctx* ctx);

#ifdef __cplusplus
}
#endif

#endif /* GUDNI_CUDA_H */
