/*
 * gudni_serialize.h -- host serializer: a flattened scene -> the piles the raster
 * kernels read (geometry, substances, picture usages, radial gradients, and per job
 * the shape and tile piles).
 *
 * This is the C++ counterpart of the reference's Haskell host path
 *   buildTileTree (Raster/TileTree.hs:81-109)
 *   buildOverScene / onSubstance / onShape (Raster/Serialize.hs:148-273)
 *   enclose / outlineToStrands / replaceKnobs / reorder (Raster/Enclosure.hs:62-73,
 *     Raster/Strand.hs:153-206, Raster/Deknob.hs:61-108, Raster/ReorderTable.hs:92-110)
 *   addShapeToTree (Raster/TileTree.hs:113-190)
 *   buildRasterJobs / accumulateRasterJobs (OpenCL/CallKernels.hs:244-255,
 *     Raster/Job.hs:132-178)
 * and produces the same bytes.
 *
 * The scene arrives already flattened: the ShapeTree traversal (overlap order,
 * compound add/subtract inversion, transforms) is done by the caller, so every
 * substance lists its compound leaves in traversal order with their compound type
 * and their outlines' curve pairs in final (transformed) coordinates.
 */
#ifndef GUDNI_SERIALIZE_H
#define GUDNI_SERIALIZE_H

#include <stddef.h>
#include <stdint.h>
#include "gudni_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GUDNI_SUBSTANCE_SOLID   0
#define GUDNI_SUBSTANCE_PICTURE 1
#define GUDNI_SUBSTANCE_RADIAL  2

#define GUDNI_COMPOUND_ADD      0
#define GUDNI_COMPOUND_SUBTRACT 1

typedef struct gudni_scene_desc {
    int32_t canvas_w, canvas_h;
    float background[4];

    /* substances (SRep) in traversal order, front-most first */
    int32_t n_substances;
    const int32_t* substance_kind;         /* GUDNI_SUBSTANCE_* */
    const float* substance_color;          /* [4*n] solid colour (sRGB-encoded floats) */
    const int32_t* substance_picture;      /* [n] picture index (PICTURE) */
    const float* substance_picture_xform;  /* [3*n] usage translate x, y, scale (PICTURE) */
    const gudni_radial* substance_radial;  /* [n] gradient (RADIAL) */
    const int32_t* substance_shape_start;  /* [n+1] offsets into the shape arrays */

    /* compound leaves in traversal order */
    const int32_t* shape_compound;         /* GUDNI_COMPOUND_* (after inversion) */
    const int32_t* shape_outline_start;    /* [n_shapes+1] offsets into outlines */
    const int32_t* outline_pair_start;     /* [n_outlines+1] offsets into pairs */
    const float* pairs;                    /* [4*n_pairs] onCurve.x, .y, offCurve.x, .y */

    /* pictures: size and byte offset of each picture in the caller's picture pile */
    int32_t n_pictures;
    const int32_t* picture_size;           /* [2*n_pictures] */
    const int32_t* picture_offset;         /* [n_pictures] */
} gudni_scene_desc;

typedef struct gudni_frame gudni_frame;

/* Serialize a scene with the given spec.  Returns NULL on bad input (message in
 * gudni_serialize_error()). */
gudni_frame* gudni_serialize(const gudni_scene_desc* scene, const gudni_spec* spec);
const char* gudni_serialize_error(void);

/* The same frame, byte for byte and with the same point provenance, computed by the
 * serializer's data-parallel passes (the ones gudni_serialize_device runs as kernels)
 * on `threads` host threads (0: all available).  gudni_serialize is the sequential
 * restatement of the reference's walk; this is its fast form. */
gudni_frame* gudni_serialize_parallel(const gudni_scene_desc* scene, const gudni_spec* spec, int threads);
void gudni_frame_free(gudni_frame* frame);

size_t gudni_frame_geometry_bytes(const gudni_frame* f);
const uint8_t* gudni_frame_geometry(const gudni_frame* f);
size_t gudni_frame_n_substances(const gudni_frame* f);
const float* gudni_frame_substances(const gudni_frame* f);
size_t gudni_frame_n_picture_uses(const gudni_frame* f);
const gudni_picture_use* gudni_frame_picture_uses(const gudni_frame* f);
size_t gudni_frame_n_radials(const gudni_frame* f);
const gudni_radial* gudni_frame_radials(const gudni_frame* f);

/* Jobs in the order the reference hands them to queueRasterJobs: job index 0 is
 * the last job built (CallKernels.hs:255). */
size_t gudni_frame_n_jobs(const gudni_frame* f);
size_t gudni_frame_job_n_shapes(const gudni_frame* f, size_t job);
const gudni_shape* gudni_frame_job_shapes(const gudni_frame* f, size_t job);
size_t gudni_frame_job_n_tiles(const gudni_frame* f, size_t job);
const gudni_tile_info* gudni_frame_job_tiles(const gudni_frame* f, size_t job);
int32_t gudni_frame_job_columns(const gudni_frame* f, size_t job);

/* Provenance of every point in the geometry pile, in pile order: the float index of
 * its x in the pile, and its value as a fixed combination of at most three scene
 * points (index 2*pair for a pair's on-curve point, 2*pair+1 for its off-curve point,
 * -1 unused) with the given weights -- knob splits (Raster/Deknob.hs:61-108) create
 * points that are such combinations.  Used to carry geometry gradients back to the
 * scene's control points. */
size_t gudni_frame_n_points(const gudni_frame* f);
const uint32_t* gudni_frame_point_offsets(const gudni_frame* f);  /* n_points */
const int32_t* gudni_frame_point_sources(const gudni_frame* f);   /* 3 * n_points */
const float* gudni_frame_point_weights(const gudni_frame* f);     /* 3 * n_points */

/* Counters of the serialized frame: [0] shapes kept, [1] shapes excluded,
 * [2] strands, [3] leaf tiles, [4] tile splits, [5] max shapes in a tile,
 * [6] max strands in a tile, [7] total tile-shape references. */
void gudni_frame_stats(const gudni_frame* f, int64_t out[8]);

#ifdef __cplusplus
}
#endif

#endif /* GUDNI_SERIALIZE_H */
