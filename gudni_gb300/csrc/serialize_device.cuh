// The serializer on the device: a flattened scene -> the piles the raster kernels read
// (geometry pile with its strand table, and the frame's shape and tile piles with the
// job of every tile), computed by data-parallel passes instead of the host walk.
//
// The output is byte for byte the host serializer's (serialize.cpp, which restates
// Raster/Strand.hs:153-206, Deknob.hs:61-108, ReorderTable.hs:92-110,
// TileTree.hs:81-204, Job.hs:132-178 and CallKernels.hs:244-255); only the order of
// the work differs:
//
//  * strands: one work item per outline.  A counting pass gives every outline its
//    byte and strand count, exclusive scans give it its place in the pile, and a
//    writing pass emits its strands there with their strand-table rows.
//  * tile tree: the reference inserts shapes one at a time and splits a leaf the first
//    time an insertion finds it full (checkTileSpace, TileTree.hs:167-172).  A leaf
//    receives, in insertion order, exactly the shapes whose boxes pass the cut tests
//    on its path, whenever it was created (a split re-inserts the old contents in
//    order), and its counts only grow, so it splits if and only if that whole list
//    holds at least MAXSHAPE shapes or at least max_strands_per_tile strands and the
//    leaf is wider (HLeaf) or taller (VLeaf) than 8 pixels.  The tree is therefore
//    built top down, one level of splits per pass: the base tiles' lists first, then
//    each splitting tile's two children filtered from its list in order.
//  * jobs: the leaves in the traversal order of traverseTileTree, cut into jobs of
//    max_tiles_per_call tiles, the last job built first (CallKernels.hs:255), each
//    tile's shapes newest first; emitted as the concatenated layout of
//    gudni_raster_tiles_device (one shape pile, tile slices into it, a job per tile).
//
// Every pass is a functor over an index range, run by an executor: CUDA kernels in the
// library (capi.cu), plain loops in the CPU tests, so the arithmetic and indexing
// checked on the CPU are the ones the GPU runs.
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "gudni_cuda.h"
#include "gudni_serialize.h"

#if defined(__CUDACC__)
#define GUDNI_SHD __host__ __device__
#else
#define GUDNI_SHD
#endif

namespace gudni {
namespace ser {

// Magnitude beyond which a coordinate disables the kernels' y culling of its strand
// (the strand table's y range becomes (-inf, inf)); the host strand table
// (strand_table.h) uses the same bound.
constexpr float kStrandCullExtent = 2097152.0f;  // 2^21

constexpr int kMaxCurves = 16;                  // curves per strand (Strand.hs:178, mAXsECTIONsIZE/2)
constexpr int kMaxPoints = 2 * kMaxCurves + 1;  // points of the largest strand
constexpr int kRows = kMaxCurves + 1;           // reorder rows, by curve count
constexpr int kMinTileSide = 8;                 // mINtILEsIZE (TileTree.hs:170)
constexpr int kMaxKnobSteps = 64;               // the knob bisection ends in <= 15 steps
constexpr int kMaxLevels = 64;                  // split passes (each halves a side >= 16)
constexpr uint32_t kNoStrand = 0xFFFFFFFFu;     // strand map: no strand starts here

struct P2 {
  float x, y;
};
struct Bez {  // start, control, end (Figure/Bezier.hs Bez)
  P2 a, c, b;
};
struct Box {
  float left, top, right, bottom;
};

// Provenance of a serialized point: a fixed combination of at most three points of
// the scene (2 * pair for a pair's on-curve point, 2 * pair + 1 for its control; -1
// unused), used to carry gradients on the geometry pile back to the scene.
struct Prov {
  int32_t src[3];
  float w[3];
};
struct BezProv {
  Prov a, c, b;
};

// A shape kept after the canvas test, with what the tile tree needs.
struct KeptShape {
  uint64_t tag;
  uint32_t geo_start;    // 16-byte units
  uint32_t num_strands;
  Box box;
};

// A tile of the tree under construction.  kind: 0 = VLeaf (splits across y),
// 1 = HLeaf (splits across x); open: may still split.
struct Node {
  int32_t left, top, right, bottom;
  int16_t hdepth, vdepth;
  uint8_t kind, open;
  uint8_t pad[2];
  uint64_t list;     // first entry of its shape list in the pool (kept-shape indices)
  uint64_t count;    // shapes in the list
  uint64_t strands;  // their strands
};

// ------------------------------------------------------------ knobs (Deknob.hs)
GUDNI_SHD inline P2 between(float t, P2 v0, P2 v1) {  // Deknob.hs:40-41
  const float u = 1.0f - t;
  return P2{v0.x * u + v1.x * t, v0.y * u + v1.y * t};
}

// findSplit (Deknob.hs:61-79): halve the parameter interval toward the half that still
// bulges in the knob's direction; the point there splits the curve.
GUDNI_SHD inline float findSplit(bool left, const Bez& z, P2& mid0, P2& on, P2& mid1) {
  float lo = 0.0f, hi = 1.0f, t = 0.5f;
  for (int step = 0; step < kMaxKnobSteps; ++step) {
    mid0 = between(t, z.a, z.c);
    mid1 = between(t, z.c, z.b);
    on = between(t, mid0, mid1);
    if (hi - lo <= 0.0001f) return t;
    if (left ? (mid1.x < on.x) : (mid1.x > on.x)) {
      const float next = t + ((hi - t) / 2.0f);
      lo = t;
      t = next;
    } else if (left ? (mid0.x < on.x) : (mid0.x > on.x)) {
      const float next = lo + ((t - lo) / 2.0f);
      hi = t;
      t = next;
    } else {
      return t;
    }
  }
  return t;
}

// fixKnob (Deknob.hs:85-100): a curve whose control lies left (right) of both ends is
// split in two; returns the number of curves written to out, with their points'
// provenance (the split points are the de Casteljau combinations at the split t).
GUDNI_SHD inline int fixKnob(const Bez& z, const BezProv& zp, Bez out[2], BezProv outp[2]) {
  const bool left = z.c.x < z.a.x && z.c.x < z.b.x;
  const bool right = !left && z.c.x > z.a.x && z.c.x > z.b.x;
  if (!left && !right) {
    out[0] = z;
    outp[0] = zp;
    return 1;
  }
  P2 mid0, on, mid1;
  const float t = findSplit(left, z, mid0, on, mid1);
  out[0] = Bez{z.a, mid0, on};
  out[1] = Bez{on, mid1, z.b};
  const int32_t ia = zp.a.src[0], ic = zp.c.src[0], ib = zp.b.src[0];
  const float u = 1.0f - t;
  const Prov pm0{{ia, ic, -1}, {u, t, 0.0f}};
  const Prov pm1{{ic, ib, -1}, {u, t, 0.0f}};
  const Prov pon{{ia, ic, ib}, {u * u, 2.0f * t * u, t * t}};
  outp[0] = BezProv{zp.a, pm0, pon};
  outp[1] = BezProv{pon, pm1, zp.b};
  return 2;
}

// Consecutive curves share a strand when both run the same horizontal way
// (Strand.hs:77-81).
GUDNI_SHD inline int runX(const Bez& z) { return z.a.x < z.b.x ? -1 : (z.a.x > z.b.x ? 1 : 0); }
GUDNI_SHD inline bool connectable(const Bez& p, const Bez& q) {
  const int h = runX(p);
  return h != 0 && h == runX(q);
}

// The de-knobbed curves of one closed outline in order, produced on the fly: pair i
// (on-curve point, control) runs to the on-curve point of pair i + 1 (the last back to
// the first), and each such curve yields one or two curves.
GUDNI_SHD inline Prov prov1(int32_t id) { return Prov{{id, -1, -1}, {1.0f, 0.0f, 0.0f}}; }

struct CurveCursor {
  const float* pairs;
  int32_t pair0;  // scene index of the outline's first pair
  int n, i, half, parts;
  Bez part[2];
  BezProv partp[2];
  GUDNI_SHD void start(const float* p, int count, int32_t first_pair) {
    pairs = p;
    pair0 = first_pair;
    n = count;
    i = 0;
    half = 0;
    load();
  }
  GUDNI_SHD void load() {
    if (i >= n) return;
    const int j = i + 1 < n ? i + 1 : 0;
    const Bez z{P2{pairs[4 * i], pairs[4 * i + 1]}, P2{pairs[4 * i + 2], pairs[4 * i + 3]},
                P2{pairs[4 * j], pairs[4 * j + 1]}};
    const BezProv zp{prov1(2 * (pair0 + i)), prov1(2 * (pair0 + i) + 1), prov1(2 * (pair0 + j))};
    parts = fixKnob(z, zp, part, partp);
  }
  GUDNI_SHD bool done() const { return i >= n; }
  GUDNI_SHD const Bez& get() const { return part[half]; }
  GUDNI_SHD const BezProv& getProv() const { return partp[half]; }
  GUDNI_SHD void next() {
    if (++half >= parts) {
      half = 0;
      ++i;
      load();
    }
  }
};

// ------------------------------------------------------------ reorder rows
// The order in which a strand of k curves (2k + 1 points) stores its points
// (ReorderTable.hs:44-110): the right end, the left end and its control, then the
// remaining point/control pairs as a complete binary search tree laid out breadth
// first.  Computed on the host into rows[k][0 .. 2k].
inline int treePartition(int n) {  // size of the left subtree of n sorted keys
  int p = 1;
  while (p <= n / 2) p *= 2;
  return (p / 2) - 1 <= n - p ? p - 1 : n - p / 2;
}

inline void buildReorderRows(int rows[kRows][kMaxPoints]) {
  for (int k = 0; k < kRows; ++k)
    for (int i = 0; i < kMaxPoints; ++i) rows[k][i] = -1;
  for (int k = 1; k < kRows; ++k) {
    const int size = 2 * k + 1;
    int* row = rows[k];
    int m = 0;
    row[m++] = size - 1;
    row[m++] = 0;
    row[m++] = 1;
    // the (size - 3) / 2 remaining pairs as a search tree over their pair indices,
    // visited level by level, left to right
    int lo[kMaxCurves], hi[kMaxCurves];
    int head = 0, tail = 0;
    const int pairs = (size - 3) / 2;
    if (pairs > 0) {
      lo[tail] = 0;
      hi[tail] = pairs;
      ++tail;
    }
    while (head < tail) {
      const int a = lo[head], b = hi[head];
      ++head;
      const int root = a + treePartition(b - a);
      row[m++] = 2 * root + 2;
      row[m++] = 2 * root + 3;
      if (root > a) {
        lo[tail] = a;
        hi[tail] = root;
        ++tail;
      }
      if (b > root + 1) {
        lo[tail] = root + 1;
        hi[tail] = b;
        ++tail;
      }
    }
  }
}

// ------------------------------------------------------------ strands of an outline
// Bytes and strands an outline serializes to (outlineToStrands, Strand.hs:153-178):
// runs of connectable curves, each cut into strands of at most 16 curves; a strand of
// k curves takes an 8-byte header and 2k + 1 points of 8 bytes.
GUDNI_SHD inline void outlineSize(const float* pairs, int n_pairs, uint64_t& bytes, uint64_t& strands) {
  bytes = 0;
  strands = 0;
  if (n_pairs < 2) return;
  CurveCursor c;
  c.start(pairs, n_pairs, 0);
  Bez prev = c.get();
  c.next();
  uint64_t run = 1, curves = 1, chunks = 0;
  while (!c.done()) {
    const Bez z = c.get();
    if (!connectable(prev, z)) {
      chunks += (run + kMaxCurves - 1) / kMaxCurves;
      run = 0;
    }
    ++run;
    ++curves;
    prev = z;
    c.next();
  }
  chunks += (run + kMaxCurves - 1) / kMaxCurves;
  bytes = 16 * chunks + 16 * curves;
  strands = chunks;
}

// Where an outline's strands go: the geometry pile, the strand table (offset in 8-byte
// units, size, left x and right x bits), the y range of each strand's points and the
// strand starting at each 16-byte unit (strand_table.h builds the same by walking a
// finished pile).
struct StrandOut {
  uint8_t* geo;
  uint4* table;
  float2* ys;
  uint32_t* first;
  const int* rows;  // kRows x kMaxPoints
  // optional point provenance, in pile order: 3 sources and 3 weights per point and
  // the float index of its x in the pile (null: not wanted)
  int32_t* psrc;
  float* pw;
  uint32_t* pat;
};

GUDNI_SHD inline uint32_t floatBits(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}

// One strand: reverseIfBackwards (Strand.hs:137-143), beziersToPoints (:130-134), then
// the header and the points in reorder-row order (:190-206).
GUDNI_SHD inline void writeStrand(const Bez* chunk, const BezProv* chunkp, int m, uint64_t off, uint32_t index,
                                  const StrandOut& o) {
  P2 pts[kMaxPoints];
  const bool backwards = chunk[0].a.x > chunk[m - 1].b.x;
  for (int k = 0; k < m; ++k) {
    const Bez& z = backwards ? chunk[m - 1 - k] : chunk[k];
    pts[2 * k] = backwards ? z.b : z.a;
    pts[2 * k + 1] = z.c;
  }
  pts[2 * m] = backwards ? chunk[0].a : chunk[m - 1].b;
  if (o.psrc) {  // the points' provenance follows them through the reversal
    Prov pp[kMaxPoints];
    for (int k = 0; k < m; ++k) {
      const BezProv& z = backwards ? chunkp[m - 1 - k] : chunkp[k];
      pp[2 * k] = backwards ? z.b : z.a;
      pp[2 * k + 1] = z.c;
    }
    pp[2 * m] = backwards ? chunkp[0].a : chunkp[m - 1].b;
    const int* prow = o.rows + m * kMaxPoints;
    const uint64_t point0 = (off - 8 * (uint64_t)index) / 8;  // points before this strand
    for (int i = 0; i < 2 * m + 1; ++i) {
      const Prov& q = pp[prow[i]];
      const uint64_t k = point0 + (uint64_t)i;
      for (int j = 0; j < 3; ++j) {
        o.psrc[3 * k + j] = q.src[j];
        o.pw[3 * k + j] = q.w[j];
      }
      o.pat[k] = (uint32_t)((off + 8 + 8 * (uint64_t)i) / 4);
    }
  }
  const int len = 2 * m + 1;
  const uint32_t size = (uint32_t)(1 + len);  // in 8-byte units, header included
  uint32_t* hdr = reinterpret_cast<uint32_t*>(o.geo + off);
  hdr[0] = size;
  hdr[1] = 0u;
  const int* row = o.rows + m * kMaxPoints;
  float lo = INFINITY, hi = -INFINITY;
  bool bad = false;  // a coordinate beyond kStrandCullExtent: the range that disables culling
  float* p = reinterpret_cast<float*>(o.geo + off + 8);
  for (int i = 0; i < len; ++i) {
    const P2 q = pts[row[i]];
    p[2 * i] = q.x;
    p[2 * i + 1] = q.y;
    if (!(fabsf(q.x) <= kStrandCullExtent) || !(fabsf(q.y) <= kStrandCullExtent)) bad = true;
    lo = q.y < lo ? q.y : lo;
    hi = hi < q.y ? q.y : hi;
  }
  o.table[index] = make_uint4((uint32_t)(off / 8), size, floatBits(p[2]), floatBits(p[0]));
  o.ys[index] = bad ? make_float2(-INFINITY, INFINITY) : make_float2(lo, hi);
  o.first[off / 16] = index;
}

// All strands of one outline from byte `off` and strand index `index` on: the run
// that ends the outline first, then the others in order (the fold's final
// accumulator heads the list, Strand.hs:98-102), each cut every 16 curves.
GUDNI_SHD inline void outlineWrite(const float* pairs, int n_pairs, int32_t pair0, uint64_t off, uint32_t index,
                                   const StrandOut& o) {
  if (n_pairs < 2) return;
  CurveCursor c;
  c.start(pairs, n_pairs, pair0);
  CurveCursor last = c;  // start of the final run
  uint64_t last_at = 0, curves = 1;
  Bez prev = c.get();
  c.next();
  while (!c.done()) {
    const Bez z = c.get();
    if (!connectable(prev, z)) {
      last = c;
      last_at = curves;
    }
    prev = z;
    ++curves;
    c.next();
  }
  Bez chunk[kMaxCurves];
  BezProv chunkp[kMaxCurves];
  for (int pass = 0; pass < 2; ++pass) {
    CurveCursor cur = last;
    uint64_t todo = curves - last_at;
    if (pass == 1) {
      cur.start(pairs, n_pairs, pair0);
      todo = last_at;
    }
    int m = 0;
    for (uint64_t k = 0; k < todo; ++k) {
      const Bez z = cur.get();
      const BezProv zp = cur.getProv();
      cur.next();
      if (m > 0 && (m == kMaxCurves || !connectable(chunk[m - 1], z))) {
        writeStrand(chunk, chunkp, m, off, index, o);
        off += 8 + 8 * (uint64_t)(2 * m + 1);
        ++index;
        m = 0;
      }
      chunk[m] = z;
      if (o.psrc) chunkp[m] = zp;
      ++m;
    }
    if (m > 0) {
      writeStrand(chunk, chunkp, m, off, index, o);
      off += 8 + 8 * (uint64_t)(2 * m + 1);
      ++index;
    }
  }
}

// ------------------------------------------------------------ tile tree helpers
GUDNI_SHD inline int adjustedLog(int x) {  // TileTree.hs:74-75: smallest d, 2^d >= x
  int d = 0;
  while (d < 31 && (1LL << d) < (long long)x) ++d;
  return x < 1 ? 0 : d;
}

// A base tile of the tree (buildTileTree, TileTree.hs:95-109) is reached by a shape
// when its box passes every cut on the way: left of a cut c when box.left < c, right
// of it when box.right > c (above / below alike).  The tile's own edges are the
// nearest such cuts, so the edges inside the canvas square decide.
GUDNI_SHD inline bool reachesRect(const Box& b, int l, int t, int r, int bo, int side) {
  return (r == side || b.left < (float)r) && (l == 0 || b.right > (float)l) && (bo == side || b.top < (float)bo) &&
         (t == 0 || b.bottom > (float)t);
}

// Base tile number `r` in traversal order: the tree cuts across y, then across x, at
// every level from the canvas square down to the tile size, visiting top before
// bottom and left before right, so r interleaves the bits of the tile's row (higher)
// and column (lower).
GUDNI_SHD inline void baseTileOf(uint64_t r, int levels, int& col, int& row) {
  col = 0;
  row = 0;
  for (int k = 0; k < levels; ++k) {
    col |= (int)((r >> (2 * k)) & 1u) << k;
    row |= (int)((r >> (2 * k + 1)) & 1u) << k;
  }
}

// The split rule of checkTileSpace over a whole list (see the file comment).
GUDNI_SHD inline bool splits(const Node& n, int max_shape, int64_t max_strands) {
  if (!n.open || n.count == 0) return false;
  const int side = n.kind == 0 ? n.bottom - n.top : n.right - n.left;
  if (side <= kMinTileSide) return false;
  return n.count >= (uint64_t)(max_shape < 0 ? 0 : max_shape) || (int64_t)n.strands >= max_strands;
}

// The cut of a splitting node and the test its children apply (insertShapeV /
// insertShapeH, TileTree.hs:117-151; vSplit / hSplit, :175-190).
GUDNI_SHD inline int cutOf(const Node& n) {
  return n.kind == 0 ? n.top + (n.bottom - n.top) / 2 : n.left + (n.right - n.left) / 2;
}
GUDNI_SHD inline bool inChild(const Node& n, int cut, int child, const Box& b) {
  const float c = (float)cut;
  if (n.kind == 0) return child == 0 ? b.top < c : b.bottom > c;
  return child == 0 ? b.left < c : b.right > c;
}
GUDNI_SHD inline Node childOf(const Node& n, int cut, int child) {
  Node k = n;
  k.open = 1;
  if (n.kind == 0) {  // VLeaf -> VTree over two HLeafs
    k.kind = 1;
    k.vdepth = (int16_t)(n.vdepth - 1);
    if (child == 0) k.bottom = cut; else k.top = cut;
  } else {            // HLeaf -> HTree over two VLeafs
    k.kind = 0;
    k.hdepth = (int16_t)(n.hdepth - 1);
    if (child == 0) k.right = cut; else k.left = cut;
  }
  return k;
}

// ------------------------------------------------------------ passes
// The flattened scene (gudni_scene_desc) on the executing side; shape, outline and
// pair indices are the scene's own (absolute), the passes cover [shape0, shape1) and
// [outline0, outline1).
struct Scene {
  int32_t canvas_w, canvas_h;
  int32_t n_substances;
  const int32_t* substance_shape_start;
  const uint64_t* substance_tag;   // per substance: type bits | id (ShapeInfo.hs:89-99)
  const int32_t* shape_compound;
  const int32_t* shape_outline_start;
  const int32_t* outline_pair_start;
  const float* pairs;
  int32_t shape0, shape1, outline0, outline1;
};

struct Limits {
  int32_t max_tile_size, threads_per_tile, max_tiles_per_call, max_shape;
  int64_t max_strands;
};

// per substance: the substance of each of its shapes
struct ShapeSubstancePass {
  Scene s;
  int32_t* shape_sub;
  GUDNI_SHD void operator()(uint64_t sub) const {
    for (int32_t sh = s.substance_shape_start[sub]; sh < s.substance_shape_start[sub + 1]; ++sh)
      shape_sub[sh - s.shape0] = (int32_t)sub;
  }
};

// per shape: its box over every pair (boxOf includes the control point), the canvas
// test (excludeBox, Serialize.hs:97-104) and the shape of each of its outlines
struct ShapeBoxPass {
  Scene s;
  Box* box;
  uint64_t* keep;
  int32_t* outline_shape;
  GUDNI_SHD void operator()(uint64_t i) const {
    const int32_t sh = s.shape0 + (int32_t)i;
    Box b{INFINITY, INFINITY, -INFINITY, -INFINITY};
    for (int32_t o = s.shape_outline_start[sh]; o < s.shape_outline_start[sh + 1]; ++o) {
      outline_shape[o - s.outline0] = sh;
      for (int32_t p = s.outline_pair_start[o]; p < s.outline_pair_start[o + 1]; ++p) {
        const float* q = s.pairs + 4 * (int64_t)p;
        for (int k = 0; k < 2; ++k) {
          const float x = q[2 * k], y = q[2 * k + 1];
          b.left = b.left <= x ? b.left : x;
          b.top = b.top <= y ? b.top : y;
          b.right = b.right <= x ? x : b.right;
          b.bottom = b.bottom <= y ? y : b.bottom;
        }
      }
    }
    box[i] = b;
    const bool out = b.left >= (float)s.canvas_w || b.top >= (float)s.canvas_h || b.right <= 0.0f || b.bottom <= 0.0f;
    keep[i] = out ? 0 : 1;
  }
};

// per outline: its bytes and strands (none for an excluded shape's outlines)
struct OutlineSizePass {
  Scene s;
  const int32_t* outline_shape;
  const uint64_t* keep;
  uint64_t* bytes;
  uint64_t* strands;
  GUDNI_SHD void operator()(uint64_t i) const {
    const int32_t o = s.outline0 + (int32_t)i;
    uint64_t b = 0, n = 0;
    if (keep[outline_shape[i] - s.shape0]) {
      const int32_t p0 = s.outline_pair_start[o];
      outlineSize(s.pairs + 4 * (int64_t)p0, s.outline_pair_start[o + 1] - p0, b, n);
    }
    bytes[i] = b;
    strands[i] = n;
  }
};

struct FillPass {
  uint32_t* out;
  uint32_t value;
  GUDNI_SHD void operator()(uint64_t i) const { out[i] = value; }
};

struct OutlineWritePass {
  Scene s;
  const int32_t* outline_shape;
  const uint64_t* keep;
  const uint64_t* byte_at;    // exclusive scan of the outlines' bytes
  const uint64_t* strand_at;  // exclusive scan of their strands
  StrandOut out;
  GUDNI_SHD void operator()(uint64_t i) const {
    if (!keep[outline_shape[i] - s.shape0]) return;
    const int32_t o = s.outline0 + (int32_t)i;
    const int32_t p0 = s.outline_pair_start[o];
    outlineWrite(s.pairs + 4 * (int64_t)p0, s.outline_pair_start[o + 1] - p0, p0, byte_at[i], (uint32_t)strand_at[i],
                 out);
  }
};

// per shape: the kept shapes in order, with tag, geometry start and strand count
// (onShape, Serialize.hs:148-177; the tag by makeTag, ShapeInfo.hs:89-99)
struct KeptPass {
  Scene s;
  const int32_t* shape_sub;
  const Box* box;
  const uint64_t* keep;
  const uint64_t* kept_at;
  const uint64_t* byte_at;
  const uint64_t* strand_at;
  KeptShape* kept;
  GUDNI_SHD void operator()(uint64_t i) const {
    if (!keep[i]) return;
    const int32_t sh = s.shape0 + (int32_t)i;
    const int32_t o0 = s.shape_outline_start[sh] - s.outline0, o1 = s.shape_outline_start[sh + 1] - s.outline0;
    KeptShape k;
    const uint64_t comb = s.shape_compound[sh] == GUDNI_COMPOUND_SUBTRACT ? GUDNI_TAG_SUBTRACT : GUDNI_TAG_ADD;
    k.tag = s.substance_tag[shape_sub[i]] | comb;
    k.geo_start = (uint32_t)(byte_at[o0] / 16);
    k.num_strands = (uint32_t)(strand_at[o1] - strand_at[o0]);
    k.box = box[i];
    kept[kept_at[i]] = k;
  }
};

// The base tiles a box reaches along one axis of the grid (n tiles of `side` pixels):
// tile i is reached when (i == n - 1 || lo_edge < (i + 1) * side) and
// (i == 0 || hi_edge > i * side) -- reachesRect's tests, each monotone in i -- so the
// reached tiles are [lo, hi] (none when lo > hi).  Binary searches with the same
// float comparisons.
GUDNI_SHD inline void reachRange(float lo_edge, float hi_edge, int n, int side, int& lo, int& hi) {
  int a = 0, b = n - 1;  // last i with (i == 0 || hi_edge > i * side)
  while (a < b) {
    const int m = a + (b - a + 1) / 2;
    if (hi_edge > (float)(m * side)) a = m; else b = m - 1;
  }
  hi = a;
  a = 0;
  b = n - 1;  // first i with (i == n - 1 || lo_edge < (i + 1) * side)
  while (a < b) {
    const int m = a + (b - a) / 2;
    if (lo_edge < (float)((m + 1) * side)) b = m; else a = m + 1;
  }
  lo = a;
}

// The traversal number of the base tile in column `col`, row `row` (baseTileOf's
// inverse).
GUDNI_SHD inline uint32_t baseTileNumber(int col, int row, int levels) {
  uint32_t r = 0;
  for (int k = 0; k < levels; ++k)
    r |= ((((uint32_t)col >> k) & 1u) << (2 * k)) | ((((uint32_t)row >> k) & 1u) << (2 * k + 1));
  return r;
}

// per kept shape: the rectangle of base tiles its box reaches and their number
struct ReachPass {
  const KeptShape* kept;
  int n, side;  // tiles per axis, tile side in pixels
  int4* rect;   // column range (x, y), row range (z, w)
  uint64_t* count;
  GUDNI_SHD void operator()(uint64_t k) const {
    const Box& b = kept[k].box;
    int c0, c1, r0, r1;
    reachRange(b.left, b.right, n, side, c0, c1);
    reachRange(b.top, b.bottom, n, side, r0, r1);
    rect[k] = make_int4(c0, c1, r0, r1);
    count[k] = (c0 <= c1 && r0 <= r1) ? (uint64_t)(c1 - c0 + 1) * (uint64_t)(r1 - r0 + 1) : 0;
  }
};

// per kept shape: a (base tile, shape) pair for every tile it reaches
struct PairPass {
  const int4* rect;
  const uint64_t* at;  // exclusive scan of the counts
  int levels;
  uint32_t* key;
  uint32_t* val;
  GUDNI_SHD void operator()(uint64_t k) const {
    const int4 q = rect[k];
    uint64_t j = at[k];
    for (int row = q.z; row <= q.w; ++row)
      for (int col = q.x; col <= q.y; ++col) {
        key[j] = baseTileNumber(col, row, levels);
        val[j] = (uint32_t)k;
        ++j;
      }
  }
};

// Stable LSD radix sort of the pairs by tile, kRadixBits per pass, in blocks of
// kRadixBlock pairs: each block counts its digits, a scan over (digit, block) gives
// every block its place per digit, and each block scatters its pairs in order.  The
// shapes of a tile thus keep their insertion order.
constexpr int kRadixBits = 8;
constexpr int kRadixDigits = 1 << kRadixBits;
constexpr uint64_t kRadixBlock = 1024;

struct RadixCountPass {
  const uint32_t* key;
  uint64_t n, blocks;
  int shift;
  uint64_t* hist;  // [digit * blocks + block]
  GUDNI_SHD void operator()(uint64_t blk) const {
    uint32_t c[kRadixDigits];
    for (int d = 0; d < kRadixDigits; ++d) c[d] = 0;
    const uint64_t end = (blk + 1) * kRadixBlock < n ? (blk + 1) * kRadixBlock : n;
    for (uint64_t i = blk * kRadixBlock; i < end; ++i) ++c[(key[i] >> shift) & (kRadixDigits - 1)];
    for (int d = 0; d < kRadixDigits; ++d) hist[(uint64_t)d * blocks + blk] = c[d];
  }
};

struct RadixScatterPass {
  const uint32_t* key;
  const uint32_t* val;
  uint64_t n, blocks;
  int shift;
  const uint64_t* at;  // exclusive scan of hist
  uint32_t* key_out;
  uint32_t* val_out;
  GUDNI_SHD void operator()(uint64_t blk) const {
    uint64_t next[kRadixDigits];
    for (int d = 0; d < kRadixDigits; ++d) next[d] = at[(uint64_t)d * blocks + blk];
    const uint64_t end = (blk + 1) * kRadixBlock < n ? (blk + 1) * kRadixBlock : n;
    for (uint64_t i = blk * kRadixBlock; i < end; ++i) {
      const uint64_t o = next[(key[i] >> shift) & (kRadixDigits - 1)]++;
      key_out[o] = key[i];
      val_out[o] = val[i];
    }
  }
};

struct Fill64Pass {
  uint64_t* out;
  uint64_t value;
  GUDNI_SHD void operator()(uint64_t i) const { out[i] = value; }
};

// per sorted pair: where its tile's run starts and ends
struct RunPass {
  const uint32_t* key;
  uint64_t n;
  uint64_t* first;
  uint64_t* end;
  GUDNI_SHD void operator()(uint64_t i) const {
    const uint32_t t = key[i];
    if (i == 0 || key[i - 1] != t) first[t] = i;
    if (i + 1 == n || key[i + 1] != t) end[t] = i + 1;
  }
};

// per base tile: its place in the tree and its list -- its run of the sorted pairs
struct BaseNodePass {
  const KeptShape* kept;
  const uint32_t* list;  // the sorted pairs' shapes (the start of the list pool)
  const uint64_t* first;
  const uint64_t* end;
  int levels, tile_side, depth;
  Node* nodes;
  GUDNI_SHD void operator()(uint64_t r) const {
    int col, row;
    baseTileOf(r, levels, col, row);
    Node n;
    n.left = col * tile_side;
    n.top = row * tile_side;
    n.right = n.left + tile_side;
    n.bottom = n.top + tile_side;
    n.hdepth = (int16_t)depth;
    n.vdepth = (int16_t)depth;
    n.kind = 0;
    n.open = 1;
    n.pad[0] = n.pad[1] = 0;
    n.list = first[r];
    n.count = end[r] - first[r];
    uint64_t strands = 0;
    for (uint64_t i = first[r]; i < end[r]; ++i) strands += kept[list[i]].num_strands;
    n.strands = strands;
    nodes[r] = n;
  }
};

// per node of a level: whether it splits, and its children's list sizes
struct SplitCountPass {
  const Node* nodes;
  const KeptShape* kept;
  const uint32_t* pool;
  Limits lim;
  uint64_t* out_nodes;   // nodes it becomes on the next level (1 or 2)
  uint64_t* out_list;    // list entries its children take
  uint64_t* child_size;  // 2 per node: children's counts
  uint64_t* child_strands;
  GUDNI_SHD void operator()(uint64_t i) const {
    const Node& n = nodes[i];
    child_size[2 * i] = child_size[2 * i + 1] = 0;
    child_strands[2 * i] = child_strands[2 * i + 1] = 0;
    if (!splits(n, lim.max_shape, lim.max_strands)) {
      out_nodes[i] = 1;
      out_list[i] = 0;
      return;
    }
    const int cut = cutOf(n);
    uint64_t c[2] = {0, 0}, st[2] = {0, 0};
    for (uint64_t k = 0; k < n.count; ++k) {
      const KeptShape& s = kept[pool[n.list + k]];
      for (int ch = 0; ch < 2; ++ch)
        if (inChild(n, cut, ch, s.box)) {
          ++c[ch];
          st[ch] += s.num_strands;
        }
    }
    out_nodes[i] = 2;
    out_list[i] = c[0] + c[1];
    child_size[2 * i] = c[0];
    child_size[2 * i + 1] = c[1];
    child_strands[2 * i] = st[0];
    child_strands[2 * i + 1] = st[1];
  }
};

// per node of a level: itself (closed) or its two children on the next level, the
// children's lists filtered from its own in order and appended to the pool
struct SplitEmitPass {
  const Node* nodes;
  const KeptShape* kept;
  uint32_t* pool;
  uint64_t pool_used;          // where this level's new lists start
  Limits lim;
  const uint64_t* node_at;     // exclusive scan of out_nodes
  const uint64_t* list_at;     // exclusive scan of out_list
  const uint64_t* child_size;
  const uint64_t* child_strands;
  Node* next;
  GUDNI_SHD void operator()(uint64_t i) const {
    const Node& n = nodes[i];
    const uint64_t at = node_at[i];
    if (!splits(n, lim.max_shape, lim.max_strands)) {
      Node k = n;
      k.open = 0;
      next[at] = k;
      return;
    }
    const int cut = cutOf(n);
    uint64_t w[2] = {pool_used + list_at[i], pool_used + list_at[i] + child_size[2 * i]};
    for (int ch = 0; ch < 2; ++ch) {
      Node k = childOf(n, cut, ch);
      k.list = w[ch];
      k.count = child_size[2 * i + ch];
      k.strands = child_strands[2 * i + ch];
      next[at + ch] = k;
    }
    for (uint64_t k = 0; k < n.count; ++k) {
      const uint32_t id = pool[n.list + k];
      for (int ch = 0; ch < 2; ++ch)
        if (inChild(n, cut, ch, kept[id].box)) pool[w[ch]++] = id;
    }
  }
};

// Leaf r (traversal order) in the concatenated layout: its job is built r / M; jobs
// are listed last built first, so the tiles of later jobs come first.
GUDNI_SHD inline uint64_t leafPosition(uint64_t r, uint64_t leaves, uint64_t per_job) {
  const uint64_t b = r / per_job;
  const uint64_t end = (b + 1) * per_job < leaves ? (b + 1) * per_job : leaves;
  return (leaves - end) + (r - b * per_job);
}

struct LeafCountPass {
  const Node* nodes;
  uint64_t leaves, per_job;
  uint64_t* counts;  // by position
  GUDNI_SHD void operator()(uint64_t r) const { counts[leafPosition(r, leaves, per_job)] = nodes[r].count; }
};

// per leaf: its tile record, its job and its shapes, newest first
// (accumulateRasterJobs, Job.hs:132-178)
struct LeafEmitPass {
  const Node* nodes;
  const KeptShape* kept;
  const uint32_t* pool;
  uint64_t leaves, per_job, n_jobs;
  int32_t threads_per_tile;
  const uint64_t* shape_at;  // by position: exclusive scan of the counts
  gudni_tile_info* tiles;
  int32_t* tile_jobs;
  gudni_shape* shapes;
  GUDNI_SHD void operator()(uint64_t r) const {
    const Node& n = nodes[r];
    const uint64_t pos = leafPosition(r, leaves, per_job);
    const uint64_t b = r / per_job;
    gudni_tile_info t;
    t.left = n.left;
    t.top = n.top;
    t.right = n.right;
    t.bottom = n.bottom;
    t.hdepth = n.hdepth;
    t.vdepth = n.vdepth;
    t.column_allocation = (int32_t)((r - b * per_job) * (uint64_t)threads_per_tile);
    t.shapes.start = (uint32_t)shape_at[pos];
    t.shapes.length = (uint32_t)n.count;
    tiles[pos] = t;
    tile_jobs[pos] = (int32_t)(n_jobs - 1 - b);
    for (uint64_t k = 0; k < n.count; ++k) {
      const KeptShape& s = kept[pool[n.list + n.count - 1 - k]];
      gudni_shape g;
      g.tag = s.tag;
      g.geo_start = s.geo_start;
      g.num_strands = s.num_strands;
      shapes[shape_at[pos] + k] = g;
    }
  }
};

// per leaf: the largest shape count and strand count over the leaves (out[0], out[1],
// zero beforehand); the maximum does not depend on the order
struct LeafMaxPass {
  const Node* nodes;
  unsigned long long* out;
  GUDNI_SHD void operator()(uint64_t i) const {
#if defined(__CUDA_ARCH__)
    atomicMax(&out[0], (unsigned long long)nodes[i].count);
    atomicMax(&out[1], (unsigned long long)nodes[i].strands);
#else  // host threads may run items at once
    for (int j = 0; j < 2; ++j) {
      const unsigned long long v = j == 0 ? nodes[i].count : nodes[i].strands;
      unsigned long long cur = __atomic_load_n(&out[j], __ATOMIC_RELAXED);
      while (v > cur && !__atomic_compare_exchange_n(&out[j], &cur, v, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
      }
    }
#endif
  }
};

// ------------------------------------------------------------ kernels of the executor
#if defined(__CUDACC__)
constexpr int kPassBlock = 256;
constexpr int kScanBlock = 1024;

// A pass over items [0, n): grid-stride, one item per thread at a time.
template <class Pass>
__global__ void __launch_bounds__(kPassBlock) pass_kernel(Pass pass, uint64_t n) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) pass(i);
}

// Exclusive prefix sum of n values by one block of kScanBlock threads, kScanBlock
// values per step with the running total carried from step to step; out[n] receives
// the total.
__global__ void __launch_bounds__(kScanBlock) scan_kernel(const uint64_t* in, uint64_t* out, uint64_t n) {
  __shared__ uint64_t warp_total[kScanBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t carry = 0;
  for (uint64_t base = 0; base < n; base += kScanBlock) {
    const uint64_t i = base + threadIdx.x;
    const uint64_t v = i < n ? in[i] : 0;
    uint64_t x = v;  // inclusive scan within the warp
    for (int d = 1; d < 32; d <<= 1) {
      const uint64_t y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) warp_total[warp] = x;
    __syncthreads();
    if (warp == 0) {  // inclusive scan of the warps' totals
      uint64_t w = warp_total[lane];
      for (int d = 1; d < 32; d <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, w, d);
        if (lane >= d) w += y;
      }
      warp_total[lane] = w;
    }
    __syncthreads();
    if (i < n) out[i] = carry + (warp ? warp_total[warp - 1] : 0) + (x - v);
    carry += warp_total[kScanBlock / 32 - 1];
    __syncthreads();  // warp_total is rewritten by the next step
  }
  if (threadIdx.x == 0) out[n] = carry;
}
#endif

// ------------------------------------------------------------ host side
// The scene's index arrays: non-negative and non-decreasing over the ranges the
// passes cover (the shapes the substances list, their outlines, their pairs).
// Returns nullptr, or why the scene is refused.
inline const char* checkScene(const gudni_scene_desc* s, const gudni_spec& spec, Scene& sc, int64_t& n_pairs) {
  auto rising = [](const int32_t* a, int32_t from, int32_t to) {
    if (a[from] < 0) return false;
    for (int32_t i = from; i < to; ++i)
      if (a[i + 1] < a[i]) return false;
    return true;
  };
  if (s->canvas_w <= 0 || s->canvas_h <= 0) return "canvas must be positive";
  if (spec.max_tile_size <= 0 || spec.max_tiles_per_call <= 0 || spec.threads_per_tile <= 0)
    return "spec sizes must be positive";
  if (s->n_substances < 0) return "negative substance count";
  sc = Scene{};
  sc.canvas_w = s->canvas_w;
  sc.canvas_h = s->canvas_h;
  sc.n_substances = s->n_substances;
  n_pairs = 0;
  if (s->n_substances == 0) return nullptr;
  if (!s->substance_kind || !s->substance_shape_start) return "missing substance arrays";
  if (!rising(s->substance_shape_start, 0, s->n_substances))
    return "substance shape starts must be non-negative and non-decreasing";
  sc.shape0 = s->substance_shape_start[0];
  sc.shape1 = s->substance_shape_start[s->n_substances];
  if (sc.shape1 == sc.shape0) return nullptr;
  if (!s->shape_compound || !s->shape_outline_start) return "missing shape arrays";
  if (!rising(s->shape_outline_start, sc.shape0, sc.shape1))
    return "shape outline starts must be non-negative and non-decreasing";
  sc.outline0 = s->shape_outline_start[sc.shape0];
  sc.outline1 = s->shape_outline_start[sc.shape1];
  if (sc.outline1 == sc.outline0) return nullptr;
  if (!s->outline_pair_start) return "missing outline array";
  if (!rising(s->outline_pair_start, sc.outline0, sc.outline1))
    return "outline pair starts must be non-negative and non-decreasing";
  n_pairs = s->outline_pair_start[sc.outline1];
  if (n_pairs > 0 && !s->pairs) return "missing pairs";
  return nullptr;
}

// Substance records, picture usages and gradients, one per substance in order, and
// each substance's tag without its compound bits (onSubstance, Serialize.hs:226-264;
// makeTag, ShapeInfo.hs:89-99): the host serializer's records.  Built on the host:
// one short record per substance.
inline const char* buildSubstances(const gudni_scene_desc* s, std::vector<float4>& subs,
                                   std::vector<gudni_picture_use>& uses, std::vector<gudni_radial>& rads,
                                   std::vector<uint64_t>& tags) {
  for (int sub = 0; sub < s->n_substances; ++sub) {
    const int kind = s->substance_kind[sub];
    float4 rec = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint64_t type;
    if (kind == GUDNI_SUBSTANCE_SOLID) {
      if (!s->substance_color) return "solid substance without colour";
      std::memcpy(&rec, s->substance_color + 4 * (size_t)sub, 16);
      type = GUDNI_TAG_SOLID;
    } else if (kind == GUDNI_SUBSTANCE_PICTURE) {
      if (!s->substance_picture || !s->substance_picture_xform || !s->picture_size || !s->picture_offset)
        return "picture substance without picture arrays";
      const int pid = s->substance_picture[sub];
      if (pid < 0 || pid >= s->n_pictures) return "picture index out of range";
      gudni_picture_use u;
      u.translate_x = s->substance_picture_xform[3 * (size_t)sub + 0];
      u.translate_y = s->substance_picture_xform[3 * (size_t)sub + 1];
      u.size_x = s->picture_size[2 * pid];
      u.size_y = s->picture_size[2 * pid + 1];
      u.mem_offset = s->picture_offset[pid];
      u.scale = s->substance_picture_xform[3 * (size_t)sub + 2];
      const uint32_t id = (uint32_t)uses.size();
      uses.push_back(u);
      std::memcpy(&rec.x, &id, 4);
      type = GUDNI_TAG_PICTURE;
    } else if (kind == GUDNI_SUBSTANCE_RADIAL) {
      if (!s->substance_radial) return "radial substance without gradient";
      const uint32_t id = (uint32_t)rads.size();
      rads.push_back(s->substance_radial[sub]);
      std::memcpy(&rec.x, &id, 4);
      type = GUDNI_TAG_RADIAL;
    } else {
      return "unknown substance kind";
    }
    subs.push_back(rec);
    tags.push_back(type | ((uint64_t)sub & GUDNI_TAG_ID_MASK));
  }
  return nullptr;
}

// Storage the passes ask their executor for.
enum Slot {
  kGeometry, kStrandTable, kStrandY, kStrandFirst, kShapes, kTiles, kTileJobs,  // results
  kShapeSub, kBox, kKeep, kKeptAt, kOutlineShape, kOutlineBytes, kByteAt, kOutlineStrands, kStrandAt,
  kKept, kNodesA, kNodesB, kPoolA, kPoolB, kOutNodes, kNodeAt, kOutList, kListAt, kChildSize,
  kChildStrands, kLeafCounts, kShapeAt, kReorder, kPointSources, kPointWeights, kPointOffsets,
  kRect, kPairCount, kPairAt, kKeysA, kKeysB, kHist, kHistAt, kTileFirst, kTileEnd, kScanSums, kScanStarts,
  kSlots
};

// ------------------------------------------------------------ long prefix sums
// Exclusive prefix sum of n values (out[n] = the total) for any n: short arrays by the
// executor's scan; long ones in three passes -- every block of kScanChunk values sums
// itself, the block sums are scanned, and every block writes its prefixes from its
// block's start -- so the work spreads over n / kScanChunk items.
constexpr uint64_t kScanChunk = 1024;
constexpr uint64_t kShortScan = 1 << 16;

struct ChunkSumPass {
  const uint64_t* in;
  uint64_t n;
  uint64_t* sums;
  GUDNI_SHD void operator()(uint64_t b) const {
    const uint64_t end = (b + 1) * kScanChunk < n ? (b + 1) * kScanChunk : n;
    uint64_t acc = 0;
    for (uint64_t i = b * kScanChunk; i < end; ++i) acc += in[i];
    sums[b] = acc;
  }
};
struct ChunkScanPass {
  const uint64_t* in;
  uint64_t n;
  const uint64_t* starts;  // exclusive scan of the chunk sums
  uint64_t* out;
  GUDNI_SHD void operator()(uint64_t b) const {
    const uint64_t end = (b + 1) * kScanChunk < n ? (b + 1) * kScanChunk : n;
    uint64_t acc = starts[b];
    for (uint64_t i = b * kScanChunk; i < end; ++i) {
      const uint64_t v = in[i];
      out[i] = acc;
      acc += v;
    }
    if (end == n) out[n] = acc;
  }
};

template <class Ex>
int scanLong(Ex& ex, const uint64_t* in, uint64_t* out, uint64_t n, int sums_slot, int starts_slot) {
  if (n <= kShortScan) return ex.scan(in, out, n);
  const uint64_t chunks = (n + kScanChunk - 1) / kScanChunk;
  uint64_t* sums = ex.template alloc<uint64_t>(Slot(sums_slot), chunks + 1);
  uint64_t* starts = ex.template alloc<uint64_t>(Slot(starts_slot), chunks + 1);
  if (!sums || !starts) return -1;
  int rc;
  if ((rc = ex.forEach(chunks, ChunkSumPass{in, n, sums}))) return rc;
  if ((rc = ex.scan(sums, starts, chunks))) return rc;
  return ex.forEach(chunks, ChunkScanPass{in, n, starts, out});
}

// ------------------------------------------------------------ strand table of a pile
// The strand table of an uploaded geometry pile (strand_table.h builds the same by one
// walk on the host).  The walk follows a chain: the strand at byte 0, then each next
// one right after it, stopping at the first header that is too short, odd, or runs past
// the pile, or where fewer than 32 bytes remain.  Here every 16-byte unit reads the
// header it would hold and points to the unit after that strand (or to a sink when the
// header is not valid there); the chain from unit 0 is then found by pointer doubling
// -- round k marks, from every unit already reached, the unit 2^k strands further --
// so after ceil(log2(units)) + 1 rounds every strand start is marked.  A marked unit
// with a valid header is a strand; a scan numbers them.
struct StrandLinkPass {
  const uint8_t* geo;
  uint64_t bytes, units;
  uint64_t* next;     // per unit: the unit after its strand, or `units` (the sink)
  uint8_t* valid;
  uint8_t* reached;
  GUDNI_SHD void operator()(uint64_t u) const {
    const uint64_t off = 16 * u;
    bool ok = off + 32 <= bytes;
    uint32_t size = 0;
    if (ok) {
      size = (uint32_t)geo[off] | ((uint32_t)geo[off + 1] << 8);
      ok = size >= 4 && (size & 1u) == 0 && off + (uint64_t)size * 8 <= bytes && off / 8 <= 0xFFFFFFFFull;
    }
    valid[u] = ok ? 1 : 0;
    next[u] = ok ? u + size / 2 : units;
    reached[u] = u == 0 ? 1 : 0;
  }
};

// one doubling round: reached' = reached plus the units `jump` leads to from reached
// ones; jump' = jump applied twice
struct StrandReachPass {
  const uint64_t* jump;
  const uint8_t* reached;
  uint64_t units;
  uint8_t* reached_next;  // a copy of `reached` beforehand
  GUDNI_SHD void operator()(uint64_t u) const {
    if (reached[u] && jump[u] < units) reached_next[jump[u]] = 1;
  }
};
struct StrandJumpPass {
  const uint64_t* jump;
  uint64_t units;
  uint64_t* jump_next;
  GUDNI_SHD void operator()(uint64_t u) const { jump_next[u] = jump[u] < units ? jump[jump[u]] : units; }
};
struct ByteCopyPass {
  const uint8_t* in;
  uint8_t* out;
  GUDNI_SHD void operator()(uint64_t i) const { out[i] = in[i]; }
};
struct StrandFlagPass {
  const uint8_t* reached;
  const uint8_t* valid;
  uint64_t* is_start;
  GUDNI_SHD void operator()(uint64_t u) const { is_start[u] = reached[u] && valid[u] ? 1 : 0; }
};

// per strand start: its table row, y range and unit mark (strand_table.h's entries)
struct StrandRowPass {
  const uint8_t* geo;
  const uint64_t* is_start;
  const uint64_t* index;  // exclusive scan of is_start
  uint4* table;
  float2* ys;
  uint32_t* first;
  GUDNI_SHD void operator()(uint64_t u) const {
    if (!is_start[u]) {
      first[u] = kNoStrand;
      return;
    }
    const uint64_t off = 16 * u;
    const uint32_t size = (uint32_t)geo[off] | ((uint32_t)geo[off + 1] << 8);
    const float* p = reinterpret_cast<const float*>(geo + off + 8);
    float lo = INFINITY, hi = -INFINITY;
    bool bad = false;
    for (uint32_t i = 0; i + 1 < size; ++i) {  // every point: (size - 1) 8-byte pairs
      const float x = p[2 * i], y = p[2 * i + 1];
      if (!(fabsf(x) <= kStrandCullExtent) || !(fabsf(y) <= kStrandCullExtent)) bad = true;
      lo = y < lo ? y : lo;
      hi = hi < y ? y : hi;
    }
    const uint32_t k = (uint32_t)index[u];
    table[k] = make_uint4((uint32_t)(off / 8), size, floatBits(p[2]), floatBits(p[0]));
    ys[k] = bad ? make_float2(-INFINITY, INFINITY) : make_float2(lo, hi);
    first[u] = k;
  }
};

struct StrandTableOut {
  uint4* table;
  float2* ys;
  uint32_t* first;
  uint64_t n_strands;
};

// The strand table of `bytes` bytes of pile at `geo` (on the executing side).  The
// table and y ranges go to slots kStrandTable / kStrandY, the per-unit map to
// kStrandFirst.  Returns 0, -1 (storage) or -2 (more strands than 32-bit indices).
template <class Ex>
int strandTable(Ex& ex, const uint8_t* geo, uint64_t bytes, StrandTableOut& out) {
  int rc;
  const uint64_t units = bytes / 16;
  uint64_t* next = ex.template alloc<uint64_t>(kKeysA, units + 1);
  uint64_t* next2 = ex.template alloc<uint64_t>(kKeysB, units + 1);
  uint8_t* valid = ex.template alloc<uint8_t>(kRect, units + 1);
  uint8_t* reached = ex.template alloc<uint8_t>(kPairCount, units + 1);
  uint8_t* reached2 = ex.template alloc<uint8_t>(kPairAt, units + 1);
  uint64_t* is_start = ex.template alloc<uint64_t>(kHist, units + 1);
  uint64_t* index = ex.template alloc<uint64_t>(kHistAt, units + 1);
  if (!next || !next2 || !valid || !reached || !reached2 || !is_start || !index) return -1;
  if ((rc = ex.forEach(units, StrandLinkPass{geo, bytes, units, next, valid, reached}))) return rc;
  int rounds = 1;
  while (rounds < 64 && (1ull << (rounds - 1)) < units) ++rounds;
  for (int k = 0; k < rounds; ++k) {
    if ((rc = ex.forEach(units, ByteCopyPass{reached, reached2}))) return rc;
    if ((rc = ex.forEach(units, StrandReachPass{next, reached, units, reached2}))) return rc;
    if ((rc = ex.forEach(units, StrandJumpPass{next, units, next2}))) return rc;
    uint8_t* tr = reached;
    reached = reached2;
    reached2 = tr;
    uint64_t* tj = next;
    next = next2;
    next2 = tj;
  }
  if ((rc = ex.forEach(units, StrandFlagPass{reached, valid, is_start}))) return rc;
  if ((rc = scanLong(ex, is_start, index, units, kScanSums, kScanStarts))) return rc;
  uint64_t n = 0;
  if ((rc = ex.read(&n, index + units, 8))) return rc;
  if (n >= 0xFFFFFFF0ull) return -2;
  out.table = ex.template alloc<uint4>(kStrandTable, n);
  out.ys = ex.template alloc<float2>(kStrandY, n);
  out.first = ex.template alloc<uint32_t>(kStrandFirst, units);
  if (!out.table || !out.ys || !out.first) return -1;
  if ((rc = ex.forEach(units, StrandRowPass{geo, is_start, index, out.table, out.ys, out.first}))) return rc;
  out.n_strands = n;
  return 0;
}

// ------------------------------------------------------------ the whole serializer

struct Result {
  uint64_t geometry_bytes = 0, n_strands = 0, n_shapes = 0, n_tiles = 0, n_jobs = 0;
  int64_t stats[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // as gudni_frame_stats
  const uint8_t* geometry = nullptr;
  const uint4* strand_table = nullptr;
  const float2* strand_y = nullptr;
  const uint32_t* strand_first = nullptr;
  const gudni_shape* shapes = nullptr;
  const gudni_tile_info* tiles = nullptr;
  const int32_t* tile_jobs = nullptr;
  uint64_t n_points = 0;                    // points of the pile (provenance, when asked)
  const uint32_t* point_offsets = nullptr;  // float index of each point's x
  const int32_t* point_sources = nullptr;   // 3 per point
  const float* point_weights = nullptr;     // 3 per point
};

// Runs every pass with executor `ex`:
//   T* ex.template alloc<T>(Slot, n)     storage for n elements (contents undefined)
//   int ex.forEach(n, pass)              pass(i) for every i < n (any order)
//   int ex.scan(in, out, n)              out[i] = in[0] + ... + in[i-1], i <= n
//   int ex.read(host_dst, src, bytes)    copy to the host
//   int ex.copy(dst, src, bytes)         copy on the executing side
//   int ex.upload(dst, host_src, bytes)  copy from the host
// each returning 0 or an error code; the first error ends the run.
template <class Ex>
int serialize(Ex& ex, const Scene& s, const Limits& lim, Result& res, bool provenance = false) {
  int rc;
#define GUDNI_SER_TRY(x) \
  if ((rc = (x)) != 0) return rc
  const uint64_t n_shapes = (uint64_t)(s.shape1 - s.shape0);
  const uint64_t n_outlines = (uint64_t)(s.outline1 - s.outline0);

  // reorder rows
  int rows_h[kRows][kMaxPoints];
  buildReorderRows(rows_h);
  int* rows = ex.template alloc<int>(kReorder, (uint64_t)kRows * kMaxPoints);
  if (!rows) return -1;
  GUDNI_SER_TRY(ex.upload(rows, &rows_h[0][0], sizeof(rows_h)));

  // shapes: substance, box, canvas test; outlines: their shape and size
  int32_t* shape_sub = ex.template alloc<int32_t>(kShapeSub, n_shapes);
  Box* box = ex.template alloc<Box>(kBox, n_shapes);
  uint64_t* keep = ex.template alloc<uint64_t>(kKeep, n_shapes + 1);
  uint64_t* kept_at = ex.template alloc<uint64_t>(kKeptAt, n_shapes + 1);
  int32_t* outline_shape = ex.template alloc<int32_t>(kOutlineShape, n_outlines);
  uint64_t* obytes = ex.template alloc<uint64_t>(kOutlineBytes, n_outlines + 1);
  uint64_t* byte_at = ex.template alloc<uint64_t>(kByteAt, n_outlines + 1);
  uint64_t* ostrands = ex.template alloc<uint64_t>(kOutlineStrands, n_outlines + 1);
  uint64_t* strand_at = ex.template alloc<uint64_t>(kStrandAt, n_outlines + 1);
  if (!shape_sub || !box || !keep || !kept_at || !outline_shape || !obytes || !byte_at || !ostrands || !strand_at)
    return -1;
  GUDNI_SER_TRY(ex.forEach((uint64_t)s.n_substances, ShapeSubstancePass{s, shape_sub}));
  GUDNI_SER_TRY(ex.forEach(n_shapes, ShapeBoxPass{s, box, keep, outline_shape}));
  GUDNI_SER_TRY(ex.forEach(n_outlines, OutlineSizePass{s, outline_shape, keep, obytes, ostrands}));
  GUDNI_SER_TRY(scanLong(ex, keep, kept_at, n_shapes, kScanSums, kScanStarts));
  GUDNI_SER_TRY(scanLong(ex, obytes, byte_at, n_outlines, kScanSums, kScanStarts));
  GUDNI_SER_TRY(scanLong(ex, ostrands, strand_at, n_outlines, kScanSums, kScanStarts));
  uint64_t n_kept = 0, geo_bytes = 0, n_strands = 0;
  GUDNI_SER_TRY(ex.read(&n_kept, kept_at + n_shapes, 8));
  GUDNI_SER_TRY(ex.read(&geo_bytes, byte_at + n_outlines, 8));
  GUDNI_SER_TRY(ex.read(&n_strands, strand_at + n_outlines, 8));
  if (n_strands >= 0xFFFFFFF0ull || geo_bytes / 16 > 0xFFFFFFFFull) return -2;

  // the geometry pile and its strand table
  StrandOut so;
  so.geo = ex.template alloc<uint8_t>(kGeometry, geo_bytes);
  so.table = ex.template alloc<uint4>(kStrandTable, n_strands);
  so.ys = ex.template alloc<float2>(kStrandY, n_strands);
  so.first = ex.template alloc<uint32_t>(kStrandFirst, geo_bytes / 16);
  so.rows = rows;
  if (!so.geo || !so.table || !so.ys || !so.first) return -1;
  const uint64_t n_points = (geo_bytes - 8 * n_strands) / 8;
  so.psrc = nullptr;
  so.pw = nullptr;
  so.pat = nullptr;
  if (provenance) {
    so.psrc = ex.template alloc<int32_t>(kPointSources, 3 * n_points);
    so.pw = ex.template alloc<float>(kPointWeights, 3 * n_points);
    so.pat = ex.template alloc<uint32_t>(kPointOffsets, n_points);
    if (!so.psrc || !so.pw || !so.pat) return -1;
  }
  GUDNI_SER_TRY(ex.forEach(geo_bytes / 16, FillPass{so.first, kNoStrand}));
  GUDNI_SER_TRY(ex.forEach(n_outlines, OutlineWritePass{s, outline_shape, keep, byte_at, strand_at, so}));
  KeptShape* kept = ex.template alloc<KeptShape>(kKept, n_kept);
  if (!kept) return -1;
  GUDNI_SER_TRY(ex.forEach(n_shapes, KeptPass{s, shape_sub, box, keep, kept_at, byte_at, strand_at, kept}));

  // the tile tree: base tiles (buildTileTree, TileTree.hs:81-109)
  const int canvas_depth = adjustedLog(s.canvas_w > s.canvas_h ? s.canvas_w : s.canvas_h);
  const int tile_depth = adjustedLog(lim.max_tile_size);
  const int depth = canvas_depth > tile_depth ? tile_depth : canvas_depth;
  const int levels = canvas_depth - depth;
  if (levels > 15) return -2;
  uint64_t n_nodes = 1ull << (2 * levels);
  const int tile_side = 1 << depth;
  const int grid_n = 1 << levels;
  // the (base tile, shape) pairs, sorted by tile with each tile's shapes in order
  int4* rect = ex.template alloc<int4>(kRect, n_kept);
  uint64_t* pair_count = ex.template alloc<uint64_t>(kPairCount, n_kept + 1);
  uint64_t* pair_at = ex.template alloc<uint64_t>(kPairAt, n_kept + 1);
  if (!rect || !pair_count || !pair_at) return -1;
  GUDNI_SER_TRY(ex.forEach(n_kept, ReachPass{kept, grid_n, tile_side, rect, pair_count}));
  GUDNI_SER_TRY(scanLong(ex, pair_count, pair_at, n_kept, kScanSums, kScanStarts));
  uint64_t n_pairs = 0;
  GUDNI_SER_TRY(ex.read(&n_pairs, pair_at + n_kept, 8));
  if (n_pairs > 0xFFFFFFFFull) return -2;
  uint64_t pool_cap = n_pairs + n_pairs / 2 + 1024;
  int pool_slot = kPoolA;
  uint32_t* keys = ex.template alloc<uint32_t>(kKeysA, n_pairs);
  uint32_t* pool = ex.template alloc<uint32_t>(kPoolA, pool_cap);
  if (!keys || !pool) return -1;
  GUDNI_SER_TRY(ex.forEach(n_kept, PairPass{rect, pair_at, levels, keys, pool}));
  const uint64_t blocks = (n_pairs + kRadixBlock - 1) / kRadixBlock;
  int key_slot = kKeysA;
  for (int shift = 0; shift < 2 * levels && n_pairs > 0; shift += kRadixBits) {
    uint64_t* hist = ex.template alloc<uint64_t>(kHist, (uint64_t)kRadixDigits * blocks + 1);
    uint64_t* hist_at = ex.template alloc<uint64_t>(kHistAt, (uint64_t)kRadixDigits * blocks + 1);
    const int other_keys = key_slot == kKeysA ? kKeysB : kKeysA;
    const int other_pool = pool_slot == kPoolA ? kPoolB : kPoolA;
    uint32_t* keys_out = ex.template alloc<uint32_t>(Slot(other_keys), n_pairs);
    uint32_t* pool_out = ex.template alloc<uint32_t>(Slot(other_pool), pool_cap);
    if (!hist || !hist_at || !keys_out || !pool_out) return -1;
    GUDNI_SER_TRY(ex.forEach(blocks, RadixCountPass{keys, n_pairs, blocks, shift, hist}));
    GUDNI_SER_TRY(scanLong(ex, hist, hist_at, (uint64_t)kRadixDigits * blocks, kScanSums, kScanStarts));
    GUDNI_SER_TRY(ex.forEach(blocks, RadixScatterPass{keys, pool, n_pairs, blocks, shift, hist_at, keys_out, pool_out}));
    keys = keys_out;
    pool = pool_out;
    key_slot = other_keys;
    pool_slot = other_pool;
  }
  // the base tiles: their runs of the sorted pairs are their lists
  Node* nodes = ex.template alloc<Node>(kNodesA, n_nodes);
  uint64_t* first = ex.template alloc<uint64_t>(kTileFirst, n_nodes);
  uint64_t* end = ex.template alloc<uint64_t>(kTileEnd, n_nodes);
  if (!nodes || !first || !end) return -1;
  GUDNI_SER_TRY(ex.forEach(n_nodes, Fill64Pass{first, 0}));
  GUDNI_SER_TRY(ex.forEach(n_nodes, Fill64Pass{end, 0}));
  GUDNI_SER_TRY(ex.forEach(n_pairs, RunPass{keys, n_pairs, first, end}));
  GUDNI_SER_TRY(ex.forEach(n_nodes, BaseNodePass{kept, pool, first, end, levels, tile_side, depth, nodes}));
  uint64_t pool_used = n_pairs;

  // splits, one level per pass, until no tile splits
  int node_slot = kNodesA;
  int64_t n_splits = 0;
  for (int level = 0; level < kMaxLevels; ++level) {
    uint64_t* out_nodes = ex.template alloc<uint64_t>(kOutNodes, n_nodes + 1);
    uint64_t* node_at = ex.template alloc<uint64_t>(kNodeAt, n_nodes + 1);
    uint64_t* out_list = ex.template alloc<uint64_t>(kOutList, n_nodes + 1);
    uint64_t* lat = ex.template alloc<uint64_t>(kListAt, n_nodes + 1);
    uint64_t* csize = ex.template alloc<uint64_t>(kChildSize, 2 * n_nodes);
    uint64_t* cstr = ex.template alloc<uint64_t>(kChildStrands, 2 * n_nodes);
    if (!out_nodes || !node_at || !out_list || !lat || !csize || !cstr) return -1;
    GUDNI_SER_TRY(ex.forEach(n_nodes, SplitCountPass{nodes, kept, pool, lim, out_nodes, out_list, csize, cstr}));
    GUDNI_SER_TRY(scanLong(ex, out_nodes, node_at, n_nodes, kScanSums, kScanStarts));
    GUDNI_SER_TRY(scanLong(ex, out_list, lat, n_nodes, kScanSums, kScanStarts));
    uint64_t next_nodes = 0, new_entries = 0;
    GUDNI_SER_TRY(ex.read(&next_nodes, node_at + n_nodes, 8));
    GUDNI_SER_TRY(ex.read(&new_entries, lat + n_nodes, 8));
    if (next_nodes == n_nodes) break;  // nothing split: every node is a leaf
    n_splits += (int64_t)(next_nodes - n_nodes);
    if (pool_used + new_entries > pool_cap) {  // grow the pool, keeping its lists
      const uint64_t cap = 2 * (pool_used + new_entries);
      const int other = pool_slot == kPoolA ? kPoolB : kPoolA;
      uint32_t* grown = ex.template alloc<uint32_t>(Slot(other), cap);
      if (!grown) return -1;
      if (pool_used) GUDNI_SER_TRY(ex.copy(grown, pool, pool_used * 4));
      pool = grown;
      pool_cap = cap;
      pool_slot = other;
    }
    const int other_nodes = node_slot == kNodesA ? kNodesB : kNodesA;
    Node* next = ex.template alloc<Node>(Slot(other_nodes), next_nodes);
    if (!next) return -1;
    GUDNI_SER_TRY(ex.forEach(n_nodes, SplitEmitPass{nodes, kept, pool, pool_used, lim, node_at, lat, csize, cstr, next}));
    pool_used += new_entries;
    nodes = next;
    node_slot = other_nodes;
    n_nodes = next_nodes;
    if (level == kMaxLevels - 1) return -2;
  }

  // jobs: leaves in traversal order, max_tiles_per_call per job, last built first
  const uint64_t per_job = (uint64_t)lim.max_tiles_per_call;
  const uint64_t n_jobs = (n_nodes + per_job - 1) / per_job;
  uint64_t* leaf_counts = ex.template alloc<uint64_t>(kLeafCounts, n_nodes + 1);
  uint64_t* shape_at = ex.template alloc<uint64_t>(kShapeAt, n_nodes + 1);
  if (!leaf_counts || !shape_at) return -1;
  GUDNI_SER_TRY(ex.forEach(n_nodes, LeafCountPass{nodes, n_nodes, per_job, leaf_counts}));
  GUDNI_SER_TRY(scanLong(ex, leaf_counts, shape_at, n_nodes, kScanSums, kScanStarts));
  uint64_t n_refs = 0;
  GUDNI_SER_TRY(ex.read(&n_refs, shape_at + n_nodes, 8));
  if (n_refs > 0xFFFFFFFFull) return -2;
  gudni_tile_info* tiles = ex.template alloc<gudni_tile_info>(kTiles, n_nodes);
  int32_t* tile_jobs = ex.template alloc<int32_t>(kTileJobs, n_nodes);
  gudni_shape* shapes = ex.template alloc<gudni_shape>(kShapes, n_refs);
  if (!tiles || !tile_jobs || !shapes) return -1;
  GUDNI_SER_TRY(ex.forEach(n_nodes, LeafEmitPass{nodes, kept, pool, n_nodes, per_job, n_jobs, lim.threads_per_tile,
                                                 shape_at, tiles, tile_jobs, shapes}));

  // the largest leaf lists (gudni_frame_stats [5], [6])
  uint64_t most[2] = {0, 0};
  {
    uint64_t* m = ex.template alloc<uint64_t>(kLeafCounts, 2);
    if (!m) return -1;
    GUDNI_SER_TRY(ex.forEach(2, Fill64Pass{m, 0}));
    GUDNI_SER_TRY(ex.forEach(n_nodes, LeafMaxPass{nodes, reinterpret_cast<unsigned long long*>(m)}));
    GUDNI_SER_TRY(ex.read(most, m, 16));
  }
  const uint64_t most_shapes = most[0], most_strands = most[1];
#undef GUDNI_SER_TRY

  res.geometry_bytes = geo_bytes;
  res.n_strands = n_strands;
  res.n_shapes = n_refs;
  res.n_tiles = n_nodes;
  res.n_jobs = n_jobs;
  res.stats[0] = (int64_t)n_kept;
  res.stats[1] = (int64_t)(n_shapes - n_kept);
  res.stats[2] = (int64_t)n_strands;
  res.stats[3] = (int64_t)n_nodes;
  res.stats[4] = n_splits;
  res.stats[5] = (int64_t)most_shapes;
  res.stats[6] = (int64_t)most_strands;
  res.stats[7] = (int64_t)n_refs;
  res.geometry = so.geo;
  res.strand_table = so.table;
  res.strand_y = so.ys;
  res.strand_first = so.first;
  res.shapes = shapes;
  res.tiles = tiles;
  res.tile_jobs = tile_jobs;
  res.n_points = provenance ? n_points : 0;
  res.point_offsets = so.pat;
  res.point_sources = so.psrc;
  res.point_weights = so.pw;
  return 0;
}

}  // namespace ser
}  // namespace gudni
