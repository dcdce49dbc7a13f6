// Device-side column machine of the raster path (sm_103a).
//
// One "column" is the reference's work item: the 1-pixel-wide slab of one tile that
// one OpenCL work-item renders (initTileState, Kernels.cl:1692-1718).  Per column the
// machine generates thresholds (generateThresholds, K:2030-2082), orders them
// (sortThresholds, K:2084-2115) and scans them into pixels (renderThresholds,
// K:2117-2167).  The arithmetic is the reference's, operation for operation, in IEEE
// single precision (the library is built with --fmad=false and IEEE division and
// square root), so results are bit-identical to the reference kernels evaluated with
// IEEE semantics.
//
// Ordering: thresholds are pushed as the reference pushes them, then sorted with a
// stable insertion or merge sort instead of the reference's bubble sort.  All produce
// the unique stable order of the comparator K:1940-1951 over the reversed push order,
// so the queue the render scan sees is identical.
//
// Safety: every loop is bounded; strand, shape, substance and picture reads are
// bounds-checked against the uploaded buffers; violations set a status bit and skip
// the read instead of faulting.
#pragma once

#include <cfloat>
#include <cstdint>

#include "gudni_cuda.h"

namespace gudni {

// status bits raised by kernels (mapped to GUDNI_ERR_* by the host)
constexpr int kStatusOverflow = 1;   // a column needed more than max_thresholds
constexpr int kStatusIterLimit = 2;  // a bounded loop hit its cap
constexpr int kStatusBadInput = 4;   // a record pointed outside its buffer

constexpr float kMinCrop = 0.2f;            // MINCROP K:47
constexpr float kLeft = 0.0f;               // LEFTBORDER K:90
constexpr float kRight = 1.0f;              // RIGHTBORDER K:91
constexpr float kFlatness = 0.25f;          // TAXICAB_FLATNESS K:250
// Hulls whose twelve coordinate magnitudes SUM to more than this are not culled (the
// strand table bounds each coordinate by it instead, so the hull test is the stricter
// of the two): below 2^21 per coordinate the intercept arithmetic stays finite and its
// rounding far inside the one-pixel culling margin.
constexpr float kCullExtent = 2097152.0f;
constexpr float kHalf = 0.5f;               // T K:249
constexpr int kLargePrime = 7919;           // K:83
// Halvings of a quadratic before giving up.  With finite coordinates the reference's
// halving ends within ~131 steps (an x or y extent of at most 2^129 halved to the 0.25
// flatness; coincident points end it sooner), so the cap changes no finite input; it
// ends the loops the reference never leaves (an endpoint at +-inf the column position
// never separates).
constexpr int kBifurcateCap = 256;
constexpr int kSectionCap = 1 << 22;        // sections per pixel before giving up

constexpr uint32_t kPositive = 0x80000000u;
constexpr uint32_t kPersistSlopeMask = 0xC0000000u;
constexpr uint32_t kPersistTop = 0xC0000000u;
constexpr uint32_t kPersistBottom = 0x40000000u;
constexpr uint32_t kPersist = 0x40000000u;
constexpr uint32_t kUnpersist = 0xBFFFFFFFu;
constexpr uint32_t kShapeBitMask = 0x0FFFFFFFu;

// Everything a column reads.  Device pointers.
struct RasterInputs {
  const uint8_t* geometry;       // strand heap
  size_t geometry_bytes;
  const float4* substances;
  uint32_t n_substances;
  const uint8_t* pictures;
  size_t picture_bytes;
  const gudni_picture_use* uses;
  uint32_t n_uses;
  const gudni_radial* radials;
  uint32_t n_radials;
  const float* random_field;     // may be null when stochastic == 0
  float stochastic;
  const gudni_shape* shapes;     // job shape pile
  uint32_t n_shapes;
  const gudni_tile_info* tiles;  // job tile pile
  int n_tiles;
  int log2_tpt;                  // computeDepth
  int bitmap_w, bitmap_h;
  int job_index;
  float4 background;
  int max_shape;
  uint32_t* out;                 // bitmap_w * bitmap_h BGRA words
  const int32_t* tile_jobs;      // optional per-tile job index (frame launches)
  int64_t* counters;             // optional work counters (see gudni_enable_counters)
  // Strand table of the geometry pile (optional; see StrandEntry).
  const uint4* strand_table;     // one entry per strand
  const float2* strand_y;        // per strand: lowest and highest point y (absolute)
  uint32_t n_strands;
  const uint32_t* strand_first;  // per 16-byte unit of the pile: strand index starting there
  uint32_t n_units;              // geometry_bytes / 16
  // Source of the stochastic area jitter (read only when stochastic != 0):
  // kRandomField, the reference's random field walked by a per-column cursor, or
  // kRandomCounter, a counter-based hash of (random_seed, pixel, the section's ordinal
  // in the column's scan), which needs no table and does not repeat every 4096
  // sections.
  uint32_t random_mode;
  uint64_t random_seed;
};

constexpr uint32_t kRandomField = 0;
constexpr uint32_t kRandomCounter = 1;

// SplitMix64's output function (Steele, Lea and Flood, "Fast splittable pseudorandom
// number generators", OOPSLA 2014): a bijective 64-bit mix.
__host__ __device__ __forceinline__ uint64_t splitMix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// The counter-based jitter of pixel (x, y) for the section with ordinal k in its
// column's scan: the top 24 bits of the mixed counter as a float in [0, 1) (exact:
// 24 bits times 2^-24).
__host__ __device__ __forceinline__ float counterRandom(uint64_t seed, int x, int y, uint32_t k) {
  const uint64_t pixel = ((uint64_t)(uint32_t)x << 32) | (uint64_t)(uint32_t)y;
  const uint64_t h = splitMix64(splitMix64(seed ^ pixel) + (uint64_t)k);
  return (float)(uint32_t)(h >> 40) * (1.0f / 16777216.0f);
}

// A strand table entry (16 bytes, one load): x = byte offset / 8 of the strand in the
// geometry pile, y = its size in 8-byte units, z = bits of the strand's left x,
// w = bits of its right x -- the two floats the column range test reads
// (checkInRange, Kernels.cl:1360-1363).  strand_first maps a shape's geo_start to
// the index of its first strand (kNoStrand where no strand starts).
constexpr uint32_t kNoStrand = 0xFFFFFFFFu;

__device__ __forceinline__ float cl_min(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float cl_max(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float cl_fmin(float x, float y) {
  return isnan(y) ? x : (isnan(x) ? y : cl_min(x, y));
}
__device__ __forceinline__ float cl_fmax(float x, float y) {
  return isnan(y) ? x : (isnan(x) ? y : cl_max(x, y));
}

__device__ __forceinline__ bool hPositive(uint32_t h) { return (h & kPositive) != 0; }
__device__ __forceinline__ bool hPersistTop(uint32_t h) { return (h & kPersistSlopeMask) == kPersistTop; }
__device__ __forceinline__ bool hPersistBottom(uint32_t h) { return (h & kPersistSlopeMask) == kPersistBottom; }
__device__ __forceinline__ bool tKeep(uint32_t h, float4 t) {
  return ((h & kPersist) != 0) || (t.y - t.x >= kMinCrop);
}
__device__ __forceinline__ float tTopX(uint32_t h, float4 t) { return hPositive(h) ? t.z : t.w; }

// thresholdInvertedSlope K:240-246
__device__ __forceinline__ float invSlope(uint32_t h, float4 t) {
  float sign = hPositive(h) ? 1.0f : -1.0f;
  return (t.x == t.y) ? FLT_MAX : (t.w - t.z) / (t.y - t.x) * sign;
}
// thresholdIntersectX K:900-913
__device__ __forceinline__ float intersectX(uint32_t h, float4 t, float y) {
  if (t.z == t.w) return t.z;
  float sy = hPositive(h) ? t.x : t.y;
  return ((y - sy) * invSlope(h, t)) + t.z;
}
// thresholdIsBelow K:1079-1094
__device__ __forceinline__ bool isBelow(uint32_t ah, float4 a, uint32_t bh, float4 b) {
  if (a.x > b.x) return true;
  if (a.x != b.x) return false;
  float ax = tTopX(ah, a), bx = tTopX(bh, b);
  if (ax > bx) return true;
  if (ax != bx) return false;
  return invSlope(ah, a) > invSlope(bh, b);
}

// Threshold queue of one column: entries live in [start, cap) of the column's slab
// and grow toward index 0 (initQueueSlice / pushTopSlot, K:402-405, K:1615-1620).
struct Queue {
  float4* thr;
  uint32_t* hdr;
  int start;
  int cap;
  bool overflow;
  __device__ __forceinline__ int length() const { return cap - start; }
  __device__ __forceinline__ float4 get(int i) const { return thr[start + i]; }
  __device__ __forceinline__ uint32_t getH(int i) const { return hdr[start + i]; }
  __device__ __forceinline__ void set(int i, float4 t) { thr[start + i] = t; }
  __device__ __forceinline__ void setH(int i, uint32_t h) { hdr[start + i] = h; }
  __device__ __forceinline__ void pop() { start += 1; }
  // pushThreshold K:1096-1103: the new entry goes to the front (unsorted)
  __device__ __forceinline__ void push(uint32_t h, float4 t) {
    if (start == 0) {
      overflow = true;
      return;
    }
    start -= 1;
    hdr[start] = h;
    thr[start] = t;
  }
  // insertThreshold K:1105-1124: the new entry goes in front of the first entry it is
  // not strictly below.
  __device__ __forceinline__ void insert(uint32_t h, float4 t) {
    if (start == 0) {
      overflow = true;
      return;
    }
    start -= 1;
    const int len = cap - start;
    int cursor = 0;
    while (cursor < len - 1) {
      uint32_t oh = hdr[start + cursor + 1];
      float4 o = thr[start + cursor + 1];
      if (!isBelow(h, t, oh, o)) break;
      hdr[start + cursor] = oh;
      thr[start + cursor] = o;
      cursor += 1;
    }
    hdr[start + cursor] = h;
    thr[start + cursor] = t;
  }
};

// The shape stack (ShapeState's shapeBits, K:270-292): one bit per shape of the
// column, 64 per word.  `nz` marks the non-zero words, so findTop skips empty words
// with one bit scan instead of a word-by-word walk (the reference walks the words;
// the bit it finds is the same).  `hiFlip` is the highest bit flipped since the last
// clearFlips(): the render scan uses it to tell whether a cached section colour
// still holds.
template <int SECTIONS>
struct ShapeStack {
  static_assert(SECTIONS >= 1 && SECTIONS <= 32, "at most 32 stack words");
  uint64_t w[SECTIONS];
  uint32_t nz;
  int hiFlip;
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int i = 0; i < SECTIONS; ++i) w[i] = 0ull;
    nz = 0u;
    hiFlip = -1;
  }
  __device__ __forceinline__ void clearFlips() { hiFlip = -1; }
  __device__ __forceinline__ void flip(uint32_t bit) {
    const int sec = (int)(bit >> 6);
    const uint64_t m = 1ull << (bit & 63);
    hiFlip = max(hiFlip, (int)bit);
    if (SECTIONS <= 8) {
      // select form: every word stays in a register
#pragma unroll
      for (int i = 0; i < SECTIONS; ++i) {
        if (i == sec) {
          w[i] ^= m;
          nz = w[i] ? (nz | (1u << i)) : (nz & ~(1u << i));
        }
      }
    } else {
      w[sec] ^= m;
      nz = w[sec] ? (nz | (1u << sec)) : (nz & ~(1u << sec));
    }
  }
  __device__ __forceinline__ uint64_t word(int sec) const {
    if (SECTIONS <= 8) {
      uint64_t r = 0ull;
#pragma unroll
      for (int i = 0; i < SECTIONS; ++i) r = (i == sec) ? w[i] : r;
      return r;
    }
    return w[sec];
  }
  __device__ __forceinline__ void pass(uint32_t h) { flip(h & kShapeBitMask); }
  __device__ __forceinline__ void passTop(uint32_t h) { if (hPersistTop(h)) pass(h); }
  __device__ __forceinline__ void passBottom(uint32_t h) { if (hPersistBottom(h)) pass(h); }
  // findTop K:281-292: the highest set bit below `ignoreAbove`, or -1
  __device__ __forceinline__ int findTop(int ignoreAbove) const {
    int sec = ignoreAbove >> 6;
    const int bits = ignoreAbove & 63;
    uint64_t s = (~(~0ull << bits)) & word(sec);
    if (s == 0ull) {
      const uint32_t below = nz & ((1u << sec) - 1u);
      if (below == 0u) return -1;
      sec = 31 - __clz((int)below);
      s = word(sec);
    }
    return (sec << 6) + (63 - __clzll((long long)s));
  }
};

// Column geometry (TileState, K:438-451 / initTileState K:1692-1718).
struct ColumnState {
  uint32_t shapeStart;
  int numShapes;
  int deltaX, deltaY;
  int internalY;
  int tileH;
  int intHeight;
  float floatHeight;
  int threadUnique;
  bool active;
};

__device__ __forceinline__ ColumnState initColumn(const RasterInputs& in, const gudni_tile_info& ti, int column,
                                                  int job_index) {
  ColumnState c;
  const int computeDepth = in.log2_tpt;
  c.shapeStart = ti.shapes.start;
  c.numShapes = (int)ti.shapes.length;
  int hDepth = ti.hdepth, vDepth = ti.vdepth;
  int diffDepth = max(0, vDepth - (computeDepth - hDepth));
  int desiredHeight = 1 << diffDepth;
  int internalX = ((1 << hDepth) - 1) & column;
  c.internalY = (column >> hDepth) << diffDepth;
  c.deltaX = internalX + ti.left;
  c.deltaY = c.internalY + ti.top;
  c.threadUnique = (ti.column_allocation + (1 << computeDepth) +
                    job_index * (1 << (computeDepth + computeDepth))) * kLargePrime;
  c.intHeight = min(desiredHeight, in.bitmap_h - c.deltaY);
  c.floatHeight = (float)c.intHeight;
  c.tileH = ti.bottom - ti.top;
  c.active = c.internalY < c.tileH && c.deltaX < in.bitmap_w && c.deltaY < in.bitmap_h;
  return c;
}

// ------------------------------------------------------------------ generate
struct Trav {
  float2 left, control, right;
  float xPos;
  int index;
};

// bifurcateCurve K:1233-1258 (bounded)
__device__ __forceinline__ void bifurcate(Trav& t, int& status) {
  if (t.left.x == t.control.x && t.left.y == t.control.y) return;
  for (int it = 0;; ++it) {
    if (it >= kBifurcateCap) {
      status |= kStatusIterLimit;
      return;
    }
    float2 lm = make_float2((1.0f - kHalf) * t.left.x + kHalf * t.control.x,
                            (1.0f - kHalf) * t.left.y + kHalf * t.control.y);
    float2 rm = make_float2((1.0f - kHalf) * t.control.x + kHalf * t.right.x,
                            (1.0f - kHalf) * t.control.y + kHalf * t.right.y);
    float2 on = make_float2((1.0f - kHalf) * lm.x + kHalf * rm.x, (1.0f - kHalf) * lm.y + kHalf * rm.y);
    float flat = fabsf(on.x - t.control.x) + fabsf(on.y - t.control.y);
    if (!(flat > kFlatness)) return;
    if (t.xPos < on.x) {
      t.control = lm;
      t.right = on;
    } else {
      t.left = on;
      t.control = rm;
    }
  }
}

// intersectCurve K:1226-1230
__device__ __forceinline__ float intersectCurve(Trav t, int& status) {
  bifurcate(t, status);
  if (t.left.x == t.right.x) return cl_min(t.left.y, t.right.y);
  return (((t.right.y - t.left.y) / (t.right.x - t.left.x)) * (t.xPos - t.left.x)) + t.left.y;
}

// Where generated thresholds go: a column's Queue, or (the cooperative generation of a
// tile, tile_coop.cuh) the few thresholds of one strand in one column.  Any sink with
// push(header, threshold).
template <class Sink>
struct GenStateOf {
  Sink* q;
  const ColumnState* c;
};
using GenState = GenStateOf<Queue>;

// addLineSegment / addThreshold K:1155-1220 (lineToThreshold/lineToHeader K:1131-1150,
// trimThresholdTop K:982-1005), inserting into sorted position.
template <class G>
__device__ __forceinline__ void addLineSegment(G& g, float2 left, float2 right, uint32_t shapeBit,
                                               bool& added, bool& enclosed) {
  float4 t = make_float4(cl_fmin(left.y, right.y), cl_fmax(left.y, right.y), left.x, right.x);
  bool positive = left.y <= right.y;
  bool persist = (left.x != right.x) && (left.x == kLeft);
  uint32_t h = (positive ? kPositive : 0u) | (persist ? kPersist : 0u) | shapeBit;
  if (!tKeep(h, t)) return;
  enclosed = enclosed || ((t.x <= 0.0f) && hPersistTop(h)) || ((t.y <= 0.0f) && hPersistBottom(h));
  if ((t.x < g.c->floatHeight) && (t.y > 0.0f) && (t.z < kRight)) {
    if (t.x <= 0.0f) {
      float splitX = intersectX(h, t, 0.0f);
      if (hPositive(h)) {
        t = make_float4(0.0f, t.y, splitX, t.w);
        h = h & kUnpersist;
      } else {
        t = make_float4(0.0f, t.y, t.z, splitX);
      }
    }
    if (t.w <= kLeft) {
      enclosed = true;
    } else {
      added = true;
      g.q->push(h, t);
    }
  }
}

// spawnThresholds K:1264-1333.  `above`: the whole strand lies at least a pixel above
// the column, so every line it spawns ends above the column top and only the
// enclosure flag (set by any persistent line, whatever its y) can change; the border
// intercepts are then not computed (any value above the column gives the same flags).
template <class G>
__device__ __forceinline__ void spawnThresholds(G& g, uint32_t shapeBit, Trav& l, Trav& r, bool& added,
                                                bool& enclosed, int& status, bool above = false) {
  float yL = (l.left.x >= kLeft) ? l.left.y : (above ? -1.0f : intersectCurve(l, status));
  bool leftWing = false;
  if ((l.right.x < kRight) && (l.right.x > kLeft)) {
    addLineSegment(g, make_float2(l.xPos, yL), l.right, shapeBit, added, enclosed);
    leftWing = true;
  }
  float yR = (r.right.x <= kRight) ? r.right.y : (above ? -1.0f : intersectCurve(r, status));
  bool rightWing = false;
  if ((r.left.x > kLeft) && (r.left.x < kRight) && (l.index != r.index)) {
    addLineSegment(g, r.left, make_float2(r.xPos, yR), shapeBit, added, enclosed);
    rightWing = true;
  }
  if (l.right.x < r.left.x || (!leftWing && !rightWing)) {
    float2 bl = (leftWing || (l.left.x == l.right.x)) ? l.right : make_float2(l.xPos, yL);
    float2 br = (rightWing || (r.left.x == r.right.x)) ? r.left : make_float2(r.xPos, yR);
    addLineSegment(g, bl, br, shapeBit, added, enclosed);
  }
}

// searchTree K:1337-1357 over the strand's complete binary tree of (point, control)
__device__ __forceinline__ void searchTree(Trav& t, const float4* tree, int treeSize, float2 d, bool isLeft) {
  t.index = 0;
  while (t.index < treeSize) {
    float4 n = tree[t.index];
    float cx = n.x - d.x, cy = n.y - d.y;
    if ((t.xPos < cx) || (isLeft && t.xPos == cx)) {
      t.right = make_float2(cx, cy);
      t.index = (t.index << 1) + 1;
    } else {
      t.left = make_float2(cx, cy);
      t.control = make_float2(n.z - d.x, n.w - d.y);
      t.index = (t.index << 1) + 2;
    }
  }
}

// traverseTree K:1378-1408 + spawnThresholds for one strand of `size` 8-byte units.
template <class G>
__device__ __forceinline__ void strandThresholds(G& g, const uint8_t* strand, uint32_t size, float2 d,
                                                 uint32_t shapeBit, bool& added, bool& enclosedByStrand,
                                                 int& status, bool above = false) {
  const int treeSize = ((int)size - 4) / 2;
  const float2 rp = *reinterpret_cast<const float2*>(strand + 8);
  const float4 lc = *reinterpret_cast<const float4*>(strand + 16);
  Trav l;
  l.right = make_float2(rp.x - d.x, rp.y - d.y);
  l.left = make_float2(lc.x - d.x, lc.y - d.y);
  l.control = make_float2(lc.z - d.x, lc.w - d.y);
  l.xPos = 0.0f;
  l.index = 0;
  if (l.left.x <= kRight && l.right.x > kLeft) {  // checkInRange K:1360-1363
    Trav r = l;
    l.xPos = cl_max(kLeft, l.left.x);
    r.xPos = cl_min(kRight, l.right.x);
    const float4* tree = reinterpret_cast<const float4*>(strand + 32);
    searchTree(l, tree, treeSize, d, true);
    searchTree(r, tree, treeSize, d, false);
    // every line spawnThresholds makes ends on a point of the two curves found or on
    // an intercept inside their hulls: cull by the hulls' y range (one-pixel margin)
    const float lo = fminf(fminf(fminf(l.left.y, l.control.y), fminf(l.right.y, r.left.y)),
                           fminf(r.control.y, r.right.y));
    const float hi = fmaxf(fmaxf(fmaxf(l.left.y, l.control.y), fmaxf(l.right.y, r.left.y)),
                           fmaxf(r.control.y, r.right.y));
    // the culling below needs intercepts that are numbers inside the hull's y range
    // (give or take rounding within the one-pixel margin): a NaN or infinite
    // coordinate, or finite ones so large that a difference or product overflows, can
    // make an intercept NaN or infinite.  The sum of the twelve magnitudes (NaN or
    // infinite whenever one is) bounds every coordinate.
    const float extent = fabsf(l.left.y) + fabsf(l.control.y) + fabsf(l.right.y) + fabsf(r.left.y) +
                       fabsf(r.control.y) + fabsf(r.right.y) + fabsf(l.left.x) + fabsf(l.control.x) +
                       fabsf(l.right.x) + fabsf(r.left.x) + fabsf(r.control.x) + fabsf(r.right.x);
    const bool ordered = extent <= kCullExtent;
    if (ordered && lo >= g.c->floatHeight + 1.0f) return;  // all below the column: dropped, no enclosure
    spawnThresholds(g, shapeBit, l, r, added, enclosedByStrand, status, above || (ordered && hi <= -1.0f));
  }
}

// buildThresholdArray K:1540-1595 with traverseTree K:1378-1408.
// Returns the number of shape bits assigned; shape indices go to `shapeIdx`.  With
// `nAsBit` (a tile of at most max_shape shapes, so no column runs out of bits) a
// shape's bit is its number n in the tile instead of the running count: the bits keep
// the shapes' order, so the colour walk meets the same shapes in the same order, and
// a tag is read straight from the tile's shape records (DirectTags).
template <int SECTIONS>
__device__ __forceinline__ uint32_t buildThresholds(const RasterInputs& in, const ColumnState& c, Queue& q,
                                                    ShapeStack<SECTIONS>& stack, uint32_t* shapeIdx,
                                                    int& status, bool nAsBit = false) {
  GenState g{&q, &c};
  const float2 d = make_float2((float)c.deltaX, (float)c.deltaY);
  uint32_t shapeBits = 0;
  for (int n = 0; n < c.numShapes && (int)shapeBits < in.max_shape; ++n) {
    const uint32_t shapeIndex = c.shapeStart + (uint32_t)n;
    const gudni_shape shape = in.shapes[shapeIndex];
    const uint32_t bit = nAsBit ? (uint32_t)n : shapeBits;
    bool added = false;
    bool enclosedByShape = false;
    uint32_t first = kNoStrand;
    if (in.strand_table && shape.geo_start < in.n_units) first = in.strand_first[shape.geo_start];
    if (first != kNoStrand && (uint64_t)first + shape.num_strands <= in.n_strands) {
      // Strand table: the range test reads one independent entry per strand; only
      // strands that cross the column touch the strand heap.  A strand that does not
      // cross it spawns nothing and leaves the enclosure unchanged.
      for (uint32_t k = 0; k < shape.num_strands; ++k) {
        const uint4 e = in.strand_table[first + k];
        const float lx = __uint_as_float(e.z) - d.x;
        const float rx = __uint_as_float(e.w) - d.x;
        if (!(lx <= kRight && rx > kLeft)) continue;
        // y culling with a one-pixel margin (every point a line can end on lies within
        // the strand's points' y range up to rounding): a strand wholly below the
        // column spawns only lines whose top is at or below its bottom, which are
        // dropped and leave the enclosure unchanged; one wholly above needs no
        // intercepts (spawnThresholds, `above`).
        const float2 yr = in.strand_y[first + k];
        if (yr.x - d.y >= c.floatHeight + 1.0f) continue;
        const bool above = yr.y - d.y <= -1.0f;
        bool enclosedByStrand = false;
        strandThresholds(g, in.geometry + (size_t)e.x * 8, e.y, d, bit, added, enclosedByStrand, status,
                         above);
        if (q.overflow) return shapeBits;
        enclosedByShape = enclosedByShape != enclosedByStrand;
      }
    } else {
      size_t off = (size_t)shape.geo_start * 16;
      for (uint32_t k = 0; k < shape.num_strands; ++k) {
        if (off + 32 > in.geometry_bytes) {
          status |= kStatusBadInput;
          break;
        }
        const uint8_t* strand = in.geometry + off;
        const uint32_t size = (uint32_t)(*reinterpret_cast<const uint16_t*>(strand));
        // a serialized strand is 2k+2 eight-byte units (k >= 1 curves); an odd size
        // would misalign the float4 reads of every strand after it
        if (size < 4 || (size & 1u) != 0 || off + (size_t)size * 8 > in.geometry_bytes) {
          status |= kStatusBadInput;
          break;
        }
        bool enclosedByStrand = false;
        strandThresholds(g, strand, size, d, bit, added, enclosedByStrand, status);
        if (q.overflow) return shapeBits;
        off += (size_t)size * 8;
        enclosedByShape = enclosedByShape != enclosedByStrand;
      }
    }
    if (enclosedByShape) stack.flip(bit);
    if (added || enclosedByShape) {
      if (!nAsBit) shapeIdx[shapeBits] = shapeIndex;
      shapeBits += 1;
    }
  }
  return shapeBits;
}

// sortThresholdArray K:1962-1976 replacement: the reference bubble-sorts the queue;
// its comparator is a strict weak order, so any stable sort gives the same order.
// isBelow is a strict weak order (lexicographic over top, top x and inverted slope)
// unless a key is NaN.  A threshold whose width and height differences are finite has
// no NaN key: top and top x are its own finite components, and the inverted slope is
// FLT_MAX or a finite width over a non-zero finite height.
__device__ __forceinline__ bool keysOrdered(float4 t) {
  return fabsf(t.w - t.z) <= FLT_MAX && fabsf(t.y - t.x) <= FLT_MAX;
}

// Short queues: insertion sort in place.  Longer ones: bottom-up merge sort using the
// free part of the column's slab below the queue as the second buffer (when it is
// large enough), O(n log n) instead of O(n^2).  Both give the stable sorted order, the
// order the reference's bubble sort gives, when the comparator is a strict weak order;
// a queue holding a threshold with a non-finite coordinate takes the reference's
// bubble sort itself (sortThresholdArray, K:1962-1976), since with a NaN key the
// orders can differ.
__device__ __forceinline__ void sortQueue(Queue& q) {
  const int n = q.length();
  const int s = q.start;
  float4* T = q.thr;
  uint32_t* H = q.hdr;
  bool ordered = true;
  for (int i = s; i < q.cap && ordered; ++i) ordered = keysOrdered(T[i]);
  if (!ordered) {
    bool done = false;
    for (int k = n; !done; --k) {
      done = true;
      for (int i = s; i < s + k - 1; ++i) {
        if (isBelow(H[i], T[i], H[i + 1], T[i + 1])) {
          const float4 t = T[i];
          const uint32_t h = H[i];
          T[i] = T[i + 1];
          H[i] = H[i + 1];
          T[i + 1] = t;
          H[i + 1] = h;
          done = false;
        }
      }
    }
    return;
  }
  if (n < 32 || s < n) {
    for (int i = s + 1; i < q.cap; ++i) {
      const float4 t = T[i];
      const uint32_t h = H[i];
      int j = i - 1;
      while (j >= s && isBelow(H[j], T[j], h, t)) {
        T[j + 1] = T[j];
        H[j + 1] = H[j];
        --j;
      }
      T[j + 1] = t;
      H[j + 1] = h;
    }
    return;
  }
  // ping-pong between [s, s+n) and [s-n, s)
  int src = s, dst = s - n;
  for (int width = 1; width < n; width *= 2) {
    for (int lo = 0; lo < n; lo += 2 * width) {
      const int mid = min(lo + width, n), hi = min(lo + 2 * width, n);
      int a = lo, b = mid, o = lo;
      while (a < mid && b < hi) {
        // take the right run's head only when the left head is strictly below it
        if (isBelow(H[src + a], T[src + a], H[src + b], T[src + b])) {
          T[dst + o] = T[src + b];
          H[dst + o] = H[src + b];
          ++b;
        } else {
          T[dst + o] = T[src + a];
          H[dst + o] = H[src + a];
          ++a;
        }
        ++o;
      }
      while (a < mid) {
        T[dst + o] = T[src + a];
        H[dst + o] = H[src + a];
        ++a;
        ++o;
      }
      while (b < hi) {
        T[dst + o] = T[src + b];
        H[dst + o] = H[src + b];
        ++b;
        ++o;
      }
    }
    const int t = src;
    src = dst;
    dst = t;
  }
  if (src != s) {
    for (int i = 0; i < n; ++i) {
      T[s + i] = T[src + i];
      H[s + i] = H[src + i];
    }
  }
}

// ------------------------------------------------------------------ render
__device__ __forceinline__ float4 composite(float4 fg, float4 bg) {  // K:878-887
  float alphaOut = fg.w + bg.w * (1.0f - fg.w);
  if (alphaOut > 0.0f) {
    // (background * ALPHA(background)) * (1 - ALPHA(foreground)), left to right
    float k = 1.0f - fg.w;
    return make_float4(((fg.x * fg.w) + ((bg.x * bg.w) * k)) / alphaOut,
                       ((fg.y * fg.w) + ((bg.y * bg.w) * k)) / alphaOut,
                       ((fg.z * fg.w) + ((bg.z * bg.w) * k)) / alphaOut, alphaOut);
  }
  return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// readColor K:1411-1442 plus the radial-gradient substance (evaluated at the
// integer pixel position like a picture texel).
__device__ __forceinline__ float4 readColor(const RasterInputs& in, int px, int py, uint64_t sid, uint64_t type,
                                            int& status, int64_t& texels) {
  if (sid >= in.n_substances) {
    status |= kStatusBadInput;
    return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  const float4 sub = in.substances[sid];
  if (type == GUDNI_TAG_SOLID) return sub;
  const uint32_t id = __float_as_uint(sub.x);
  if (type == GUDNI_TAG_RADIAL) {
    if (id >= in.n_radials) {
      status |= kStatusBadInput;
      return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    const gudni_radial& g = in.radials[id];
    float dx = (float)px - g.center_x, dy = (float)py - g.center_y;
    float dist = sqrtf(dx * dx + dy * dy);
    float t = dist / g.radius;
    t = t < 1.0f ? t : 1.0f;
    return make_float4(g.inner[0] + (g.outer[0] - g.inner[0]) * t, g.inner[1] + (g.outer[1] - g.inner[1]) * t,
                       g.inner[2] + (g.outer[2] - g.inner[2]) * t, g.inner[3] + (g.outer[3] - g.inner[3]) * t);
  }
  if (id >= in.n_uses) {
    status |= kStatusBadInput;
    return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  const gudni_picture_use u = in.uses[id];
  // a texel is read as one aligned 4-byte word: the picture's offset must be a
  // non-negative multiple of 4 (checked here as well as by the uploads, so that a
  // record written straight into device memory cannot misalign the read)
  if (u.mem_offset < 0 || (u.mem_offset & 3) != 0) {
    status |= kStatusBadInput;
    return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  float scale = u.scale < 1e-7f ? 1e-7f : u.scale;
  int rx = (int)(((float)px / scale) - u.translate_x);  // cvt.rzi: saturating, NaN -> 0
  int ry = (int)(((float)py / scale) - u.translate_y);
  if (rx >= 0 && ry >= 0 && rx < u.size_x && ry < u.size_y) {
    size_t o = (size_t)u.mem_offset + 4 * ((size_t)ry * (size_t)u.size_x + (size_t)rx);
    if (o + 4 > in.picture_bytes) {
      status |= kStatusBadInput;
      return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    uchar4 p = *reinterpret_cast<const uchar4*>(in.pictures + o);
    ++texels;
    return make_float4((float)p.x / 255.0f, (float)p.y / 255.0f, (float)p.z / 255.0f, (float)p.w / 255.0f);
  }
  return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// Whether a newly met substance with compound bits `comp` is composited
// (lastIsSet for a new substance, K:1496).
__device__ __forceinline__ bool lastIsSetFor(uint64_t comp) {
  return comp == GUDNI_TAG_ADD || comp == GUDNI_TAG_CONTINUE;
}

// determineColor K:1447-1513
//
// `stopBit` receives the lowest bit position the walk read: the colour is a function
// of the stack bits at and above it only (below it the walk had reached an opaque
// composite and stopped), or of every bit (-1) when it reached the background.
// How the colour walk finds the tag of a shape bit: through the column's table of
// shape indices (bit -> index into the job's shape pile, the per-column generation's
// numbering), or directly when the bits are the tile's own shape numbers (the
// warp-cooperative unit, whose tile records are staged in shared memory).
struct IndexedTags {
  const uint32_t* idx;
  const gudni_shape* shapes;
  __device__ __forceinline__ uint64_t tag(int bit) const { return shapes[idx[bit]].tag; }
};
struct DirectTags {
  const gudni_shape* shapes;  // the tile's shape records: bit n is record n
  __device__ __forceinline__ uint64_t tag(int bit) const { return shapes[bit].tag; }
};

template <int SECTIONS, class Tags>
__device__ __forceinline__ float4 determineColorT(const RasterInputs& in, const ShapeStack<SECTIONS>& stack,
                                                  const Tags& tags, int px, int py, int& status,
                                                 int64_t& texels, int topStart, bool& positional, int& stopBit) {
  // The reference starts at MAXSHAPE (K:1453); no bit at or above the column's
  // assigned shape-bit count is ever set, so starting there finds the same bits.
  int topBit = topStart;
  positional = false;
  float4 base = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float4 next = base;
  bool done = false;
  uint64_t lastId = ~0ull;
  bool lastIsContinue = true;
  bool lastIsSet = false;
  while (!done) {
    bool shouldComposite = true;
    topBit = stack.findTop(topBit);
    if (topBit < 0) {
      next = in.background;
      done = true;
      lastIsSet = true;
    } else {
      const uint64_t tag = tags.tag(topBit);
      const uint64_t sid = tag & GUDNI_TAG_ID_MASK;
      const uint64_t comp = tag & GUDNI_TAG_COMPOUND_MASK;
      if (sid == lastId) {
        if (lastIsContinue) {
          if (comp != GUDNI_TAG_CONTINUE) {
            lastIsSet = comp == GUDNI_TAG_ADD;
            lastIsContinue = false;
          } else {
            lastIsSet = !lastIsSet;
          }
        }
        shouldComposite = false;
      } else {
        const uint64_t type = tag & GUDNI_TAG_SUBSTANCE_MASK;
        next = readColor(in, px, py, sid, type, status, texels);
        positional = positional || (type != GUDNI_TAG_SOLID && lastIsSetFor(comp));
        lastIsSet = comp == GUDNI_TAG_ADD || comp == GUDNI_TAG_CONTINUE;
      }
      lastId = sid;
    }
    if (shouldComposite && lastIsSet) {
      base = composite(base, next);
      if (base.w == 1.0f) done = true;
    }
  }
  stopBit = topBit;
  return base;
}

template <int SECTIONS>
__device__ __forceinline__ float4 determineColor(const RasterInputs& in, const ShapeStack<SECTIONS>& stack,
                                                 const uint32_t* shapeIdx, int px, int py, int& status,
                                                 int64_t& texels, int topStart, bool& positional, int& stopBit) {
  return determineColorT<SECTIONS>(in, stack, IndexedTags{shapeIdx, in.shapes}, px, py, status, texels, topStart,
                                   positional, stopBit);
}

// Second-level memo for columns whose shape bits fit in one stack word: the last few
// (word, colour) pairs, exact -- the colour is a function of the word and, when a
// picture or gradient layer was composited, of the pixel row.
struct WordCache {
  static constexpr int N = 4;
  uint64_t key[N];
  float4 color[N];
  int stop[N];
  int row[N];  // -2 empty, -1 any row, else the pixel row
  int next;
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int e = 0; e < N; ++e) row[e] = -2;
    next = 0;
  }
  __device__ __forceinline__ int find(uint64_t k, int py) const {
#pragma unroll
    for (int e = 0; e < N; ++e)
      if (row[e] != -2 && key[e] == k && (row[e] == -1 || row[e] == py)) return e;
    return -1;
  }
  __device__ __forceinline__ void put(uint64_t k, int py, bool positional, float4 c, int stopBit) {
    const int e = next;
    next = (next + 1) & (N - 1);
    key[e] = k;
    color[e] = c;
    stop[e] = stopBit;
    row[e] = positional ? py : -1;
  }
};

struct Parse {
  int current, numActive;
  float sStartX, sStartY, sEndX, sEndY;
  float pixelY;
};

// The split of one active threshold at `slicePoint` (sliceActive K:1040-1067): the
// part above stays in place (returned through ch/cur), the part below is returned in
// sh/split.
__device__ __forceinline__ void splitAt(uint32_t& ch, float4& cur, float slicePoint, uint32_t& sh, float4& split) {
  const float splitX = intersectX(ch, cur, slicePoint);
  if (hPositive(ch)) {
    split = make_float4(slicePoint, cur.y, splitX, cur.w);
    cur = make_float4(cur.x, slicePoint, cur.z, splitX);
    sh = ch & kUnpersist;
  } else {
    split = make_float4(slicePoint, cur.y, cur.z, splitX);
    cur = make_float4(cur.x, slicePoint, splitX, cur.w);
    sh = ch;
    ch = ch & kUnpersist;
  }
}

// splitNext K:1069-1077 (countActive K:1007, nextSlicePoint K:1026, sliceActive K:1040)
//
// The reference inserts each kept lower part with insertThreshold, which walks from
// the queue front past every entry the part is strictly below -- all n active entries
// (their tops are below slicePoint, the part's top) and then the equal-top entries
// ahead of it.  Done literally that is n steps per part.  Here, when every active top
// compares below slicePoint and the slab has room, the parts are first collected below
// the queue, the active block is moved down by their number once, and each part is
// inserted into the rest of the queue by the same walk started past the active block:
// the resulting order is the reference's entry for entry.  Otherwise the literal
// insertion runs.
__device__ __forceinline__ float splitNext(Queue& q, Parse& p) {
  const int len = q.length();
  float slicePoint = FLT_MAX;
  const float top = q.get(0).x;
  int n = 1;
  while (n < len) {
    float t = q.get(n).x;
    if (t > top) {
      slicePoint = t;
      break;
    }
    n += 1;
  }
  p.numActive = n;
  float sp = slicePoint;
  for (int i = 0; i < n; ++i) {
    float bottom = q.get(i).y;
    if (top < bottom) sp = cl_min(sp, bottom);
  }
  slicePoint = cl_min(slicePoint, sp);
  bool batched = q.start >= 2 * n;
  for (int i = 0; batched && i < n; ++i) batched = q.get(i).x < slicePoint;
  if (!batched) {
    for (int cursor = 0; cursor < n; ++cursor) {
      uint32_t ch = q.getH(cursor);
      float4 cur = q.get(cursor);
      if (cur.x < slicePoint && slicePoint < cur.y) {
        uint32_t sh;
        float4 split;
        splitAt(ch, cur, slicePoint, sh, split);
        q.setH(cursor, ch);
        q.set(cursor, cur);
        if (tKeep(sh, split)) {
          q.insert(sh, split);
          if (q.overflow) return slicePoint;
        }
      }
    }
    return slicePoint;
  }
  // split in place, parts to [start - n - m, start - n), part j at start - n - 1 - j
  const int s0 = q.start;
  int m = 0;
  for (int cursor = 0; cursor < n; ++cursor) {
    uint32_t ch = q.hdr[s0 + cursor];
    float4 cur = q.thr[s0 + cursor];
    if (cur.x < slicePoint && slicePoint < cur.y) {
      uint32_t sh;
      float4 split;
      splitAt(ch, cur, slicePoint, sh, split);
      q.hdr[s0 + cursor] = ch;
      q.thr[s0 + cursor] = cur;
      if (tKeep(sh, split)) {
        q.hdr[s0 - n - 1 - m] = sh;
        q.thr[s0 - n - 1 - m] = split;
        ++m;
      }
    }
  }
  if (m == 0) return slicePoint;
  // Many parts: when no key involved is NaN the comparator is a strict weak order, so
  // inserting the parts one by one equals sorting them (ties: the later part first)
  // and merging them ahead of equal keys into the sorted rest of the queue.
  bool merge = m >= 8 && s0 >= n + 2 * m;
  for (int j = 0; merge && j < m; ++j) {
    const uint32_t h = q.hdr[s0 - n - 1 - j];
    const float4 t = q.thr[s0 - n - 1 - j];
    const float tx = tTopX(h, t), sl = invSlope(h, t);
    merge = tx == tx && sl == sl;
  }
  int rEnd = s0 + n;  // end of the equal-top group at the front of the rest
  while (merge && rEnd < q.cap && q.thr[rEnd].x == slicePoint) {
    const float tx = tTopX(q.hdr[rEnd], q.thr[rEnd]), sl = invSlope(q.hdr[rEnd], q.thr[rEnd]);
    merge = tx == tx && sl == sl;
    ++rEnd;
  }
  if (merge && rEnd < q.cap) merge = q.thr[rEnd].x > slicePoint;
  // the active block moves down by m (destinations below sources; the parts lie below
  // the block's new place since m <= n)
  for (int i = 0; i < n; ++i) {
    q.hdr[s0 - m + i] = q.hdr[s0 + i];
    q.thr[s0 - m + i] = q.thr[s0 + i];
  }
  q.start = s0 - m;
  if (merge) {
    // stable bottom-up merge sort of the parts, stored newest first at [lo, lo + m),
    // through [lo - m, lo)
    const int lo = s0 - n - m;
    int src = lo, dst = lo - m;
    for (int width = 1; width < m; width *= 2) {
      for (int a0 = 0; a0 < m; a0 += 2 * width) {
        const int mid = min(a0 + width, m), hi = min(a0 + 2 * width, m);
        int a = a0, b = mid, o = a0;
        while (a < mid && b < hi) {
          if (isBelow(q.hdr[src + a], q.thr[src + a], q.hdr[src + b], q.thr[src + b])) {
            q.hdr[dst + o] = q.hdr[src + b];
            q.thr[dst + o] = q.thr[src + b];
            ++b;
          } else {
            q.hdr[dst + o] = q.hdr[src + a];
            q.thr[dst + o] = q.thr[src + a];
            ++a;
          }
          ++o;
        }
        for (; a < mid; ++a, ++o) {
          q.hdr[dst + o] = q.hdr[src + a];
          q.thr[dst + o] = q.thr[src + a];
        }
        for (; b < hi; ++b, ++o) {
          q.hdr[dst + o] = q.hdr[src + b];
          q.thr[dst + o] = q.thr[src + b];
        }
      }
      const int t = src;
      src = dst;
      dst = t;
    }
    // merge into the gap ahead of the rest: a rest entry goes first only when the part
    // is strictly below it (writes never pass the rest's read position)
    int o = s0 - m + n, r = s0 + n;
    for (int j = 0; j < m; ++o) {
      const uint32_t ph = q.hdr[src + j];
      const float4 pt = q.thr[src + j];
      if (r < q.cap && isBelow(ph, pt, q.hdr[r], q.thr[r])) {
        q.hdr[o] = q.hdr[r];
        q.thr[o] = q.thr[r];
        ++r;
      } else {
        q.hdr[o] = ph;
        q.thr[o] = pt;
        ++j;
      }
    }
    return slicePoint;
  }
  // insert the parts in order into the queue past the active block
  int f = s0 + n;
  for (int j = 0; j < m; ++j) {
    const uint32_t h = q.hdr[s0 - n - 1 - j];
    const float4 t = q.thr[s0 - n - 1 - j];
    f -= 1;
    int at = f;
    while (at + 1 < q.cap) {
      const uint32_t oh = q.hdr[at + 1];
      const float4 o = q.thr[at + 1];
      if (!isBelow(h, t, oh, o)) break;
      q.hdr[at] = oh;
      q.thr[at] = o;
      at += 1;
    }
    q.hdr[at] = h;
    q.thr[at] = t;
  }
  return slicePoint;
}

// verticalAdvance K:1744-1824
template <int SECTIONS>
__device__ __forceinline__ void verticalAdvance(Queue& q, const ColumnState& c, Parse& p,
                                                ShapeStack<SECTIONS>& stack) {
  if (p.sEndX != kRight) return;
  for (int i = 0; i < p.numActive; ++i) stack.pass(q.getH(i));
  const float nextBreak = cl_min(c.floatHeight, p.pixelY);
  const float activeBottom = q.length() > 0 ? q.get(0).y : FLT_MAX;
  if (activeBottom == p.sEndY) {
    while (p.numActive > 0) {
      stack.passBottom(q.getH(0));
      q.pop();
      p.numActive -= 1;
    }
  }
  float nextBottom;
  if (p.numActive > 0) {
    nextBottom = cl_min(activeBottom, nextBreak);
  } else {
    const float nextTop = p.numActive < q.length() ? q.get(p.numActive).x : FLT_MAX;
    if (nextTop > p.sEndY) {
      nextBottom = cl_min(nextBreak, nextTop);
    } else {
      nextBottom = cl_min(nextBreak, splitNext(q, p));
      while (p.numActive > 0 && q.get(0).x == q.get(0).y) {
        stack.passTop(q.getH(0));
        q.pop();
        p.numActive -= 1;
      }
      for (int i = 0; i < p.numActive; ++i) {
        if (q.get(i).x > 0.0f) stack.passTop(q.getH(i));
      }
    }
  }
  p.sStartY = p.sEndY;
  p.sEndY = nextBottom;
  p.sStartX = p.sEndX = kLeft;
  p.current = 0;
}

// convert_uchar of colour * 255: round toward zero, clamp to [0,255], NaN -> 0
__device__ __forceinline__ uint32_t toByte(float v) {
  if (!(v > 0.0f)) return 0u;
  if (v >= 255.0f) return 255u;
  return (uint32_t)(int)v;
}

// renderThresholdArray K:1978-2028 (calculatePixel K:1881-1916, horizontalAdvance
// K:1826-1851, sectionColor K:1724-1742, writePixelGlobal K:1853-1862).
// `image` (optional): instead of the BGRA word, write each pixel's colour before the
// byte conversion and its section-area sum as a float4 (the adjoint's forward pass).
// `stage` (optional): write the BGRA word of the column's row r to stage[32 * r]
// instead of the output (the cooperative unit's shared-memory tile).
// kCounterJitter: take the stochastic jitter from counterRandom (kRandomCounter) in
// place of the random field; the default instantiation is the reference's scan.
template <int SECTIONS, bool kCounterJitter, class Tags>
__device__ __forceinline__ void renderColumnT(const RasterInputs& in, const ColumnState& c, Queue& q,
                                              ShapeStack<SECTIONS>& stack, const Tags& tags, int& status,
                                              int shapeBits, float4* image, uint32_t* stage) {
  Parse p;
  p.current = 0;
  p.numActive = 0;
  p.sStartX = kLeft;
  p.sStartY = 0.0f;
  p.sEndX = kRight;
  p.sEndY = 0.0f;
  int cursor = 0;  // the random field cursor, or the column's section ordinal (kCounterJitter)
  if (!kCounterJitter && in.stochastic != 0.0f && in.random_field) {  // initRandomField K:1597-1606
    cursor = (int)(__float_as_uint(in.random_field[c.threadUnique & (GUDNI_RANDOM_FIELD_SIZE - 1)]) &
                   (GUDNI_RANDOM_FIELD_SIZE - 1));
  }
  const int px = c.deltaX;
  int py = c.deltaY;
  uint32_t* outp = image ? nullptr : in.out + (size_t)c.deltaY * (size_t)in.bitmap_w + (size_t)c.deltaX;
  int64_t sections = 0;
  int64_t texels = 0;
  // Section-colour memo, exact: determineColor reads the stack bits from the top
  // down to `colorStop` and nothing below, so its result holds until a bit at or
  // above colorStop flips (stack.hiFlip), or, when a picture or gradient layer was
  // composited, until the pixel row changes.
  float4 color = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  bool colorOk = false;
  bool colorPositional = false;
  int colorStop = 0;
  WordCache words;
  words.clear();
  const bool oneWord = shapeBits <= 64;
  // The reference's two loops -- pixel rows (renderThresholdArray) and the sections of
  // a row (calculatePixel) -- run as one loop whose step is either the next section of
  // the row or, once the row is complete, its pixel.  Per column the operations and
  // their order are the reference's; across the lanes of a warp a lane whose row is
  // short goes on to its next row instead of waiting for the warp's longest row.
  p.pixelY = 1.0f;
  float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f, acc4 = 0.0f;
  int guard = 0;
  while (p.pixelY <= c.floatHeight) {
    if ((p.sEndX < kRight) || (p.sEndY < p.pixelY)) {
      if (++guard > kSectionCap) {
        status |= kStatusIterLimit;
        return;
      }
      verticalAdvance(q, c, p, stack);
      if (q.overflow) return;
      // horizontalAdvance
      float nextX = kRight;
      if (p.current < p.numActive) {
        const float4 t = q.get(p.current);
        const uint32_t h = q.getH(p.current);
        const float yMid = p.sStartY + ((p.sEndY - p.sStartY) * 0.5f);
        const float x = intersectX(h, t, yMid);
        nextX = x >= kRight ? kLeft : cl_max(kLeft, x);  // thresholdMidXLow K:916-926
      }
      p.sStartX = p.sEndX;
      p.sEndX = nextX;
      if (!colorOk || stack.hiFlip >= colorStop) {
        const int e = oneWord ? words.find(stack.word(0), py) : -1;
        if (e >= 0) {
          color = words.color[e];
          colorStop = words.stop[e];
          colorPositional = words.row[e] >= 0;
        } else {
          color = determineColorT<SECTIONS>(in, stack, tags, px, py, status, texels, shapeBits, colorPositional,
                                            colorStop);
          if (oneWord) words.put(stack.word(0), py, colorPositional, color, colorStop);
        }
        colorOk = true;
        stack.clearFlips();
      }
      float area = (p.sEndX - p.sStartX) * (p.sEndY - p.sStartY);
      if (in.stochastic != 0.0f) {  // getRandom K:1608-1613
        float random;
        if (kCounterJitter) {
          random = counterRandom(in.random_seed, px, py, (uint32_t)cursor);
          cursor += 1;
        } else {
          cursor = (cursor + 1) & (GUDNI_RANDOM_FIELD_SIZE - 1);
          random = in.random_field ? in.random_field[cursor] : 0.0f;
        }
        area = area + (area * random * in.stochastic);
      }
      acc0 += color.x * area;
      acc1 += color.y * area;
      acc2 += color.z * area;
      acc4 += area;
      if (p.current < p.numActive) stack.pass(q.getH(p.current));
      p.current += 1;
      ++sections;
    } else {
      // the row is complete: its pixel (writePixelGlobal K:1853-1862), then the next row
      const float r = acc0 / acc4, g = acc1 / acc4, b = acc2 / acc4;
      if (image) {
        image[(size_t)py * (size_t)in.bitmap_w + (size_t)px] = make_float4(r, g, b, acc4);
      } else if (stage) {
        stage[32 * (py - c.deltaY)] =
            toByte(b * 255.0f) | (toByte(g * 255.0f) << 8) | (toByte(r * 255.0f) << 16) | (255u << 24);
      } else {
        *outp = toByte(b * 255.0f) | (toByte(g * 255.0f) << 8) | (toByte(r * 255.0f) << 16) | (255u << 24);
        outp += in.bitmap_w;
      }
      p.sStartX = kLeft;
      p.sStartY = p.pixelY;
      py += 1;
      p.pixelY += 1.0f;
      acc0 = acc1 = acc2 = acc4 = 0.0f;
      guard = 0;
      if (colorPositional) colorOk = false;
    }
  }
  if (in.counters) {
    atomicAdd(reinterpret_cast<unsigned long long*>(&in.counters[0]), (unsigned long long)sections);
    atomicAdd(reinterpret_cast<unsigned long long*>(&in.counters[1]), (unsigned long long)texels);
  }
}

template <int SECTIONS, bool kCounterJitter = false>
__device__ __forceinline__ void renderColumn(const RasterInputs& in, const ColumnState& c, Queue& q,
                                             ShapeStack<SECTIONS>& stack, const uint32_t* shapeIdx, int& status,
                                             int shapeBits, float4* image = nullptr, uint32_t* stage = nullptr) {
  renderColumnT<SECTIONS, kCounterJitter>(in, c, q, stack, IndexedTags{shapeIdx, in.shapes}, status, shapeBits,
                                          image, stage);
}

// One column, start to finish.  Returns true when the queue overflowed `cap`.
template <int SECTIONS, bool kCounterJitter = false>
__device__ __forceinline__ bool runColumn(const RasterInputs& in, const gudni_tile_info& ti, int column,
                                          float4* thr, uint32_t* hdr, int cap, uint32_t* idx, int& status) {
  const ColumnState c = initColumn(in, ti, column, in.job_index);
  if (!c.active) return false;
  Queue q{thr, hdr, cap, cap, false};
  ShapeStack<SECTIONS> stack;
  stack.clear();
  // a tile of at most 64 shapes (and no more than max_shape): its shape numbers are
  // the bits, one stack word holds them, and the colour walk reads each tag from the
  // tile's records, which the warp's lanes share, instead of through the per-lane
  // index
  const bool direct = c.numShapes <= 64 && c.numShapes <= in.max_shape;
  const uint32_t bits = buildThresholds<SECTIONS>(in, c, q, stack, idx, status, direct);
  if (q.overflow) return true;
  sortQueue(q);
  if (in.counters) {
    atomicAdd(reinterpret_cast<unsigned long long*>(&in.counters[2]), (unsigned long long)q.length());
    atomicMax(reinterpret_cast<unsigned long long*>(&in.counters[3]), (unsigned long long)bits);
  }
  if (direct) {
    ShapeStack<1> one;
    one.clear();
    one.w[0] = stack.word(0);
    one.nz = one.w[0] ? 1u : 0u;
    renderColumnT<1, kCounterJitter>(in, c, q, one, DirectTags{in.shapes + c.shapeStart}, status, c.numShapes,
                                     nullptr, nullptr);
  } else if (SECTIONS > 1 && bits <= 64) {
    // every shape bit of the column sits in the first stack word: scan with a
    // one-word stack (flips and findTop on a single register)
    ShapeStack<1> one;
    one.clear();
    one.w[0] = stack.word(0);
    one.nz = one.w[0] ? 1u : 0u;
    renderColumn<1, kCounterJitter>(in, c, q, one, idx, status, (int)bits);
  } else {
    renderColumn<SECTIONS, kCounterJitter>(in, c, q, stack, idx, status, (int)bits);
  }
  return q.overflow;
}

}  // namespace gudni
