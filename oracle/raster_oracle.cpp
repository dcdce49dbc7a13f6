// ORACLE -- test infrastructure only.
//
// A CPU restatement of gudni's OpenCL raster kernels (src/Graphics/Gudni/OpenCL/
// Kernels.cl lines 43-2167; debug printers at 2169-2552 are left out).  It exists to
// check the CUDA path: only tests, the package's smoke() and bench.py's CPU-baseline
// leg may load it, and never as the thing measured or shipped.
//
// Pinning: the reference has no golden vectors.  This restatement is pinned against
// the reference's own Kernels.cl compiled for the CPU (oracle/build_ref.py writes
// oracle/_ref/), bit-exact on the committed fixture scenes.
//
// Arithmetic: IEEE single precision, no contraction (-ffp-contract=off), OpenCL
// min/max select semantics, float->int conversions round toward zero.  The
// float->uchar conversion of the final colour (convert_uchar4, which OpenCL leaves
// undefined outside [0,255]) clamps to [0,255] with NaN -> 0.
//
// One work item = one (tile, column) pair, exactly as the reference's NDRange
// (Work2D numTiles threadsPerTile); work items run as OpenMP loop iterations.

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/gudni_cuda.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------------ vectors
struct f2 { float x, y; };
struct f4 { float x, y, z, w; };  // THRESHOLD: top, bottom, left, right

inline f2 sub2(f2 a, f2 b) { return f2{a.x - b.x, a.y - b.y}; }
inline float cl_min(float x, float y) { return y < x ? y : x; }  // OpenCL min
inline float cl_max(float x, float y) { return x < y ? y : x; }  // OpenCL max
inline int cl_imin(int x, int y) { return y < x ? y : x; }
// OpenCL fmin/fmax: the select above, except that a NaN argument yields the other.
inline float cl_fmin(float x, float y) { return std::isnan(y) ? x : (std::isnan(x) ? y : cl_min(x, y)); }
inline float cl_fmax(float x, float y) { return std::isnan(y) ? x : (std::isnan(x) ? y : cl_max(x, y)); }
// convert_int (round toward zero); out of range saturates and NaN gives 0, as the
// GPU's cvt.rzi does.
inline int to_int_rtz(float v) {
  if (std::isnan(v)) return 0;
  if (v >= 2147483647.0f) return 2147483647;
  if (v <= -2147483648.0f) return (-2147483647 - 1);
  return (int)v;
}
inline int cl_imax(int x, int y) { return x < y ? y : x; }

constexpr float MINCROP = 0.2f;           // K:47
constexpr float LEFTBORDER = 0.0f;        // K:90
constexpr float RIGHTBORDER = 1.0f;       // K:91
constexpr float TAXICAB_FLATNESS = 0.25f; // K:250
constexpr float T_HALF = 0.5f;            // K:249
constexpr float VERTICALSLOPE = FLT_MAX;  // K:216
constexpr int LARGE_PRIME = 7919;         // K:83

// Header bits, K:168-185
constexpr uint32_t POSITIVE_SLOPE = 0x80000000u;
constexpr uint32_t PERSIST_AND_SLOPE_MASK = 0xC0000000u;
constexpr uint32_t PERSIST_TOP = 0xC0000000u;
constexpr uint32_t PERSIST_BOTTOM = 0x40000000u;
constexpr uint32_t PERSIST = 0x40000000u;
constexpr uint32_t UNPERSISTMASK = 0xBFFFFFFFu;
constexpr uint32_t SHAPEBIT_MASK = 0x0FFFFFFFu;

inline bool hPositive(uint32_t h) { return (h & POSITIVE_SLOPE) != 0; }
inline bool hPersistTop(uint32_t h) { return (h & PERSIST_AND_SLOPE_MASK) == PERSIST_TOP; }
inline bool hPersistBottom(uint32_t h) { return (h & PERSIST_AND_SLOPE_MASK) == PERSIST_BOTTOM; }
inline bool hPersistEither(uint32_t h) { return (h & PERSIST) != 0; }
inline uint32_t hShapeBit(uint32_t h) { return h & SHAPEBIT_MASK; }
inline uint32_t unPersist(uint32_t h) { return h & UNPERSISTMASK; }

inline float tTop(f4 t) { return t.x; }
inline float tBottom(f4 t) { return t.y; }
inline float tLeft(f4 t) { return t.z; }
inline float tRight(f4 t) { return t.w; }
inline f2 tStart(uint32_t h, f4 t) { return f2{t.z, hPositive(h) ? t.x : t.y}; }  // K:226
inline float tTopX(uint32_t h, f4 t) { return hPositive(h) ? t.z : t.w; }         // K:228
inline bool tIsHorizontal(f4 t) { return t.x == t.y; }                            // K:232
inline bool tKeep(uint32_t h, f4 t) { return hPersistEither(h) || (t.y - t.x >= MINCROP); }

// K:240-246
inline float invertedSlope(uint32_t h, f4 t) {
  float sign = hPositive(h) ? 1.0f : -1.0f;
  return tIsHorizontal(t) ? VERTICALSLOPE : (t.w - t.z) / (t.y - t.x) * sign;
}

// K:900-913
inline float intersectX(uint32_t h, f4 t, float y) {
  if (t.z == t.w) return t.z;
  f2 e = tStart(h, t);
  return ((y - e.y) * invertedSlope(h, t)) + e.x;  // xInterceptInvertedSlope K:832-834
}

// K:916-926
inline float midXLow(f4 t, uint32_t h, float yTop, float yBottom, float clampLow, float clampHigh) {
  float yMid = yTop + ((yBottom - yTop) * 0.5f);
  float x = intersectX(h, t, yMid);
  return x >= clampHigh ? clampLow : cl_max(clampLow, x);
}

// K:1079-1094 (also the sort comparator at K:1940-1951)
inline bool isBelow(uint32_t ah, f4 a, uint32_t bh, f4 b) {
  return (a.x > b.x) ||
         ((a.x == b.x) && ((tTopX(ah, a) > tTopX(bh, b)) ||
                           ((tTopX(ah, a) == tTopX(bh, b)) &&
                            (invertedSlope(ah, a) > invertedSlope(bh, b)))));
}

// ------------------------------------------------------------------ queue
// K:369-411, K:1096-1124.  Entries occupy [start, start+length) of a column slab of
// `cap` slots; pushes grow toward index 0.
struct Queue {
  f4* thr;
  uint32_t* hdr;
  int start, length, cap;
  bool overflow;
  int minStart;
  f4 get(int i) const { return thr[start + i]; }
  uint32_t getH(int i) const { return hdr[start + i]; }
  void set(int i, f4 t) { thr[start + i] = t; }
  void setH(int i, uint32_t h) { hdr[start + i] = h; }
  bool pushTopSlot() {
    if (start == 0) { overflow = true; return false; }  // the reference writes out of its slab here
    start -= 1;
    length += 1;
    if (start < minStart) minStart = start;
    return true;
  }
  void popTop() { start += 1; length -= 1; }
  void push(uint32_t h, f4 t) {  // pushThreshold K:1096-1103
    if (!pushTopSlot()) return;
    setH(0, h);
    set(0, t);
  }
  void insert(uint32_t h, f4 t) {  // insertThreshold K:1105-1124
    if (!pushTopSlot()) return;
    int cursor = 0;
    bool below = true;
    while (cursor < length - 1 && below) {
      uint32_t oh = getH(cursor + 1);
      f4 o = get(cursor + 1);
      below = isBelow(h, t, oh, o);
      if (below) {
        setH(cursor, oh);
        set(cursor, o);
        cursor += 1;
      }
    }
    setH(cursor, h);
    set(cursor, t);
  }
};

// ------------------------------------------------------------------ shape state
struct ShapeState {  // K:417-421
  uint32_t shapeBits;
  uint64_t* indices;   // MAXSHAPE entries
  uint64_t* stack;     // SHAPESTACKSECTIONS words
  int sections;
};

inline void flipBit(ShapeState& s, uint32_t bit) {  // K:298-304
  s.stack[bit >> 6] ^= (1ULL << (bit & 63));
}
inline void passHeader(ShapeState& s, uint32_t h) { flipBit(s, hShapeBit(h)); }
inline void passHeaderTop(ShapeState& s, uint32_t h) { if (hPersistTop(h)) passHeader(s, h); }
inline void passHeaderBottom(ShapeState& s, uint32_t h) { if (hPersistBottom(h)) passHeader(s, h); }

inline int clz64(uint64_t v) { return v == 0 ? 64 : __builtin_clzll(v); }

// findTop K:281-292
inline int findTop(const uint64_t* stack, int ignoreAbove) {
  int sec = ignoreAbove >> 6;
  int bits = ignoreAbove & 63;
  uint64_t section = bits >= 64 ? stack[sec] : (~(~0ULL << bits)) & stack[sec];
  while (section == 0 && sec > 0) {
    sec -= 1;
    section = stack[sec];
  }
  return (sec << 6) + (64 - clz64(section)) - 1;
}

// ------------------------------------------------------------------ tile state
struct TileState {  // K:438-451
  uint32_t shapeStart;
  int numShapes;
  int threadId;
  int tileW, tileH;
  int bitmapW, bitmapH;
  int internalX, internalY;
  int deltaX, deltaY;
  int intHeight;
  float floatHeight;
  int threadUnique;
};

// initTileState K:1692-1718
void initTileState(TileState& ts, const gudni_tile_info& ti, int bw, int bh, int column, int jobIndex,
                   int computeDepth) {
  ts.shapeStart = ti.shapes.start;
  ts.numShapes = (int)ti.shapes.length;
  ts.bitmapW = bw;
  ts.bitmapH = bh;
  ts.threadId = ti.column_allocation + column;
  int hDepth = ti.hdepth, vDepth = ti.vdepth;
  int diffDepth = cl_imax(0, vDepth - (computeDepth - hDepth));
  int desiredHeight = 1 << diffDepth;
  ts.internalX = ((1 << hDepth) - 1) & column;
  ts.internalY = (column >> hDepth) << diffDepth;
  ts.deltaX = ts.internalX + ti.left;
  ts.deltaY = ts.internalY + ti.top;
  ts.threadUnique = (ti.column_allocation + (1 << computeDepth) +
                     jobIndex * (1 << (computeDepth + computeDepth))) * LARGE_PRIME;
  ts.intHeight = cl_imin(desiredHeight, bh - ts.deltaY);
  ts.floatHeight = (float)ts.intHeight;
  ts.tileW = ti.right - ti.left;
  ts.tileH = ti.bottom - ti.top;
}

inline bool isActive(const TileState& ts) {  // K:1720-1722
  return ts.internalY < ts.tileH && ts.deltaX < ts.bitmapW && ts.deltaY < ts.bitmapH;
}

// ------------------------------------------------------------------ generate
struct Trav {  // K:453-458
  f2 left, control, right;
  float xPos;
  int index;
};

// bifurcateCurve K:1233-1258
void bifurcate(Trav& t) {
  if (!(t.left.x == t.control.x && t.left.y == t.control.y)) {
    for (;;) {
      f2 lm{(1 - T_HALF) * t.left.x + T_HALF * t.control.x, (1 - T_HALF) * t.left.y + T_HALF * t.control.y};
      f2 rm{(1 - T_HALF) * t.control.x + T_HALF * t.right.x, (1 - T_HALF) * t.control.y + T_HALF * t.right.y};
      f2 on{(1 - T_HALF) * lm.x + T_HALF * rm.x, (1 - T_HALF) * lm.y + T_HALF * rm.y};
      float flat = std::fabs(on.x - t.control.x) + std::fabs(on.y - t.control.y);
      if (flat > TAXICAB_FLATNESS) {
        if (t.xPos < on.x) {
          t.control = lm;
          t.right = on;
        } else {
          t.left = on;
          t.control = rm;
        }
      } else {
        break;
      }
    }
  }
}

// intersectCurve K:1226-1230
float intersectCurve(Trav t) {
  bifurcate(t);
  if (t.left.x == t.right.x) return cl_min(t.left.y, t.right.y);
  return (((t.right.y - t.left.y) / (t.right.x - t.left.x)) * (t.xPos - t.left.x)) + t.left.y;  // K:818-820
}

struct GenCtx {
  Queue* q;
  ShapeState* s;
  const TileState* ts;
};

// addThreshold K:1175-1220 (with lineToThreshold/lineToHeader K:1131-1150)
void addLineSegment(GenCtx& g, f2 left, f2 right, uint32_t shapeBit, bool* added, bool* enclosed) {
  f4 t{cl_fmin(left.y, right.y), cl_fmax(left.y, right.y), left.x, right.x};
  bool positive = left.y <= right.y;
  bool notVertical = left.x != right.x;
  bool touchLeft = left.x == LEFTBORDER;
  uint32_t h = (positive ? POSITIVE_SLOPE : 0u) | ((notVertical && touchLeft) ? PERSIST : 0u) | shapeBit;
  if (tKeep(h, t)) {
    *enclosed = *enclosed || ((t.x <= 0.0f) && hPersistTop(h)) || ((t.y <= 0.0f) && hPersistBottom(h));
    if ((t.x < g.ts->floatHeight) && (t.y > 0.0f) && t.z < RIGHTBORDER) {
      if (t.x <= 0.0f) {  // trimThresholdTop K:982-1005
        float splitX = intersectX(h, t, 0.0f);
        if (hPositive(h)) {
          t = f4{0.0f, t.y, splitX, t.w};
          h = unPersist(h);
        } else {
          t = f4{0.0f, t.y, t.z, splitX};
        }
      }
      if (t.w <= LEFTBORDER) {
        *enclosed = true;
      } else {
        *added = true;
        g.q->push(h, t);
      }
    }
  }
}

// spawnThresholds K:1264-1333
void spawnThresholds(GenCtx& g, uint32_t shapeBit, Trav& l, Trav& r, bool* added, bool* enclosed) {
  float yL = (l.left.x >= LEFTBORDER) ? l.left.y : intersectCurve(l);
  bool leftWing = false;
  if ((l.right.x < RIGHTBORDER) && (l.right.x > LEFTBORDER)) {
    addLineSegment(g, f2{l.xPos, yL}, l.right, shapeBit, added, enclosed);
    leftWing = true;
  }
  float yR = (r.right.x <= RIGHTBORDER) ? r.right.y : intersectCurve(r);
  bool rightWing = false;
  if ((r.left.x > LEFTBORDER) && (r.left.x < RIGHTBORDER) && (l.index != r.index)) {
    addLineSegment(g, r.left, f2{r.xPos, yR}, shapeBit, added, enclosed);
    rightWing = true;
  }
  if (l.right.x < r.left.x || (!leftWing && !rightWing)) {
    f2 bl = (leftWing || (l.left.x == l.right.x)) ? l.right : f2{l.xPos, yL};
    f2 br = (rightWing || (r.left.x == r.right.x)) ? r.left : f2{r.xPos, yR};
    addLineSegment(g, bl, br, shapeBit, added, enclosed);
  }
}

// searchTree K:1337-1357
void searchTree(Trav& t, const float* tree, int treeSize, f2 d, bool isLeft) {
  t.index = 0;
  while (t.index < treeSize) {
    const float* n = tree + 4 * t.index;
    float cx = n[0] - d.x, cy = n[1] - d.y, kx = n[2] - d.x, ky = n[3] - d.y;
    if ((t.xPos < cx) || (isLeft && t.xPos == cx)) {
      t.right = f2{cx, cy};
      t.index = (t.index << 1) + 1;
    } else {
      t.left = f2{cx, cy};
      t.control = f2{kx, ky};
      t.index = (t.index << 1) + 2;
    }
  }
}

// buildThresholdArray K:1540-1595 (traverseTree K:1378-1408 inlined)
void buildThresholdArray(GenCtx& g, const uint8_t* geo, const gudni_shape* shapes, int maxShape) {
  const TileState& ts = *g.ts;
  ShapeState& s = *g.s;
  const f2 d{(float)ts.deltaX, (float)ts.deltaY};
  for (int n = 0; n < ts.numShapes && (int)s.shapeBits < maxShape; ++n) {
    uint32_t shapeIndex = ts.shapeStart + (uint32_t)n;
    bool added = false;
    const gudni_shape& shape = shapes[shapeIndex];
    const float* strand = reinterpret_cast<const float*>(geo + (size_t)shape.geo_start * 16);
    bool enclosedByShape = false;
    for (uint32_t k = 0; k < shape.num_strands; ++k) {
      uint16_t size;
      std::memcpy(&size, strand, 2);
      bool enclosedByStrand = false;
      int treeSize = ((int)size - 4) / 2;
      Trav l, r;
      l.right = f2{strand[2] - d.x, strand[3] - d.y};
      l.left = f2{strand[4] - d.x, strand[5] - d.y};
      l.control = f2{strand[6] - d.x, strand[7] - d.y};
      l.xPos = 0.0f;
      l.index = 0;
      const float* tree = strand + 8;
      if (l.left.x <= RIGHTBORDER && l.right.x > LEFTBORDER) {  // checkInRange K:1360-1363
        r = l;
        l.xPos = cl_max(LEFTBORDER, l.left.x);
        r.xPos = cl_min(RIGHTBORDER, l.right.x);
        searchTree(l, tree, treeSize, d, true);
        searchTree(r, tree, treeSize, d, false);
        spawnThresholds(g, s.shapeBits, l, r, &added, &enclosedByStrand);
      }
      strand += 2 * (int)size;  // size counts 8-byte units
      enclosedByShape = enclosedByShape != enclosedByStrand;
    }
    if (enclosedByShape) flipBit(s, s.shapeBits);
    if (added || enclosedByShape) {
      if ((int)s.shapeBits < maxShape) s.indices[s.shapeBits] = shapeIndex;
      s.shapeBits += 1;
    }
  }
}

// sortThresholdArray K:1932-1976: the reference's bubble sort (kept as written; the
// comparator is a strict weak order, so the result is the stable sorted order).
void sortQueue(Queue& q) {
  bool done = false;
  int k = q.length;
  while (!done) {
    done = true;
    for (int i = 0; i < k - 1; ++i) {
      uint32_t ah = q.getH(i), bh = q.getH(i + 1);
      f4 a = q.get(i), b = q.get(i + 1);
      if (isBelow(ah, a, bh, b)) {
        q.setH(i, bh); q.set(i, b);
        q.setH(i + 1, ah); q.set(i + 1, a);
        done = false;
      }
    }
    k--;
  }
}

// ------------------------------------------------------------------ render
struct Common {
  const uint8_t* geo;
  const f4* substances;
  const uint8_t* pict;
  const gudni_picture_use* uses;
  const gudni_radial* radials;
  const float* random;
  const gudni_shape* shapes;
  f4 background;
  float stochastic;
  int random_mode;       // 0: the random field (K:1597-1613); 1: counter-based (below)
  uint64_t random_seed;
};

// Counter-based jitter (no counterpart in the reference, which only has the random
// field): the section with ordinal k in its column's scan, in pixel (x, y), takes the
// top 24 bits of SplitMix64's output function (Steele, Lea and Flood, OOPSLA 2014)
// applied twice, to seed ^ (x << 32 | y) and then to that plus k, as a float in
// [0, 1).
inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline float counterJitter(uint64_t seed, int x, int y, uint32_t k) {
  const uint64_t key = seed ^ (((uint64_t)(uint32_t)x << 32) | (uint64_t)(uint32_t)y);
  const uint64_t h = mix64(mix64(key) + (uint64_t)k);
  return (float)(uint32_t)(h >> 40) / 16777216.0f;
}

inline f4 composite(f4 fg, f4 bg) {  // K:878-887
  float alphaOut = fg.w + bg.w * (1.0f - fg.w);
  if (alphaOut > 0) {
    // (background * ALPHA(background)) * (1 - ALPHA(foreground)), left to right
    float k = 1.0f - fg.w;
    return f4{((fg.x * fg.w) + ((bg.x * bg.w) * k)) / alphaOut, ((fg.y * fg.w) + ((bg.y * bg.w) * k)) / alphaOut,
              ((fg.z * fg.w) + ((bg.z * bg.w) * k)) / alphaOut, alphaOut};
  }
  return f4{0, 0, 0, 0};
}

// readColor K:1411-1442, plus the radial-gradient substance (new, no reference
// counterpart): evaluated at the integer pixel position like a picture texel.
f4 readColor(const Common& c, int px, int py, uint64_t sid, uint64_t type) {
  f4 sub = c.substances[sid];
  if (type == GUDNI_TAG_SOLID) return sub;
  uint32_t id;
  std::memcpy(&id, &sub.x, 4);
  if (type == GUDNI_TAG_RADIAL) {
    const gudni_radial& g = c.radials[id];
    float dx = (float)px - g.center_x, dy = (float)py - g.center_y;
    float dist = std::sqrt(dx * dx + dy * dy);
    float t = dist / g.radius;
    t = t < 1.0f ? t : 1.0f;
    return f4{g.inner[0] + (g.outer[0] - g.inner[0]) * t, g.inner[1] + (g.outer[1] - g.inner[1]) * t,
              g.inner[2] + (g.outer[2] - g.inner[2]) * t, g.inner[3] + (g.outer[3] - g.inner[3]) * t};
  }
  const gudni_picture_use& u = c.uses[id];
  float scale = u.scale < 1e-7f ? 1e-7f : u.scale;
  // convert_int2 rounds toward zero
  int rx = to_int_rtz(((float)px / scale) - u.translate_x);
  int ry = to_int_rtz(((float)py / scale) - u.translate_y);
  if (rx >= 0 && ry >= 0 && rx < u.size_x && ry < u.size_y) {
    const uint8_t* p = c.pict + u.mem_offset + 4 * ((size_t)ry * u.size_x + rx);
    return f4{(float)p[0] / 255.0f, (float)p[1] / 255.0f, (float)p[2] / 255.0f, (float)p[3] / 255.0f};
  }
  return f4{0, 0, 0, 0};
}

// determineColor K:1447-1513
f4 determineColor(const Common& c, const ShapeState& s, int maxShape, int px, int py) {
  int topBit = maxShape;
  f4 base{0, 0, 0, 0};
  f4 next{0, 0, 0, 0};
  bool done = false;
  const uint64_t NULLID = ~0ULL;
  uint64_t lastId = NULLID;
  bool lastIsContinue = true;
  bool lastIsSet = false;
  while (!done) {
    bool shouldComposite = true;
    topBit = findTop(s.stack, topBit);
    if (topBit < 0) {
      next = c.background;
      done = true;
      shouldComposite = true;
      lastIsSet = true;
    } else {
      uint64_t ref = s.indices[topBit];
      uint64_t tag = c.shapes[ref].tag;
      uint64_t sid = tag & GUDNI_TAG_ID_MASK;
      uint64_t comp = tag & GUDNI_TAG_COMPOUND_MASK;
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
      }
      if (sid != lastId) {
        next = readColor(c, px, py, sid, tag & GUDNI_TAG_SUBSTANCE_MASK);
        shouldComposite = true;
        lastIsSet = comp == GUDNI_TAG_ADD || comp == GUDNI_TAG_CONTINUE;
      }
      lastId = sid;
    }
    if (shouldComposite && lastIsSet) {
      base = composite(base, next);
      if (base.w == 1.0f) done = true;
    }
  }
  return base;
}

struct Parse {  // K:423-436
  int current, numActive;
  f2 sStart, sEnd;
  float pixelY;
  float acc[8];
  int cursor;  // random field cursor
};

// splitNext K:1069-1077 with countActive/nextSlicePoint/sliceActive K:1007-1067
float splitNext(Queue& q, Parse& p) {
  float slicePoint = FLT_MAX;
  {
    float top = q.get(0).x;
    bool notDone = true;
    int n = 1;
    while (notDone && n < q.length) {
      f4 nx = q.get(n);
      if (nx.x > top) {
        notDone = false;
        slicePoint = nx.x;
      } else {
        n += 1;
      }
    }
    p.numActive = n;
  }
  {
    float top = q.get(0).x;
    float sp = slicePoint;
    for (int i = 0; i < p.numActive; ++i) {
      float bottom = q.get(i).y;
      if (top < bottom) sp = cl_min(sp, bottom);
    }
    slicePoint = cl_min(slicePoint, sp);
  }
  for (int cursor = 0; cursor < p.numActive; ++cursor) {
    uint32_t ch = q.getH(cursor);
    f4 cur = q.get(cursor);
    if (cur.x < slicePoint && slicePoint < cur.y) {
      // splitThreshold / divideThreshold K:928-979
      float splitX = intersectX(ch, cur, slicePoint);
      uint32_t sh;
      f4 split;
      if (hPositive(ch)) {
        split = f4{slicePoint, cur.y, splitX, cur.w};
        cur = f4{cur.x, slicePoint, cur.z, splitX};
        sh = unPersist(ch);
      } else {
        split = f4{slicePoint, cur.y, cur.z, splitX};
        cur = f4{cur.x, slicePoint, splitX, cur.w};
        sh = ch;
        ch = unPersist(ch);
      }
      q.setH(cursor, ch);
      q.set(cursor, cur);
      if (tKeep(sh, split)) q.insert(sh, split);
    }
  }
  return slicePoint;
}

// verticalAdvance K:1744-1824
void verticalAdvance(Queue& q, const TileState& ts, Parse& p, ShapeState& s) {
  if (p.sEnd.x != RIGHTBORDER) return;
  for (int i = 0; i < p.numActive; ++i) passHeader(s, q.getH(i));
  float nextBreak = cl_min(ts.floatHeight, p.pixelY);
  float activeBottom = q.length > 0 ? q.get(0).y : FLT_MAX;
  if (activeBottom == p.sEnd.y) {
    while (p.numActive > 0) {
      passHeaderBottom(s, q.getH(0));
      q.popTop();
      p.numActive -= 1;
    }
  }
  float nextBottom;
  if (p.numActive > 0) {
    nextBottom = cl_min(activeBottom, nextBreak);
  } else {
    float nextTop = p.numActive < q.length ? q.get(p.numActive).x : FLT_MAX;
    if (nextTop > p.sEnd.y) {
      nextBottom = cl_min(nextBreak, nextTop);
    } else {
      nextBottom = cl_min(nextBreak, splitNext(q, p));
      while (p.numActive > 0 && tIsHorizontal(q.get(0))) {
        passHeaderTop(s, q.getH(0));
        q.popTop();
        p.numActive -= 1;
      }
      for (int i = 0; i < p.numActive; ++i) {
        if (q.get(i).x > 0.0f) passHeaderTop(s, q.getH(i));
      }
    }
  }
  p.sStart.y = p.sEnd.y;
  p.sEnd.y = nextBottom;
  p.sStart.x = p.sEnd.x = LEFTBORDER;
  p.current = 0;
}

// horizontalAdvance K:1826-1851
void horizontalAdvance(Queue& q, Parse& p) {
  float nextX = (p.current < p.numActive)
                    ? midXLow(q.get(p.current), q.getH(p.current), p.sStart.y, p.sEnd.y, LEFTBORDER, RIGHTBORDER)
                    : RIGHTBORDER;
  p.sStart.x = p.sEnd.x;
  p.sEnd.x = nextX;
}

inline uint8_t toByte(float v) {  // convert_uchar (rtz); clamps outside [0,255], NaN -> 0
  if (!(v > 0.0f)) return 0;
  if (v >= 255.0f) return 255;
  return (uint8_t)(int)v;
}

struct Stats {
  int64_t maxQueue = 0;
  int64_t thresholds = 0;
  int64_t sections = 0;
  int64_t maxShapeBits = 0;
  int overflow = 0;
};

// one work item: generate -> sort -> render (K:2030-2167)
void runColumn(const Common& c, const gudni_tile_info* tiles, int tileIndex, int column, int bw, int bh,
               int computeDepth, int jobIndex, int maxT, int maxShape, int sections, uint32_t* out,
               std::vector<f4>& thrBuf, std::vector<uint32_t>& hdrBuf, std::vector<uint64_t>& idx,
               std::vector<uint64_t>& stack, Stats& st) {
  TileState ts;
  initTileState(ts, tiles[tileIndex], bw, bh, column, jobIndex, computeDepth);
  if (!isActive(ts)) return;
  Queue q{thrBuf.data(), hdrBuf.data(), maxT, 0, maxT, false, maxT};
  ShapeState s{0, idx.data(), stack.data(), sections};
  std::fill(stack.begin(), stack.end(), 0ULL);
  GenCtx g{&q, &s, &ts};
  buildThresholdArray(g, c.geo, c.shapes, maxShape);
  st.thresholds += q.length;
  st.maxQueue = std::max<int64_t>(st.maxQueue, q.length);
  st.maxShapeBits = std::max<int64_t>(st.maxShapeBits, s.shapeBits);
  sortQueue(q);

  // renderThresholdArray K:1978-2028
  Parse p;
  p.current = 0;
  p.numActive = 0;
  std::fill(p.acc, p.acc + 8, 0.0f);
  p.sStart = f2{LEFTBORDER, 0.0f};
  p.sEnd = f2{RIGHTBORDER, 0.0f};
  {
    int startIx = ts.threadUnique & (GUDNI_RANDOM_FIELD_SIZE - 1);  // initRandomField K:1597-1606
    uint32_t bits = 0;
    if (c.random) std::memcpy(&bits, &c.random[startIx], 4);
    p.cursor = c.random_mode == 1 ? 0 : (int)(bits & (GUDNI_RANDOM_FIELD_SIZE - 1));
  }
  int px = ts.deltaX, py = ts.deltaY;
  int yInt = -1;
  for (p.pixelY = 1.0f; p.pixelY <= ts.floatHeight; p.pixelY += 1.0f) {
    yInt += 1;
    // calculatePixel K:1881-1916
    while ((p.sEnd.x < RIGHTBORDER) || (p.sEnd.y < p.pixelY)) {
      verticalAdvance(q, ts, p, s);
      horizontalAdvance(q, p);
      f4 color = determineColor(c, s, maxShape, px, py);
      float random;
      if (c.random_mode == 1) {
        random = counterJitter(c.random_seed, px, py, (uint32_t)p.cursor);
        p.cursor += 1;
      } else {
        p.cursor = (p.cursor + 1) & (GUDNI_RANDOM_FIELD_SIZE - 1);  // getRandom K:1608-1613
        random = c.random ? c.random[p.cursor] : 0.0f;
      }
      float area = (p.sEnd.x - p.sStart.x) * (p.sEnd.y - p.sStart.y);
      float adj = area + (area * random * c.stochastic);
      p.acc[0] += color.x * adj;
      p.acc[1] += color.y * adj;
      p.acc[2] += color.z * adj;
      p.acc[3] += color.w * adj;
      p.acc[4] += adj;
      p.acc[5] += adj;
      p.acc[6] += adj;
      p.acc[7] += adj;
      if (p.current < p.numActive) passHeader(s, q.getH(p.current));
      p.current += 1;
      st.sections += 1;
    }
    float r = p.acc[0] / p.acc[4], gr = p.acc[1] / p.acc[5], b = p.acc[2] / p.acc[6];
    // colorToSolidPixel_Word32_BGRA K:842-844 (bytes B, G, R, 255 in memory order)
    uint32_t word = (uint32_t)toByte(b * 255.0f) | ((uint32_t)toByte(gr * 255.0f) << 8) |
                    ((uint32_t)toByte(r * 255.0f) << 16) | (255u << 24);
    out[(size_t)(ts.deltaY + yInt) * bw + ts.deltaX] = word;  // writePixelGlobal K:1853-1862
    std::fill(p.acc, p.acc + 8, 0.0f);
    p.sStart = f2{LEFTBORDER, p.pixelY};
    py += 1;
  }
  st.maxQueue = std::max<int64_t>(st.maxQueue, (int64_t)(maxT - q.minStart));
  if (q.overflow) st.overflow = 1;
}

}  // namespace

extern "C" {

// Counters returned by oracle_raster_job.
typedef struct oracle_stats {
  int64_t max_queue;      // largest per-column queue (generation or render time)
  int64_t thresholds;     // thresholds generated over all columns
  int64_t sections;       // sections scanned over all pixels
  int64_t max_shape_bits; // largest shape-bit count of a column
  int64_t overflow;       // 1 if a column overflowed max_thresholds
} oracle_stats;

static int g_random_mode = 0;
static uint64_t g_random_seed = 0;

// Source of the stochastic jitter for the following oracle_raster_job calls: 0 = the
// random field, 1 = the counter-based jitter with `seed`.
void oracle_set_random_source(int mode, uint64_t seed) {
  g_random_mode = mode;
  g_random_seed = seed;
}

// Rasterize one job on the CPU.  Arguments mirror gudni_raster_job plus the common
// buffers and the spec knobs; `out` is bitmap_w*bitmap_h BGRA words.
int oracle_raster_job(const uint8_t* geometry, const float* substances, const uint8_t* pictures,
                      const gudni_picture_use* picture_uses, const gudni_radial* radials,
                      const float* random_field, const gudni_shape* shapes, const gudni_tile_info* tiles,
                      int n_tiles, int threads_per_tile, int compute_depth, int bitmap_w, int bitmap_h,
                      int frame_number, int job_index, const float* background, int max_thresholds,
                      int max_shape, int stack_sections, float stochastic_factor, uint32_t* out,
                      int n_threads, oracle_stats* stats) {
  (void)frame_number;
  if (max_shape > 64 * stack_sections - 1 || max_thresholds <= 0 || threads_per_tile <= 0) return -1;
  Common c;
  c.geo = geometry;
  c.substances = reinterpret_cast<const f4*>(substances);
  c.pict = pictures;
  c.uses = picture_uses;
  c.radials = radials;
  c.random = random_field;
  c.shapes = shapes;
  c.background = f4{background[0], background[1], background[2], background[3]};
  c.stochastic = stochastic_factor;
  c.random_mode = g_random_mode;
  c.random_seed = g_random_seed;
  const long long total = (long long)n_tiles * threads_per_tile;
  Stats agg;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
#pragma omp parallel
  {
    std::vector<f4> thr(max_thresholds);
    std::vector<uint32_t> hdr(max_thresholds);
    std::vector<uint64_t> idx(max_shape > 0 ? max_shape : 1);
    std::vector<uint64_t> stack(stack_sections);
    Stats st;
#pragma omp for schedule(dynamic, 4)
    for (long long w = 0; w < total; ++w) {
      runColumn(c, tiles, (int)(w / threads_per_tile), (int)(w % threads_per_tile), bitmap_w, bitmap_h,
                compute_depth, job_index, max_thresholds, max_shape, stack_sections, out, thr, hdr, idx,
                stack, st);
    }
#pragma omp critical
    {
      agg.maxQueue = std::max(agg.maxQueue, st.maxQueue);
      agg.thresholds += st.thresholds;
      agg.sections += st.sections;
      agg.maxShapeBits = std::max(agg.maxShapeBits, st.maxShapeBits);
      agg.overflow |= st.overflow;
    }
  }
  if (stats) {
    stats->max_queue = agg.maxQueue;
    stats->thresholds = agg.thresholds;
    stats->sections = agg.sections;
    stats->max_shape_bits = agg.maxShapeBits;
    stats->overflow = agg.overflow;
  }
  return agg.overflow ? -2 : 0;
}

}  // extern "C"
