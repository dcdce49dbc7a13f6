// ORACLE -- test infrastructure only.
//
// FP64 host reference of the raster path's adjoint: the gradient of the per-pixel L2
// loss  L = sum_p sum_{c in RGB} (I_c(p) - T_c(p))^2  with respect to every point of
// the geometry pile and every solid substance colour, where I(p) = sum_s col_s a_s /
// sum_s a_s is the pixel's colour before the byte conversion (the reference's
// accumulation, Kernels.cl:1897-1904, 2017).
//
// The forward decisions are the reference kernels' own (the column machine of
// raster_oracle.cpp, restated here with provenance): every threshold remembers the
// line it lies on -- two end points, each either a strand point of the pile or the
// intercept of a de Casteljau sub-curve with a column border (Kernels.cl:1226-1333) --
// and every section y-bound remembers which line end point produced it.  The
// gradient then flows through the coverage integral's boundary terms:
//   a_s = (x1 - x0)(y1 - y0),  x = X_line((y0 + y1)/2)  (thresholdMidXLow, K:916-926),
// y-bounds from line end points (section splits, K:1007-1077), colours through the
// front-to-back composite chain (K:878-887, 1447-1513).  Discrete choices (which
// shapes cover a section, bifurcation branches, threshold keep/drop) are held fixed.
// All gradient arithmetic is double precision.

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

struct f2 { float x, y; };
struct f4 { float x, y, z, w; };

inline float cl_min(float x, float y) { return y < x ? y : x; }
inline float cl_max(float x, float y) { return x < y ? y : x; }
inline float cl_fmin(float x, float y) { return std::isnan(y) ? x : (std::isnan(x) ? y : cl_min(x, y)); }
inline float cl_fmax(float x, float y) { return std::isnan(y) ? x : (std::isnan(x) ? y : cl_max(x, y)); }

constexpr float MINCROP = 0.2f, LEFT = 0.0f, RIGHT = 1.0f, FLAT = 0.25f, HALF = 0.5f;
constexpr uint32_t POS = 0x80000000u, PSMASK = 0xC0000000u, PTOP = 0xC0000000u, PBOT = 0x40000000u,
                   PERSIST = 0x40000000u, UNPERSIST = 0xBFFFFFFFu, BITMASK = 0x0FFFFFFFu;

inline bool hPos(uint32_t h) { return (h & POS) != 0; }
inline bool hTop(uint32_t h) { return (h & PSMASK) == PTOP; }
inline bool hBot(uint32_t h) { return (h & PSMASK) == PBOT; }
inline bool tKeep(uint32_t h, f4 t) { return ((h & PERSIST) != 0) || (t.y - t.x >= MINCROP); }
inline float topX(uint32_t h, f4 t) { return hPos(h) ? t.z : t.w; }
inline float invSlope(uint32_t h, f4 t) {
  float sign = hPos(h) ? 1.0f : -1.0f;
  return (t.x == t.y) ? FLT_MAX : (t.w - t.z) / (t.y - t.x) * sign;
}
inline float intersectX(uint32_t h, f4 t, float y) {
  if (t.z == t.w) return t.z;
  float sy = hPos(h) ? t.x : t.y;
  return ((y - sy) * invSlope(h, t)) + t.z;
}
inline bool isBelow(uint32_t ah, f4 a, uint32_t bh, f4 b) {
  return (a.x > b.x) || ((a.x == b.x) && ((topX(ah, a) > topX(bh, b)) ||
                                          ((topX(ah, a) == topX(bh, b)) && (invSlope(ah, a) > invSlope(bh, b)))));
}

// ------------------------------------------------------------------ provenance
struct EP {          // line end point
  float x, y;        // tile-relative value
  int kind;          // 0: strand point; 1: intercept; 2: intercept, y = min of the sub-curve's ends
  int64_t pt;        // kind 0: float index of x in the pile
  int64_t xsrc;      // kinds 1-2: float index of the pile x that is xPos, or -1 (a border)
  int64_t q[3];      // kinds 1-2: float indices of P0, P1, P2
  double t0, t1;     // kinds 1-2: the sub-curve [t0, t1]
};
struct Line { EP a, b; double g[4]; };  // g: dL/d(xa, ya, xb, yb)

struct Entry {
  f4 t;
  uint32_t h;
  int32_t line;
  int64_t top, bot;  // y sources: line*2 + end (0 = a, 1 = b), or -1 (a constant)
};

struct Queue {
  std::vector<Entry>* e;
  int start, cap;
  bool overflow;
  int len() const { return cap - start; }
  Entry& at(int i) { return (*e)[start + i]; }
  void insert(const Entry& n) {
    if (start == 0) { overflow = true; return; }
    start -= 1;
    int cursor = 0;
    while (cursor < len() - 1) {
      Entry& o = (*e)[start + cursor + 1];
      if (!isBelow(n.h, n.t, o.h, o.t)) break;
      (*e)[start + cursor] = o;
      cursor += 1;
    }
    (*e)[start + cursor] = n;
  }
};

struct Trav {
  f2 left, control, right;
  float xPos;
  int index;
  int64_t oL, oC, oR;  // float indices of left, control, right in the pile
};

struct Col {
  int deltaX, deltaY, intHeight, internalY, tileH, numShapes;
  uint32_t shapeStart;
  float floatHeight;
  bool active;
};

struct Ctx {
  const uint8_t* geo;
  const f4* subs;
  uint32_t nSub;
  const uint8_t* pict;
  const gudni_picture_use* uses;
  const gudni_radial* radials;
  const gudni_shape* shapes;
  f4 background;
  int maxShape, bw, bh, log2tpt, cap;
};

// bifurcateCurve K:1233-1258, tracking the parameter interval of the sub-curve
void bifurcate(Trav& t, double& t0, double& t1) {
  t0 = 0.0;
  t1 = 1.0;
  if (t.left.x == t.control.x && t.left.y == t.control.y) return;
  for (int it = 0; it < 96; ++it) {
    f2 lm{(1 - HALF) * t.left.x + HALF * t.control.x, (1 - HALF) * t.left.y + HALF * t.control.y};
    f2 rm{(1 - HALF) * t.control.x + HALF * t.right.x, (1 - HALF) * t.control.y + HALF * t.right.y};
    f2 on{(1 - HALF) * lm.x + HALF * rm.x, (1 - HALF) * lm.y + HALF * rm.y};
    float flat = std::fabs(on.x - t.control.x) + std::fabs(on.y - t.control.y);
    if (!(flat > FLAT)) return;
    double mid = 0.5 * (t0 + t1);
    if (t.xPos < on.x) {
      t.control = lm;
      t.right = on;
      t1 = mid;
    } else {
      t.left = on;
      t.control = rm;
      t0 = mid;
    }
  }
}

// intersectCurve K:1226-1230 as an end point with provenance; xsrc is the pile x
// that xPos equals (or -1 for a border)
EP interceptEP(const Trav& l, int64_t xsrc) {
  Trav t = l;
  EP ep;
  ep.q[0] = l.oL;
  ep.q[1] = l.oC;
  ep.q[2] = l.oR;
  ep.xsrc = xsrc;
  bifurcate(t, ep.t0, ep.t1);
  ep.x = l.xPos;
  ep.pt = -1;
  if (t.left.x == t.right.x) {
    ep.kind = 2;
    ep.y = cl_min(t.left.y, t.right.y);
  } else {
    ep.kind = 1;
    ep.y = (((t.right.y - t.left.y) / (t.right.x - t.left.x)) * (t.xPos - t.left.x)) + t.left.y;
  }
  return ep;
}

EP pointEP(f2 p, float x, int64_t off) {
  EP ep;
  ep.x = x;
  ep.y = p.y;
  ep.kind = 0;
  ep.pt = off;
  ep.xsrc = -1;
  ep.q[0] = ep.q[1] = ep.q[2] = -1;
  ep.t0 = ep.t1 = 0.0;
  return ep;
}

struct Gen {
  Queue* q;
  std::vector<Line>* lines;
  const Col* c;
};

void addLine(Gen& g, const EP& A, const EP& B, uint32_t bit, bool& added, bool& enclosed) {
  f4 t{cl_fmin(A.y, B.y), cl_fmax(A.y, B.y), A.x, B.x};
  bool positive = A.y <= B.y;
  uint32_t h = (positive ? POS : 0u) | (((A.x != B.x) && (A.x == LEFT)) ? PERSIST : 0u) | bit;
  if (!tKeep(h, t)) return;
  enclosed = enclosed || ((t.x <= 0.0f) && hTop(h)) || ((t.y <= 0.0f) && hBot(h));
  if ((t.x < g.c->floatHeight) && (t.y > 0.0f) && t.z < RIGHT) {
    const int32_t id = (int32_t)g.lines->size();
    // y sources of the threshold's top and bottom (cl_fmin / cl_fmax choices)
    int64_t top = (B.y < A.y) ? (int64_t)id * 2 + 1 : (int64_t)id * 2;
    int64_t bot = (A.y < B.y) ? (int64_t)id * 2 + 1 : (int64_t)id * 2;
    if (t.x <= 0.0f) {  // trimThresholdTop at 0: the top becomes a constant
      float splitX = intersectX(h, t, 0.0f);
      if (hPos(h)) {
        t = f4{0.0f, t.y, splitX, t.w};
        h = h & UNPERSIST;
      } else {
        t = f4{0.0f, t.y, t.z, splitX};
      }
      top = -1;
    }
    if (t.w <= LEFT) {
      enclosed = true;
    } else {
      added = true;
      g.lines->push_back(Line{A, B, {0, 0, 0, 0}});
      g.q->insert(Entry{t, h, id, top, bot});
    }
  }
}

void spawn(Gen& g, uint32_t bit, Trav& l, Trav& r, bool& added, bool& enclosed) {
  EP yl = (l.left.x >= LEFT) ? pointEP(l.left, l.xPos, l.oL) : interceptEP(l, -1);
  bool leftWing = false;
  if ((l.right.x < RIGHT) && (l.right.x > LEFT)) {
    addLine(g, yl, pointEP(l.right, l.right.x, l.oR), bit, added, enclosed);
    leftWing = true;
  }
  EP yr = (r.right.x <= RIGHT) ? pointEP(r.right, r.xPos, r.oR) : interceptEP(r, -1);
  bool rightWing = false;
  if ((r.left.x > LEFT) && (r.left.x < RIGHT) && (l.index != r.index)) {
    addLine(g, pointEP(r.left, r.left.x, r.oL), yr, bit, added, enclosed);
    rightWing = true;
  }
  if (l.right.x < r.left.x || (!leftWing && !rightWing)) {
    EP bl = (leftWing || (l.left.x == l.right.x)) ? pointEP(l.right, l.right.x, l.oR) : yl;
    EP br = (rightWing || (r.left.x == r.right.x)) ? pointEP(r.left, r.left.x, r.oL) : yr;
    addLine(g, bl, br, bit, added, enclosed);
  }
}

void search(Trav& t, const float* tree, int64_t treeBase, int treeSize, f2 d, bool isLeft) {
  t.index = 0;
  while (t.index < treeSize) {
    const float* n = tree + 4 * t.index;
    const int64_t o = treeBase + 4 * t.index;
    float cx = n[0] - d.x, cy = n[1] - d.y;
    if ((t.xPos < cx) || (isLeft && t.xPos == cx)) {
      t.right = f2{cx, cy};
      t.oR = o;
      t.index = (t.index << 1) + 1;
    } else {
      t.left = f2{cx, cy};
      t.control = f2{n[2] - d.x, n[3] - d.y};
      t.oL = o;
      t.oC = o + 2;
      t.index = (t.index << 1) + 2;
    }
  }
}

uint32_t generate(const Ctx& x, const Col& c, Queue& q, std::vector<Line>& lines, uint64_t* stack,
                  std::vector<uint32_t>& idx) {
  Gen g{&q, &lines, &c};
  const f2 d{(float)c.deltaX, (float)c.deltaY};
  uint32_t bits = 0;
  for (int n = 0; n < c.numShapes && (int)bits < x.maxShape; ++n) {
    const uint32_t si = c.shapeStart + (uint32_t)n;
    const gudni_shape& shape = x.shapes[si];
    bool added = false, encShape = false;
    size_t off = (size_t)shape.geo_start * 16;
    for (uint32_t k = 0; k < shape.num_strands; ++k) {
      const float* s = reinterpret_cast<const float*>(x.geo + off);
      const int64_t sb = (int64_t)(off / 4);
      uint16_t size;
      std::memcpy(&size, x.geo + off, 2);
      bool encStrand = false;
      Trav l;
      l.right = f2{s[2] - d.x, s[3] - d.y};
      l.left = f2{s[4] - d.x, s[5] - d.y};
      l.control = f2{s[6] - d.x, s[7] - d.y};
      l.oR = sb + 2;
      l.oL = sb + 4;
      l.oC = sb + 6;
      l.xPos = 0;
      l.index = 0;
      if (l.left.x <= RIGHT && l.right.x > LEFT) {
        Trav r = l;
        l.xPos = cl_max(LEFT, l.left.x);
        r.xPos = cl_min(RIGHT, l.right.x);
        search(l, s + 8, sb + 8, ((int)size - 4) / 2, d, true);
        search(r, s + 8, sb + 8, ((int)size - 4) / 2, d, false);
        spawn(g, bits, l, r, added, encStrand);
        if (q.overflow) return bits;
      }
      off += (size_t)size * 8;
      encShape = encShape != encStrand;
    }
    if (encShape) stack[bits >> 6] ^= 1ULL << (bits & 63);
    if (added || encShape) {
      idx[bits] = si;
      bits += 1;
    }
  }
  return bits;
}

inline int clz64(uint64_t v) { return v == 0 ? 64 : __builtin_clzll(v); }
int findTop(const uint64_t* st, int above) {
  int sec = above >> 6, b = above & 63;
  uint64_t s = (~(~0ULL << b)) & st[sec];
  while (s == 0 && sec > 0) s = st[--sec];
  return (sec << 6) + (64 - clz64(s)) - 1;
}

f4 composite(f4 fg, f4 bg) {
  float ao = fg.w + bg.w * (1.0f - fg.w);
  if (ao > 0) {
    float k = 1.0f - fg.w;
    return f4{((fg.x * fg.w) + ((bg.x * bg.w) * k)) / ao, ((fg.y * fg.w) + ((bg.y * bg.w) * k)) / ao,
              ((fg.z * fg.w) + ((bg.z * bg.w) * k)) / ao, ao};
  }
  return f4{0, 0, 0, 0};
}

f4 readColor(const Ctx& x, int px, int py, uint64_t sid, uint64_t type) {
  f4 sub = x.subs[sid];
  if (type == GUDNI_TAG_SOLID) return sub;
  uint32_t id;
  std::memcpy(&id, &sub.x, 4);
  if (type == GUDNI_TAG_RADIAL) {
    const gudni_radial& g = x.radials[id];
    float dx = (float)px - g.center_x, dy = (float)py - g.center_y;
    float t = std::sqrt(dx * dx + dy * dy) / g.radius;
    t = t < 1.0f ? t : 1.0f;
    return f4{g.inner[0] + (g.outer[0] - g.inner[0]) * t, g.inner[1] + (g.outer[1] - g.inner[1]) * t,
              g.inner[2] + (g.outer[2] - g.inner[2]) * t, g.inner[3] + (g.outer[3] - g.inner[3]) * t};
  }
  const gudni_picture_use& u = x.uses[id];
  float scale = u.scale < 1e-7f ? 1e-7f : u.scale;
  float fx = ((float)px / scale) - u.translate_x, fy = ((float)py / scale) - u.translate_y;
  int rx = std::isnan(fx) ? 0 : (int)std::max(-2147483648.0f, std::min(2147483520.0f, fx));
  int ry = std::isnan(fy) ? 0 : (int)std::max(-2147483648.0f, std::min(2147483520.0f, fy));
  if (rx >= 0 && ry >= 0 && rx < u.size_x && ry < u.size_y) {
    const uint8_t* p = x.pict + u.mem_offset + 4 * ((size_t)ry * u.size_x + rx);
    return f4{(float)p[0] / 255.0f, (float)p[1] / 255.0f, (float)p[2] / 255.0f, (float)p[3] / 255.0f};
  }
  return f4{0, 0, 0, 0};
}

struct Layer {
  f4 next;
  int64_t sid;  // solid substance id, or -1 (no colour parameter)
};

// determineColor K:1447-1513, recording the composited layers
f4 determineColor(const Ctx& x, const uint64_t* stack, const std::vector<uint32_t>& idx, int bits, int px, int py,
                  std::vector<Layer>& layers) {
  layers.clear();
  int topBit = bits;
  f4 base{0, 0, 0, 0}, next{0, 0, 0, 0};
  int64_t nextSid = -1;
  bool done = false;
  uint64_t lastId = ~0ULL;
  bool lastIsContinue = true, lastIsSet = false;
  while (!done) {
    bool shouldComposite = true;
    topBit = findTop(stack, topBit);
    if (topBit < 0) {
      next = x.background;
      nextSid = -1;
      done = true;
      lastIsSet = true;
    } else {
      uint64_t tag = x.shapes[idx[topBit]].tag;
      uint64_t sid = tag & GUDNI_TAG_ID_MASK, comp = tag & GUDNI_TAG_COMPOUND_MASK;
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
        uint64_t type = tag & GUDNI_TAG_SUBSTANCE_MASK;
        next = readColor(x, px, py, sid, type);
        nextSid = type == GUDNI_TAG_SOLID ? (int64_t)sid : -1;
        lastIsSet = comp == GUDNI_TAG_ADD || comp == GUDNI_TAG_CONTINUE;
      }
      lastId = sid;
    }
    if (shouldComposite && lastIsSet) {
      layers.push_back(Layer{next, nextSid});
      base = composite(base, next);
      if (base.w == 1.0f) done = true;
    }
  }
  return base;
}

// d(composite(f, b)) -> df, db (double)
void compositeAdjoint(const double f[4], const double b[4], const double dout[4], double df[4], double db[4]) {
  const double fa = f[3], ba = b[3];
  const double ao = fa + ba * (1.0 - fa);
  for (int i = 0; i < 4; ++i) df[i] = db[i] = 0.0;
  if (!(ao > 0.0)) return;
  const double k = 1.0 - fa;
  double out[3];
  for (int c = 0; c < 3; ++c) out[c] = (f[c] * fa + b[c] * ba * k) / ao;
  double dfa = dout[3] * (1.0 - ba), dba = dout[3] * k;
  for (int c = 0; c < 3; ++c) {
    df[c] = dout[c] * fa / ao;
    db[c] = dout[c] * ba * k / ao;
    dfa += dout[c] * ((f[c] - b[c] * ba) - out[c] * (1.0 - ba)) / ao;
    dba += dout[c] * k * (b[c] - out[c]) / ao;
  }
  df[3] = dfa;
  db[3] = dba;
}

// X of a line at y and its partials w.r.t. (xa, ya, xb, yb) and y
bool lineX(const Line& L, double y, double dX[4], double& dXdy) {
  const double xa = L.a.x, ya = L.a.y, xb = L.b.x, yb = L.b.y;
  if (yb == ya) return false;
  const double s = (y - ya) / (yb - ya);
  const double m = (xb - xa) / (yb - ya);
  dX[0] = 1.0 - s;
  dX[1] = m * (s - 1.0);
  dX[2] = s;
  dX[3] = -m * s;
  dXdy = m;
  return true;
}

struct Src {
  int64_t v = -1;  // line*2 + end, or -1
};

struct ColumnGrad {
  std::vector<double>* gGeo;  // per pile float
  std::vector<double>* gSub;  // per substance x 4
};

void addY(std::vector<Line>& lines, int64_t src, double g) {
  if (src < 0) return;
  Line& L = lines[src >> 1];
  L.g[(src & 1) ? 3 : 1] += g;
}

// The render scan (K:1744-2028); with `grad`, accumulate gradients given dL/dI.
void scan(const Ctx& x, const Col& c, Queue& q, std::vector<Line>& lines, uint64_t* stack,
          const std::vector<uint32_t>& idx, int bits, float* img, const float* target, bool grad,
          ColumnGrad* cg, std::vector<double>& bitGrad) {
  int current = 0, numActive = 0;
  float sx0 = LEFT, sy0 = 0.0f, sx1 = RIGHT, sy1 = 0.0f;
  int64_t srcY0 = -1, srcY1 = -1, srcX0 = -1, srcX1 = -1;  // x sources: line id or -1
  const int px = c.deltaX;
  int py = c.deltaY;
  std::vector<Layer> layers;
  std::vector<f4> bases;
  for (float pixelY = 1.0f; pixelY <= c.floatHeight; pixelY += 1.0f) {
    float acc[4] = {0, 0, 0, 0};
    float area = 0.0f;
    const size_t pix = (size_t)py * x.bw + px;
    double gI[3] = {0, 0, 0}, I[3] = {0, 0, 0}, A = 1.0;
    if (grad) {
      for (int ch = 0; ch < 3; ++ch) {
        I[ch] = img[4 * pix + ch];
        gI[ch] = 2.0 * ((double)img[4 * pix + ch] - (double)target[4 * pix + ch]);
      }
      A = img[4 * pix + 3];
    }
    while ((sx1 < RIGHT) || (sy1 < pixelY)) {
      if (sx1 == RIGHT) {  // verticalAdvance K:1744-1824
        for (int i = 0; i < numActive; ++i) {
          uint32_t b = q.at(i).h & BITMASK;
          stack[b >> 6] ^= 1ULL << (b & 63);
        }
        const float nextBreak = cl_min(c.floatHeight, pixelY);
        const float activeBottom = q.len() > 0 ? q.at(0).t.y : FLT_MAX;
        const int64_t activeSrc = q.len() > 0 ? q.at(0).bot : -1;
        if (activeBottom == sy1) {
          while (numActive > 0) {
            uint32_t h = q.at(0).h;
            if (hBot(h)) {
              uint32_t b = h & BITMASK;
              stack[b >> 6] ^= 1ULL << (b & 63);
            }
            q.start += 1;
            numActive -= 1;
          }
        }
        float nextBottom;
        int64_t nextSrc;
        if (numActive > 0) {
          bool brk = nextBreak < activeBottom;  // cl_min(activeBottom, nextBreak)
          nextBottom = brk ? nextBreak : activeBottom;
          nextSrc = brk ? -1 : activeSrc;
        } else {
          const float nextTop = numActive < q.len() ? q.at(numActive).t.x : FLT_MAX;
          const int64_t nextTopSrc = numActive < q.len() ? q.at(numActive).top : -1;
          if (nextTop > sy1) {
            bool top = nextTop < nextBreak;  // cl_min(nextBreak, nextTop)
            nextBottom = top ? nextTop : nextBreak;
            nextSrc = top ? nextTopSrc : -1;
          } else {
            // splitNext K:1069-1077
            float sp = FLT_MAX;
            int64_t spSrc = -1;
            const float top0 = q.at(0).t.x;
            int n = 1;
            while (n < q.len()) {
              if (q.at(n).t.x > top0) {
                sp = q.at(n).t.x;
                spSrc = q.at(n).top;
                break;
              }
              n += 1;
            }
            numActive = n;
            float sp2 = sp;
            int64_t sp2Src = spSrc;
            for (int i = 0; i < n; ++i) {
              float b = q.at(i).t.y;
              if (top0 < b && b < sp2) {
                sp2 = b;
                sp2Src = q.at(i).bot;
              }
            }
            if (sp2 < sp) {
              sp = sp2;
              spSrc = sp2Src;
            }
            for (int cur = 0; cur < n; ++cur) {
              Entry e = q.at(cur);
              if (e.t.x < sp && sp < e.t.y) {
                float splitX = intersectX(e.h, e.t, sp);
                Entry lo = e, hi = e;
                if (hPos(e.h)) {
                  lo.t = f4{sp, e.t.y, splitX, e.t.w};
                  hi.t = f4{e.t.x, sp, e.t.z, splitX};
                  lo.h = e.h & UNPERSIST;
                } else {
                  lo.t = f4{sp, e.t.y, e.t.z, splitX};
                  hi.t = f4{e.t.x, sp, splitX, e.t.w};
                  lo.h = e.h;
                  hi.h = e.h & UNPERSIST;
                }
                lo.top = spSrc;
                hi.bot = spSrc;
                q.at(cur) = hi;
                if (tKeep(lo.h, lo.t)) {
                  q.insert(lo);
                  if (q.overflow) return;
                }
              }
            }
            bool brk = sp < nextBreak;  // cl_min(nextBreak, sp)
            nextBottom = brk ? sp : nextBreak;
            nextSrc = brk ? spSrc : -1;
            while (numActive > 0 && q.at(0).t.x == q.at(0).t.y) {
              uint32_t h = q.at(0).h;
              if (hTop(h)) {
                uint32_t b = h & BITMASK;
                stack[b >> 6] ^= 1ULL << (b & 63);
              }
              q.start += 1;
              numActive -= 1;
            }
            for (int i = 0; i < numActive; ++i) {
              if (q.at(i).t.x > 0.0f && hTop(q.at(i).h)) {
                uint32_t b = q.at(i).h & BITMASK;
                stack[b >> 6] ^= 1ULL << (b & 63);
              }
            }
          }
        }
        sy0 = sy1;
        srcY0 = srcY1;
        sy1 = nextBottom;
        srcY1 = nextSrc;
        sx0 = sx1 = LEFT;
        srcX0 = srcX1 = -1;
        current = 0;
      }
      // horizontalAdvance K:1826-1851
      float nextX = RIGHT;
      int64_t nextXSrc = -1;
      if (current < numActive) {
        const Entry& e = q.at(current);
        float ym = sy0 + ((sy1 - sy0) * 0.5f);
        float xx = intersectX(e.h, e.t, ym);
        if (xx >= RIGHT) {
          nextX = LEFT;
        } else if (LEFT < xx) {
          nextX = xx;
          nextXSrc = e.line;
        } else {
          nextX = LEFT;
        }
      }
      sx0 = sx1;
      srcX0 = srcX1;
      sx1 = nextX;
      srcX1 = nextXSrc;
      f4 col = determineColor(x, stack, idx, bits, px, py, layers);
      float a = (sx1 - sx0) * (sy1 - sy0);
      acc[0] += col.x * a;
      acc[1] += col.y * a;
      acc[2] += col.z * a;
      area += a;
      if (grad) {
        // dL/da and dL/dcol for this section
        const double cc[3] = {col.x, col.y, col.z};
        double dA = 0.0;
        for (int ch = 0; ch < 3; ++ch) dA += gI[ch] * (cc[ch] - I[ch]) / A;
        const double w = (double)sy1 - (double)sy0, hgt = (double)sx1 - (double)sx0;
        double dx1 = dA * w, dx0 = -dA * w, dy1 = dA * hgt, dy0 = -dA * hgt;
        const double ym = (double)sy0 + ((double)sy1 - (double)sy0) * 0.5;
        double dym = 0.0;
        double dX[4], dXdy;
        if (srcX1 >= 0 && lineX(lines[srcX1], ym, dX, dXdy)) {
          for (int k = 0; k < 4; ++k) lines[srcX1].g[k] += dx1 * dX[k];
          dym += dx1 * dXdy;
        }
        if (srcX0 >= 0 && lineX(lines[srcX0], ym, dX, dXdy)) {
          for (int k = 0; k < 4; ++k) lines[srcX0].g[k] += dx0 * dX[k];
          dym += dx0 * dXdy;
        }
        dy0 += 0.5 * dym;
        dy1 += 0.5 * dym;
        addY(lines, srcY0, dy0);
        addY(lines, srcY1, dy1);
        // colour: back through the composite chain
        const int K = (int)layers.size();
        bases.assign(K + 1, f4{0, 0, 0, 0});
        for (int k = 0; k < K; ++k) bases[k + 1] = composite(bases[k], layers[k].next);
        double d[4] = {gI[0] * a / A, gI[1] * a / A, gI[2] * a / A, 0.0};
        for (int k = K - 1; k >= 0; --k) {
          const double f[4] = {bases[k].x, bases[k].y, bases[k].z, bases[k].w};
          const double b[4] = {layers[k].next.x, layers[k].next.y, layers[k].next.z, layers[k].next.w};
          double df[4], db[4];
          compositeAdjoint(f, b, d, df, db);
          if (layers[k].sid >= 0)
            for (int ch = 0; ch < 4; ++ch) (*cg->gSub)[4 * layers[k].sid + ch] += db[ch];
          for (int ch = 0; ch < 4; ++ch) d[ch] = df[ch];
        }
      }
      if (current < numActive) {
        uint32_t b = q.at(current).h & BITMASK;
        stack[b >> 6] ^= 1ULL << (b & 63);
      }
      current += 1;
    }
    if (!grad) {
      img[4 * pix + 0] = acc[0] / area;
      img[4 * pix + 1] = acc[1] / area;
      img[4 * pix + 2] = acc[2] / area;
      img[4 * pix + 3] = area;
    }
    sx0 = LEFT;
    srcX0 = -1;
    sy0 = pixelY;
    srcY0 = -1;
    py += 1;
  }
  (void)bitGrad;
}

// Full chain of a line's end points, reading the pile for the sub-curve ends.
void chainLine(const Line& L, const float* pile, const f2 d, std::vector<double>& gGeo) {
  const EP* eps[2] = {&L.a, &L.b};
  const double gxs[2] = {L.g[0], L.g[2]}, gys[2] = {L.g[1], L.g[3]};
  for (int k = 0; k < 2; ++k) {
    const EP& e = *eps[k];
    const double gx = gxs[k], gy = gys[k];
    if (gx == 0.0 && gy == 0.0) continue;
    if (e.kind == 0) {
      gGeo[e.pt] += gx;
      gGeo[e.pt + 1] += gy;
      continue;
    }
    double wt0[3] = {(1 - e.t0) * (1 - e.t0), 2 * e.t0 * (1 - e.t0), e.t0 * e.t0};
    double wt1[3] = {(1 - e.t1) * (1 - e.t1), 2 * e.t1 * (1 - e.t1), e.t1 * e.t1};
    double x0 = 0, y0 = 0, x1 = 0, y1 = 0;
    for (int i = 0; i < 3; ++i) {
      const double px = (double)pile[e.q[i]] - d.x, py = (double)pile[e.q[i] + 1] - d.y;
      x0 += wt0[i] * px;
      y0 += wt0[i] * py;
      x1 += wt1[i] * px;
      y1 += wt1[i] * py;
    }
    double dydx0, dydy0, dydx1, dydy1, dydxp;
    if (e.kind == 2) {  // y = min(y0, y1)
      const bool second = (float)y1 < (float)y0;
      dydx0 = dydx1 = dydxp = 0.0;
      dydy0 = second ? 0.0 : 1.0;
      dydy1 = second ? 1.0 : 0.0;
    } else {
      const double m = (y1 - y0) / (x1 - x0), u = ((double)e.x - x0) / (x1 - x0);
      dydx0 = m * (u - 1.0);
      dydy0 = 1.0 - u;
      dydx1 = -m * u;
      dydy1 = u;
      dydxp = m;
    }
    if (e.xsrc >= 0) gGeo[e.xsrc] += gx + gy * dydxp;
    for (int i = 0; i < 3; ++i) {
      gGeo[e.q[i]] += gy * (dydx0 * wt0[i] + dydx1 * wt1[i]);
      gGeo[e.q[i] + 1] += gy * (dydy0 * wt0[i] + dydy1 * wt1[i]);
    }
  }
}

Col initCol(const Ctx& x, const gudni_tile_info& ti, int column) {
  Col c;
  c.shapeStart = ti.shapes.start;
  c.numShapes = (int)ti.shapes.length;
  int diff = std::max(0, ti.vdepth - (x.log2tpt - ti.hdepth));
  int internalX = ((1 << ti.hdepth) - 1) & column;
  c.internalY = (column >> ti.hdepth) << diff;
  c.deltaX = internalX + ti.left;
  c.deltaY = c.internalY + ti.top;
  c.intHeight = std::min(1 << diff, x.bh - c.deltaY);
  c.floatHeight = (float)c.intHeight;
  c.tileH = ti.bottom - ti.top;
  c.active = c.internalY < c.tileH && c.deltaX < x.bw && c.deltaY < x.bh;
  return c;
}

}  // namespace

extern "C" {

// Float image and (with a target) the FP64 gradient of one job.  img: H*W*4 floats
// (I rgb, total area); target: H*W*4 floats (rgb used) or NULL for the image only;
// grad_geo: geometry_bytes/4 doubles (per pile float); grad_sub: 4 per substance.
// Gradients are added to the arrays.  Returns 0, or -2 on a queue overflow.
int oracle_adjoint_job(const uint8_t* geometry, size_t geometry_bytes, const float* substances, size_t n_substances,
                       const uint8_t* pictures, const gudni_picture_use* uses, const gudni_radial* radials,
                       const gudni_shape* shapes, const gudni_tile_info* tiles, int n_tiles, int threads_per_tile,
                       int compute_depth, int bitmap_w, int bitmap_h, const float* background, int max_thresholds,
                       int max_shape, float* img, const float* target, double* grad_geo, double* grad_sub,
                       int n_threads) {
  Ctx x;
  x.geo = geometry;
  x.subs = reinterpret_cast<const f4*>(substances);
  x.nSub = (uint32_t)n_substances;
  x.pict = pictures;
  x.uses = uses;
  x.radials = radials;
  x.shapes = shapes;
  x.background = f4{background[0], background[1], background[2], background[3]};
  x.maxShape = max_shape;
  x.bw = bitmap_w;
  x.bh = bitmap_h;
  x.log2tpt = compute_depth;
  x.cap = max_thresholds;
  const long long total = (long long)n_tiles * threads_per_tile;
  const size_t nGeo = geometry_bytes / 4;
  const int sections = (max_shape + 64) / 64;
  int overflow = 0;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
  const bool grad = target != nullptr;
#pragma omp parallel
  {
    std::vector<Entry> entries(max_thresholds);
    std::vector<Line> lines;
    std::vector<uint32_t> idx(max_shape > 0 ? max_shape : 1);
    std::vector<uint64_t> stack(sections + 1);
    std::vector<double> gGeo(grad ? nGeo : 0, 0.0), gSub(grad ? 4 * n_substances : 0, 0.0), bitGrad;
    ColumnGrad cg{&gGeo, &gSub};
    int ov = 0;
#pragma omp for schedule(dynamic, 4)
    for (long long w = 0; w < total; ++w) {
      const gudni_tile_info& ti = tiles[w / threads_per_tile];
      Col c = initCol(x, ti, (int)(w % threads_per_tile));
      if (!c.active) continue;
      for (int pass = 0; pass < (grad ? 2 : 1); ++pass) {
        // pass 0 renders the float image; pass 1 regenerates and scans with gradients
        Queue q{&entries, max_thresholds, max_thresholds, false};
        lines.clear();
        std::fill(stack.begin(), stack.end(), 0ULL);
        int bits = (int)generate(x, c, q, lines, stack.data(), idx);
        if (q.overflow) { ov = 1; break; }
        scan(x, c, q, lines, stack.data(), idx, bits, img, target, pass == 1, &cg, bitGrad);
        if (q.overflow) { ov = 1; break; }
        if (pass == 1) {
          const f2 d{(float)c.deltaX, (float)c.deltaY};
          for (const Line& L : lines) chainLine(L, reinterpret_cast<const float*>(geometry), d, gGeo);
        }
      }
    }
#pragma omp critical
    {
      overflow |= ov;
      if (grad) {
        for (size_t i = 0; i < nGeo; ++i) grad_geo[i] += gGeo[i];
        for (size_t i = 0; i < 4 * n_substances; ++i) grad_sub[i] += gSub[i];
      }
    }
  }
  return overflow ? -2 : 0;
}

}  // extern "C"
