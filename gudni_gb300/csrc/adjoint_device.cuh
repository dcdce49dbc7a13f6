// Per-column device code of the adjoint (adjoint.cu): the column machine with
// provenance -- line end points that remember where they come from in the geometry
// pile, the threshold queue with y sources, the scan that accumulates boundary-term
// and composite-chain gradients, and one column's two passes (adjointColumn).  The
// warp-level gathering of gradients and the kernel are in adjoint.cu.
#pragma once

#include "raster_device.cuh"

namespace gudni {

namespace {

// Line end point with provenance (36 bytes).
struct EP {
  float x, y;        // tile-relative value
  int32_t kind;      // 0 strand point, 1 intercept, 2 intercept with y = min of the sub-curve's ends
  int32_t pt;        // kind 0: float index of x in the pile; kinds 1-2: pile x of xPos, or -1
  int32_t q0, q1, q2;  // kinds 1-2: float indices of P0, P1, P2
  float t0, t1;      // kinds 1-2: the sub-curve [t0, t1]
};

struct LineRec {
  EP a, b;
  float invDy;  // 1 / (b.y - a.y), or 0 for a horizontal line
};

// y source: line*2 + end (0 = a, 1 = b), or -1 for a constant
constexpr int32_t kConst = -1;

struct AdjQueue {
  float4* thr;
  uint32_t* hdr;
  int4* prov;  // x: line, y: top source, z: bottom source
  int start, cap;
  bool overflow;
  __device__ __forceinline__ int length() const { return cap - start; }
  __device__ __forceinline__ void push(uint32_t h, float4 t, int4 p) {
    if (start == 0) {
      overflow = true;
      return;
    }
    start -= 1;
    hdr[start] = h;
    thr[start] = t;
    prov[start] = p;
  }
  __device__ __forceinline__ void insert(uint32_t h, float4 t, int4 p) {
    if (start == 0) {
      overflow = true;
      return;
    }
    start -= 1;
    const int len = cap - start;
    int cursor = 0;
    while (cursor < len - 1) {
      const uint32_t oh = hdr[start + cursor + 1];
      const float4 o = thr[start + cursor + 1];
      if (!isBelow(h, t, oh, o)) break;
      hdr[start + cursor] = oh;
      thr[start + cursor] = o;
      prov[start + cursor] = prov[start + cursor + 1];
      cursor += 1;
    }
    hdr[start + cursor] = h;
    thr[start + cursor] = t;
    prov[start + cursor] = p;
  }
  __device__ __forceinline__ void move(int to, int from) {
    thr[to] = thr[from];
    hdr[to] = hdr[from];
    prov[to] = prov[from];
  }
  // sliceActive of the first n (active) entries at sp: the part above stays in place,
  // the part below (when kept) is inserted as insertThreshold would; the same batched
  // form as the forward scan's splitNext (parts collected below the queue, the active
  // block moved once, the parts walked in past it) when every active top is below sp
  // and the slab has room.  y sources: the split point's for the new bottom / top.
  __device__ __forceinline__ void splitActive(int n, float sp, int32_t spSrc) {
    bool batched = start >= 2 * n;
    for (int i = 0; batched && i < n; ++i) batched = thr[start + i].x < sp;
    const int s0 = start;
    int m = 0;
    for (int cur = 0; cur < n; ++cur) {
      const int at = batched ? s0 + cur : start + cur;
      const uint32_t ch = hdr[at];
      const float4 e = thr[at];
      const int4 pv = prov[at];
      if (e.x < sp && sp < e.y) {
        const float splitX = intersectX(ch, e, sp);
        float4 lo, hi;
        uint32_t lh, hh;
        if (hPositive(ch)) {
          lo = make_float4(sp, e.y, splitX, e.w);
          hi = make_float4(e.x, sp, e.z, splitX);
          lh = ch & kUnpersist;
          hh = ch;
        } else {
          lo = make_float4(sp, e.y, e.z, splitX);
          hi = make_float4(e.x, sp, splitX, e.w);
          lh = ch;
          hh = ch & kUnpersist;
        }
        hdr[at] = hh;
        thr[at] = hi;
        prov[at] = make_int4(pv.x, pv.y, spSrc, 0);
        if (tKeep(lh, lo)) {
          const int4 lp = make_int4(pv.x, spSrc, pv.z, 0);
          if (batched) {
            hdr[s0 - n - 1 - m] = lh;
            thr[s0 - n - 1 - m] = lo;
            prov[s0 - n - 1 - m] = lp;
            ++m;
          } else {
            insert(lh, lo, lp);
            if (overflow) return;
          }
        }
      }
    }
    if (!batched || m == 0) return;
    for (int i = 0; i < n; ++i) move(s0 - m + i, s0 + i);
    start = s0 - m;
    int f = s0 + n;
    for (int j = 0; j < m; ++j) {
      const int src = s0 - n - 1 - j;
      const uint32_t h = hdr[src];
      const float4 t = thr[src];
      const int4 pv = prov[src];
      f -= 1;
      int at = f;
      while (at + 1 < cap && isBelow(h, t, hdr[at + 1], thr[at + 1])) {
        move(at, at + 1);
        at += 1;
      }
      hdr[at] = h;
      thr[at] = t;
      prov[at] = pv;
    }
  }
  // stable sort (the order the forward pass's sort produces): bottom-up merge sort
  // through the free slab space below the queue when it has room, else insertion sort;
  // with a non-finite coordinate in the queue the reference's bubble sort, as
  // sortQueue does
  __device__ __forceinline__ void sort() {
    const int n = cap - start;
    bool ordered = true;
    for (int i = start; i < cap && ordered; ++i) ordered = keysOrdered(thr[i]);
    if (!ordered) {
      bool done = false;
      for (int k = n; !done; --k) {
        done = true;
        for (int i = start; i < start + k - 1; ++i) {
          if (isBelow(hdr[i], thr[i], hdr[i + 1], thr[i + 1])) {
            const float4 t = thr[i];
            const uint32_t h = hdr[i];
            const int4 p = prov[i];
            thr[i] = thr[i + 1];
            hdr[i] = hdr[i + 1];
            prov[i] = prov[i + 1];
            thr[i + 1] = t;
            hdr[i + 1] = h;
            prov[i + 1] = p;
            done = false;
          }
        }
      }
      return;
    }
    if (n >= 32 && start >= n) {
      int src = start, dst = start - n;
      for (int width = 1; width < n; width *= 2) {
        for (int lo = 0; lo < n; lo += 2 * width) {
          const int mid = min(lo + width, n), hi = min(lo + 2 * width, n);
          int a = lo, b = mid, o = lo;
          while (a < mid && b < hi) {
            if (isBelow(hdr[src + a], thr[src + a], hdr[src + b], thr[src + b])) {
              move(dst + o, src + b);
              ++b;
            } else {
              move(dst + o, src + a);
              ++a;
            }
            ++o;
          }
          while (a < mid) move(dst + o++, src + a++);
          while (b < hi) move(dst + o++, src + b++);
        }
        const int t = src;
        src = dst;
        dst = t;
      }
      if (src != start)
        for (int i = 0; i < n; ++i) move(start + i, src + i);
      return;
    }
    for (int i = start + 1; i < cap; ++i) {
      const float4 t = thr[i];
      const uint32_t h = hdr[i];
      const int4 p = prov[i];
      int j = i - 1;
      while (j >= start && isBelow(hdr[j], thr[j], h, t)) {
        thr[j + 1] = thr[j];
        hdr[j + 1] = hdr[j];
        prov[j + 1] = prov[j];
        --j;
      }
      thr[j + 1] = t;
      hdr[j + 1] = h;
      prov[j + 1] = p;
    }
  }
};

struct Trav {
  float2 left, control, right;
  float xPos;
  int index;
  int32_t oL, oC, oR;
};

// bifurcateCurve K:1233-1258, tracking the sub-curve's parameter interval
__device__ __forceinline__ void bifurcateP(Trav& t, float& t0, float& t1, int& status) {
  t0 = 0.0f;
  t1 = 1.0f;
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
    const float mid = 0.5f * (t0 + t1);
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

__device__ __forceinline__ EP interceptEP(const Trav& l, int& status) {
  Trav t = l;
  EP e;
  e.q0 = l.oL;
  e.q1 = l.oC;
  e.q2 = l.oR;
  e.pt = -1;
  bifurcateP(t, e.t0, e.t1, status);
  e.x = l.xPos;
  if (t.left.x == t.right.x) {
    e.kind = 2;
    e.y = cl_min(t.left.y, t.right.y);
  } else {
    e.kind = 1;
    e.y = (((t.right.y - t.left.y) / (t.right.x - t.left.x)) * (t.xPos - t.left.x)) + t.left.y;
  }
  return e;
}

__device__ __forceinline__ EP pointEP(float2 p, float x, int32_t off) {
  EP e;
  e.x = x;
  e.y = p.y;
  e.kind = 0;
  e.pt = off;
  e.q0 = e.q1 = e.q2 = -1;
  e.t0 = e.t1 = 0.0f;
  return e;
}

struct AdjGen {
  AdjQueue* q;
  LineRec* lines;
  int* n_lines;
  int line_cap;
  const ColumnState* c;
};

__device__ __forceinline__ void addLineP(AdjGen& g, const EP& A, const EP& B, uint32_t bit, bool& added,
                                         bool& enclosed) {
  float4 t = make_float4(cl_fmin(A.y, B.y), cl_fmax(A.y, B.y), A.x, B.x);
  const bool positive = A.y <= B.y;
  const bool persist = (A.x != B.x) && (A.x == kLeft);
  uint32_t h = (positive ? kPositive : 0u) | (persist ? kPersist : 0u) | bit;
  if (!tKeep(h, t)) return;
  enclosed = enclosed || ((t.x <= 0.0f) && hPersistTop(h)) || ((t.y <= 0.0f) && hPersistBottom(h));
  if ((t.x < g.c->floatHeight) && (t.y > 0.0f) && (t.z < kRight)) {
    const int32_t id = *g.n_lines;
    int32_t top = (B.y < A.y) ? id * 2 + 1 : id * 2;
    const int32_t bot = (A.y < B.y) ? id * 2 + 1 : id * 2;
    if (t.x <= 0.0f) {
      float splitX = intersectX(h, t, 0.0f);
      if (hPositive(h)) {
        t = make_float4(0.0f, t.y, splitX, t.w);
        h = h & kUnpersist;
      } else {
        t = make_float4(0.0f, t.y, t.z, splitX);
      }
      top = kConst;
    }
    if (t.w <= kLeft) {
      enclosed = true;
    } else {
      added = true;
      if (id >= g.line_cap) {
        g.q->overflow = true;
        return;
      }
      g.lines[id].a = A;
      g.lines[id].b = B;
      g.lines[id].invDy = (B.y != A.y) ? 1.0f / (B.y - A.y) : 0.0f;
      *g.n_lines = id + 1;
      g.q->push(h, t, make_int4(id, top, bot, 0));
    }
  }
}

// `above`: as spawnThresholds -- the strand lies wholly above the column, only the
// enclosure flag can change, and the intercepts are not computed.
__device__ __forceinline__ EP aboveEP(float x) {
  EP e = pointEP(make_float2(x, -1.0f), x, -1);
  return e;
}

__device__ __forceinline__ void spawnP(AdjGen& g, uint32_t bit, Trav& l, Trav& r, bool& added, bool& enclosed,
                                       int& status, bool above) {
  const EP yl = (l.left.x >= kLeft) ? pointEP(l.left, l.xPos, l.oL) : (above ? aboveEP(l.xPos) : interceptEP(l, status));
  bool leftWing = false;
  if ((l.right.x < kRight) && (l.right.x > kLeft)) {
    addLineP(g, yl, pointEP(l.right, l.right.x, l.oR), bit, added, enclosed);
    leftWing = true;
  }
  const EP yr = (r.right.x <= kRight) ? pointEP(r.right, r.xPos, r.oR) : (above ? aboveEP(r.xPos) : interceptEP(r, status));
  bool rightWing = false;
  if ((r.left.x > kLeft) && (r.left.x < kRight) && (l.index != r.index)) {
    addLineP(g, pointEP(r.left, r.left.x, r.oL), yr, bit, added, enclosed);
    rightWing = true;
  }
  if (l.right.x < r.left.x || (!leftWing && !rightWing)) {
    const EP bl = (leftWing || (l.left.x == l.right.x)) ? pointEP(l.right, l.right.x, l.oR) : yl;
    const EP br = (rightWing || (r.left.x == r.right.x)) ? pointEP(r.left, r.left.x, r.oL) : yr;
    addLineP(g, bl, br, bit, added, enclosed);
  }
}

__device__ __forceinline__ void searchP(Trav& t, const float4* tree, int32_t treeBase, int treeSize, float2 d,
                                        bool isLeft) {
  t.index = 0;
  while (t.index < treeSize) {
    const float4 n = tree[t.index];
    const int32_t o = treeBase + 4 * t.index;
    const float cx = n.x - d.x, cy = n.y - d.y;
    if ((t.xPos < cx) || (isLeft && t.xPos == cx)) {
      t.right = make_float2(cx, cy);
      t.oR = o;
      t.index = (t.index << 1) + 1;
    } else {
      t.left = make_float2(cx, cy);
      t.control = make_float2(n.z - d.x, n.w - d.y);
      t.oL = o;
      t.oC = o + 2;
      t.index = (t.index << 1) + 2;
    }
  }
}

// traverseTree + spawnThresholds for one strand at byte offset `off` of the pile
__device__ __forceinline__ void strandP(const RasterInputs& in, AdjGen& g, size_t off, uint32_t size, float2 d,
                                        uint32_t bits, bool& added, bool& encStrand, int& status, bool above) {
  const uint8_t* strand = in.geometry + off;
  const int32_t sb = (int32_t)(off / 4);
  const float2 rp = *reinterpret_cast<const float2*>(strand + 8);
  const float4 lc = *reinterpret_cast<const float4*>(strand + 16);
  Trav l;
  l.right = make_float2(rp.x - d.x, rp.y - d.y);
  l.left = make_float2(lc.x - d.x, lc.y - d.y);
  l.control = make_float2(lc.z - d.x, lc.w - d.y);
  l.oR = sb + 2;
  l.oL = sb + 4;
  l.oC = sb + 6;
  l.xPos = 0.0f;
  l.index = 0;
  if (l.left.x <= kRight && l.right.x > kLeft) {
    Trav r = l;
    l.xPos = cl_max(kLeft, l.left.x);
    r.xPos = cl_min(kRight, l.right.x);
    const float4* tree = reinterpret_cast<const float4*>(strand + 32);
    const int treeSize = ((int)size - 4) / 2;
    searchP(l, tree, sb + 8, treeSize, d, true);
    searchP(r, tree, sb + 8, treeSize, d, false);
    // the same hull culling as the forward generation (strandThresholds)
    const float lo = fminf(fminf(fminf(l.left.y, l.control.y), fminf(l.right.y, r.left.y)),
                           fminf(r.control.y, r.right.y));
    const float hi = fmaxf(fmaxf(fmaxf(l.left.y, l.control.y), fmaxf(l.right.y, r.left.y)),
                           fmaxf(r.control.y, r.right.y));
    const float extent = fabsf(l.left.y) + fabsf(l.control.y) + fabsf(l.right.y) + fabsf(r.left.y) +
                       fabsf(r.control.y) + fabsf(r.right.y) + fabsf(l.left.x) + fabsf(l.control.x) +
                       fabsf(l.right.x) + fabsf(r.left.x) + fabsf(r.control.x) + fabsf(r.right.x);
    const bool ordered = extent <= kCullExtent;
    if (ordered && lo >= g.c->floatHeight + 1.0f) return;
    spawnP(g, bits, l, r, added, encStrand, status, above || (ordered && hi <= -1.0f));
  }
}

// buildThresholdArray with provenance; the same strand-table range test and y
// culling as the forward generation (buildThresholds), so the decisions match.
template <int SECTIONS>
__device__ __forceinline__ uint32_t generateP(const RasterInputs& in, const ColumnState& c, AdjGen& g,
                                              ShapeStack<SECTIONS>& stack, uint32_t* shapeIdx, int& status) {
  const float2 d = make_float2((float)c.deltaX, (float)c.deltaY);
  uint32_t bits = 0;
  for (int n = 0; n < c.numShapes && (int)bits < in.max_shape; ++n) {
    const uint32_t si = c.shapeStart + (uint32_t)n;
    const gudni_shape shape = in.shapes[si];
    bool added = false, encShape = false;
    uint32_t first = kNoStrand;
    if (in.strand_table && shape.geo_start < in.n_units) first = in.strand_first[shape.geo_start];
    if (first != kNoStrand && (uint64_t)first + shape.num_strands <= in.n_strands) {
      for (uint32_t k = 0; k < shape.num_strands; ++k) {
        const uint4 e = in.strand_table[first + k];
        const float lx = __uint_as_float(e.z) - d.x;
        const float rx = __uint_as_float(e.w) - d.x;
        if (!(lx <= kRight && rx > kLeft)) continue;
        const float2 yr = in.strand_y[first + k];
        if (yr.x - d.y >= c.floatHeight + 1.0f) continue;
        const bool above = yr.y - d.y <= -1.0f;
        bool encStrand = false;
        strandP(in, g, (size_t)e.x * 8, e.y, d, bits, added, encStrand, status, above);
        if (g.q->overflow) return bits;
        encShape = encShape != encStrand;
      }
    } else {
      size_t off = (size_t)shape.geo_start * 16;
      for (uint32_t k = 0; k < shape.num_strands; ++k) {
        if (off + 32 > in.geometry_bytes) {
          status |= kStatusBadInput;
          break;
        }
        const uint32_t size = (uint32_t)(*reinterpret_cast<const uint16_t*>(in.geometry + off));
        if (size < 4 || (size & 1u) != 0 || off + (size_t)size * 8 > in.geometry_bytes) {
          status |= kStatusBadInput;
          break;
        }
        bool encStrand = false;
        strandP(in, g, off, size, d, bits, added, encStrand, status, false);
        if (g.q->overflow) return bits;
        off += (size_t)size * 8;
        encShape = encShape != encStrand;
      }
    }
    if (encShape) stack.flip(bits);
    if (added || encShape) {
      shapeIdx[bits] = si;
      bits += 1;
    }
  }
  return bits;
}

// determineColor K:1447-1513 recording the composited layers: colour, the composite
// in front of it, and its shape bit (kSolidLayer set for a solid colour; -1 for the
// background).  Every layer is a distinct substance of a distinct shape bit or the
// background, so a column with `bits` shape bits has at most bits + 1 layers.
// Returns the layer count, or -1 past `cap` layers; `stopBit` and `positional` as for
// determineColor's memo (the lowest bit read; whether a picture or gradient layer was
// composited).
constexpr int32_t kSolidLayer = 0x40000000;

template <int SECTIONS>
__device__ __forceinline__ int layersOf(const RasterInputs& in, const ShapeStack<SECTIONS>& stack,
                                        const uint32_t* shapeIdx, int px, int py, int topStart, float4* next,
                                        float4* front, int32_t* bitOf, int cap, int ls, float4& color,
                                        bool& positional, int& stopBit, int& status) {
  int64_t texels = 0;
  int topBit = topStart;
  float4 base = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float4 nx = base;
  int nbit = -1;
  bool nsolid = false;
  bool done = false;
  uint64_t lastId = ~0ull;
  bool lastIsContinue = true, lastIsSet = false;
  int K = 0;
  positional = false;
  while (!done) {
    bool shouldComposite = true;
    topBit = stack.findTop(topBit);
    if (topBit < 0) {
      nx = in.background;
      nbit = -1;
      nsolid = false;
      done = true;
      lastIsSet = true;
    } else {
      const uint64_t tag = in.shapes[shapeIdx[topBit]].tag;
      const uint64_t sid = tag & GUDNI_TAG_ID_MASK, comp = tag & GUDNI_TAG_COMPOUND_MASK;
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
        nx = readColor(in, px, py, sid, type, status, texels);
        nbit = topBit;
        nsolid = type == GUDNI_TAG_SOLID;
        lastIsSet = comp == GUDNI_TAG_ADD || comp == GUDNI_TAG_CONTINUE;
      }
      lastId = sid;
    }
    if (shouldComposite && lastIsSet) {
      if (K >= cap) return -1;
      next[K * ls] = nx;
      front[K * ls] = base;
      bitOf[K * ls] = (nsolid && nbit >= 0) ? (nbit | kSolidLayer) : nbit;
      positional = positional || (nbit >= 0 && !nsolid);
      ++K;
      base = composite(base, nx);
      if (base.w == 1.0f) done = true;
    }
  }
  color = base;
  stopBit = topBit;
  return K;
}

// d(composite(f, b)) given d(out): partials of K:878-887
__device__ __forceinline__ void compositeAdjoint(float4 f, float4 b, float4 dout, float4& df, float4& db) {
  const float fa = f.w, ba = b.w;
  const float ao = fa + ba * (1.0f - fa);
  if (!(ao > 0.0f)) {
    df = db = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return;
  }
  const float k = 1.0f - fa;
  const float inv = 1.0f / ao;
  const float fr[3] = {f.x, f.y, f.z}, br[3] = {b.x, b.y, b.z}, dr[3] = {dout.x, dout.y, dout.z};
  float dfa = dout.w * (1.0f - ba), dba = dout.w * k;
  float dfc[3], dbc[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float out = (fr[c] * fa + br[c] * ba * k) * inv;
    dfc[c] = dr[c] * fa * inv;
    dbc[c] = dr[c] * ba * k * inv;
    dfa += dr[c] * ((fr[c] - br[c] * ba) - out * (1.0f - ba)) * inv;
    dba += dr[c] * k * (br[c] - out) * inv;
  }
  df = make_float4(dfc[0], dfc[1], dfc[2], dfa);
  db = make_float4(dbc[0], dbc[1], dbc[2], dba);
}

// X of a line at y and its partials w.r.t. (xa, ya, xb, yb) and y
__device__ __forceinline__ bool lineX(const LineRec& L, float y, float dX[4], float& dXdy) {
  const float xa = L.a.x, ya = L.a.y, xb = L.b.x, yb = L.b.y;
  if (yb == ya) return false;
  const float s = (y - ya) * L.invDy;
  const float m = (xb - xa) * L.invDy;
  dX[0] = 1.0f - s;
  dX[1] = m * (s - 1.0f);
  dX[2] = s;
  dX[3] = -m * s;
  dXdy = m;
  return true;
}

__device__ __forceinline__ void addY(float4* lg, int32_t src, float g) {
  if (src < 0) return;
  float* p = reinterpret_cast<float*>(&lg[src >> 1]);
  p[(src & 1) ? 3 : 1] += g;
}

// A line end point's (gx, gy) carried to pile floats: up to seven (float index, value)
// pairs -- a strand point's x and y, or an intercept's x source and the x and y of the
// three points of its sub-curve.  Unused pairs have index -1.
constexpr int kEpTargets = 7;

__device__ __forceinline__ void epTargets(const EP& e, float gx, float gy, const float* pile, float2 d,
                                          int32_t* idx, float* val) {
#pragma unroll
  for (int k = 0; k < kEpTargets; ++k) {
    idx[k] = -1;
    val[k] = 0.0f;
  }
  if (gx == 0.0f && gy == 0.0f) return;
  if (e.kind == 0) {
    if (e.pt < 0) return;  // a stand-in end point (never on a kept line)
    idx[0] = e.pt;
    val[0] = gx;
    idx[1] = e.pt + 1;
    val[1] = gy;
    return;
  }
  const float u0 = 1.0f - e.t0, u1 = 1.0f - e.t1;
  const float w0[3] = {u0 * u0, 2.0f * e.t0 * u0, e.t0 * e.t0};
  const float w1[3] = {u1 * u1, 2.0f * e.t1 * u1, e.t1 * e.t1};
  const int32_t q[3] = {e.q0, e.q1, e.q2};
  float x0 = 0.0f, y0 = 0.0f, x1 = 0.0f, y1 = 0.0f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float px = pile[q[i]] - d.x, py = pile[q[i] + 1] - d.y;
    x0 += w0[i] * px;
    y0 += w0[i] * py;
    x1 += w1[i] * px;
    y1 += w1[i] * py;
  }
  float dydx0, dydy0, dydx1, dydy1, dydxp;
  if (e.kind == 2) {
    const bool second = y1 < y0;
    dydx0 = dydx1 = dydxp = 0.0f;
    dydy0 = second ? 0.0f : 1.0f;
    dydy1 = second ? 1.0f : 0.0f;
  } else {
    const float m = (y1 - y0) / (x1 - x0), u = (e.x - x0) / (x1 - x0);
    dydx0 = m * (u - 1.0f);
    dydy0 = 1.0f - u;
    dydx1 = -m * u;
    dydy1 = u;
    dydxp = m;
  }
  if (e.pt >= 0) {
    idx[0] = e.pt;
    val[0] = gx + gy * dydxp;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    idx[1 + 2 * i] = q[i];
    val[1 + 2 * i] = gy * (dydx0 * w0[i] + dydx1 * w1[i]);
    idx[2 + 2 * i] = q[i] + 1;
    val[2 + 2 * i] = gy * (dydy0 * w0[i] + dydy1 * w1[i]);
  }
}

struct AdjSlot {
  float4* thr;
  uint32_t* hdr;
  float4* thrFwd;  // the forward scan's copy of the sorted queue
  uint32_t* hdrFwd;
  int4* prov;
  LineRec* lines;
  float4* lineGrad;
  uint32_t* idx;
  float4* bitGrad;
  float4* layer;     // composited layers of the current section
  float4* front;     // the composite in front of each layer
  int32_t* layerBit;
  int cap;
  int layerCap;
  int ls;  // element stride of layer, front and layerBit: 32 on the device (a warp's lanes interleaved), 1 on a host
};

// The scan of K:1744-2028 with provenance.  grad == true (the kernel's second pass):
// read I(p), A(p) back from `image` and accumulate gradients; grad == false writes
// them instead (the kernel's first pass uses the raster scan for that).
template <int SECTIONS>
__device__ __forceinline__ void scanP(const RasterInputs& in, const ColumnState& c, AdjQueue& q, const AdjSlot& s,
                                      ShapeStack<SECTIONS>& stack, int bits, float4* image, const float4* target,
                                      bool grad, int& status) {
  int current = 0, numActive = 0;
  float sx0 = kLeft, sy0 = 0.0f, sx1 = kRight, sy1 = 0.0f;
  int32_t srcY0 = kConst, srcY1 = kConst, srcX0 = kConst, srcX1 = kConst;
  const int px = c.deltaX;
  int py = c.deltaY;
  // Section colours are memoised exactly as in the forward scan (the layers read
  // from the top down to `colorStop` only); while they hold, the colour gradient of
  // successive sections is linear in the same chain, so their areas are summed in
  // `chainArea` and the chain runs once per layer list and pixel.
  float4 col = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  bool colorOk = false, colorPositional = false;
  int colorStop = 0, K = 0;
  float chainArea = 0.0f;
  // invA: 1 / the pixel's section-area sum, taken once per pixel (the gradients need
  // no bit-exact match, only the forward image does)
  float gI[3] = {0.0f, 0.0f, 0.0f}, I[3] = {0.0f, 0.0f, 0.0f}, invA = 1.0f;
  // Geometry gradients are gathered per band: every section of a band shares its y
  // sources, and a threshold line is the right edge of one section and the left edge
  // of the next at the same mid-height, so its two contributions are summed
  // (pendCoef) and applied once.
  float gY0 = 0.0f, gY1 = 0.0f, pendCoef = 0.0f;
  // The chain's reverse pass is linear in the gradient of its result, so a pixel's
  // share (dL/dI times the area its sections took under this layer list, over the
  // pixel area) is folded into dP when the pixel ends, and the chain runs once per
  // layer list, when the list changes or the scan ends.
  float dP0 = 0.0f, dP1 = 0.0f, dP2 = 0.0f;
  auto foldPixel = [&]() {
    if (grad && chainArea != 0.0f) {
      const float w = chainArea * invA;
      dP0 += gI[0] * w;
      dP1 += gI[1] * w;
      dP2 += gI[2] * w;
    }
    chainArea = 0.0f;
  };
  auto flushChain = [&]() {
    foldPixel();
    if (grad && K > 0 && (dP0 != 0.0f || dP1 != 0.0f || dP2 != 0.0f)) {
      float4 d = make_float4(dP0, dP1, dP2, 0.0f);
      // The lanes flushing together walk their chains at the same depth k (a lane
      // idles above its own K), so their reads of the interleaved layer records share
      // lines.
#ifdef __CUDA_ARCH__
      const int kTop = __reduce_max_sync(__activemask(), K);
#else
      const int kTop = K;
#endif
      for (int k = kTop - 1; k >= 0; --k) {
        if (k >= K) continue;
        float4 df, db;
        compositeAdjoint(s.front[k * s.ls], s.layer[k * s.ls], d, df, db);
        const int32_t lb = s.layerBit[k * s.ls];
        if (lb >= 0 && (lb & kSolidLayer)) {
          float4& bg = s.bitGrad[lb & ~kSolidLayer];
          bg.x += db.x;
          bg.y += db.y;
          bg.z += db.z;
          bg.w += db.w;
        }
        d = df;
      }
    }
    dP0 = dP1 = dP2 = 0.0f;
  };
  // The rows and the sections of a row run as one loop (as in the forward scan,
  // renderColumnT): a step is the next section of the row or, once the row is
  // complete, its pixel's end and the next row's start.  Per column the operations
  // and their order are unchanged; across a warp, a lane whose row is short goes on to
  // its next row instead of waiting for the longest row.
  float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f, area = 0.0f;
  size_t pix = 0;
  int guard = 0;
  auto rowStart = [&]() {
    acc0 = acc1 = acc2 = area = 0.0f;
    if (colorPositional) colorOk = false;
    pix = (size_t)py * (size_t)in.bitmap_w + (size_t)px;
    if (grad) {
      const float4 im = image[pix], tg = target[pix];
      I[0] = im.x;
      I[1] = im.y;
      I[2] = im.z;
      invA = 1.0f / im.w;
      gI[0] = 2.0f * (im.x - tg.x);
      gI[1] = 2.0f * (im.y - tg.y);
      gI[2] = 2.0f * (im.z - tg.z);
    }
    guard = 0;
  };
  float pixelY = 1.0f;
  if (pixelY <= c.floatHeight) rowStart();
  while (pixelY <= c.floatHeight) {
    if ((sx1 < kRight) || (sy1 < pixelY)) {
      if (++guard > kSectionCap) {
        status |= kStatusIterLimit;
        return;
      }
      if (sx1 == kRight) {  // verticalAdvance K:1744-1824
        for (int i = 0; i < numActive; ++i) stack.pass(q.hdr[q.start + i]);
        const float nextBreak = cl_min(c.floatHeight, pixelY);
        const float activeBottom = q.length() > 0 ? q.thr[q.start].y : FLT_MAX;
        const int32_t activeSrc = q.length() > 0 ? q.prov[q.start].z : kConst;
        if (activeBottom == sy1) {
          while (numActive > 0) {
            stack.passBottom(q.hdr[q.start]);
            q.start += 1;
            numActive -= 1;
          }
        }
        float nextBottom;
        int32_t nextSrc;
        if (numActive > 0) {
          const bool brk = nextBreak < activeBottom;
          nextBottom = brk ? nextBreak : activeBottom;
          nextSrc = brk ? kConst : activeSrc;
        } else {
          const float nextTop = numActive < q.length() ? q.thr[q.start + numActive].x : FLT_MAX;
          const int32_t nextTopSrc = numActive < q.length() ? q.prov[q.start + numActive].y : kConst;
          if (nextTop > sy1) {
            const bool top = nextTop < nextBreak;
            nextBottom = top ? nextTop : nextBreak;
            nextSrc = top ? nextTopSrc : kConst;
          } else {
            // splitNext K:1069-1077
            float sp = FLT_MAX;
            int32_t spSrc = kConst;
            const float top0 = q.thr[q.start].x;
            int n = 1;
            while (n < q.length()) {
              if (q.thr[q.start + n].x > top0) {
                sp = q.thr[q.start + n].x;
                spSrc = q.prov[q.start + n].y;
                break;
              }
              n += 1;
            }
            numActive = n;
            float sp2 = sp;
            int32_t sp2Src = spSrc;
            for (int i = 0; i < n; ++i) {
              const float b = q.thr[q.start + i].y;
              if (top0 < b && b < sp2) {
                sp2 = b;
                sp2Src = q.prov[q.start + i].z;
              }
            }
            if (sp2 < sp) {
              sp = sp2;
              spSrc = sp2Src;
            }
            q.splitActive(n, sp, spSrc);
            if (q.overflow) return;
            const bool brk = sp < nextBreak;
            nextBottom = brk ? sp : nextBreak;
            nextSrc = brk ? spSrc : kConst;
            while (numActive > 0 && q.thr[q.start].x == q.thr[q.start].y) {
              stack.passTop(q.hdr[q.start]);
              q.start += 1;
              numActive -= 1;
            }
            for (int i = 0; i < numActive; ++i) {
              if (q.thr[q.start + i].x > 0.0f) stack.passTop(q.hdr[q.start + i]);
            }
          }
        }
        if (grad) {
          addY(s.lineGrad, srcY0, gY0);
          addY(s.lineGrad, srcY1, gY1);
          gY0 = gY1 = 0.0f;
        }
        sy0 = sy1;
        srcY0 = srcY1;
        sy1 = nextBottom;
        srcY1 = nextSrc;
        sx0 = sx1 = kLeft;
        srcX0 = srcX1 = kConst;
        current = 0;
      }
      // horizontalAdvance K:1826-1851 (thresholdMidXLow K:916-926)
      float nextX = kRight;
      int32_t nextXSrc = kConst;
      if (current < numActive) {
        const float4 e = q.thr[q.start + current];
        const float ym = sy0 + ((sy1 - sy0) * 0.5f);
        const float xx = intersectX(q.hdr[q.start + current], e, ym);
        if (xx >= kRight) {
          nextX = kLeft;
        } else if (kLeft < xx) {
          nextX = xx;
          nextXSrc = q.prov[q.start + current].x;
        } else {
          nextX = kLeft;
        }
      }
      sx0 = sx1;
      srcX0 = srcX1;
      sx1 = nextX;
      srcX1 = nextXSrc;
      if (!colorOk || stack.hiFlip >= colorStop) {
        flushChain();
        K = layersOf<SECTIONS>(in, stack, s.idx, px, py, bits, s.layer, s.front, s.layerBit, s.layerCap, s.ls, col,
                               colorPositional, colorStop, status);
        if (K < 0) {
          status |= kStatusIterLimit;
          return;
        }
        colorOk = true;
        stack.clearFlips();
      }
      const float a = (sx1 - sx0) * (sy1 - sy0);
      acc0 += col.x * a;
      acc1 += col.y * a;
      acc2 += col.z * a;
      area += a;
      if (grad) {
        // a = (x1 - x0)(y1 - y0): d/dx1 = w, d/dx0 = -w, d/dy1 = h, d/dy0 = -h
        const float dA = (gI[0] * (col.x - I[0]) + gI[1] * (col.y - I[1]) + gI[2] * (col.z - I[2])) * invA;
        const float w = sy1 - sy0, hgt = sx1 - sx0;
        gY0 -= dA * hgt;
        gY1 += dA * hgt;
        if (srcX0 >= 0) {  // the previous section's right edge: both contributions at once
          const float coef = pendCoef - dA * w;
          float dX[4], dXdy;
          if (lineX(s.lines[srcX0], sy0 + (sy1 - sy0) * 0.5f, dX, dXdy)) {
            float4& g = s.lineGrad[srcX0];
            g.x += coef * dX[0];
            g.y += coef * dX[1];
            g.z += coef * dX[2];
            g.w += coef * dX[3];
            gY0 += 0.5f * coef * dXdy;
            gY1 += 0.5f * coef * dXdy;
          }
        }
        pendCoef = dA * w;  // for srcX1, applied with the next section
        chainArea += a;  // colour: back through the composite chain at the next flush
      }
      if (current < numActive) stack.pass(q.hdr[q.start + current]);
      current += 1;
    } else {
      foldPixel();  // dL/dI changes with the pixel
      if (grad) {  // the row's last band
        addY(s.lineGrad, srcY0, gY0);
        addY(s.lineGrad, srcY1, gY1);
        gY0 = gY1 = 0.0f;
      }
      if (!grad) image[pix] = make_float4(acc0 / area, acc1 / area, acc2 / area, area);
      sx0 = kLeft;
      srcX0 = kConst;
      sy0 = pixelY;
      srcY0 = kConst;
      py += 1;
      pixelY += 1.0f;
      if (pixelY <= c.floatHeight) rowStart();
    }
  }
  flushChain();  // the last layer list
}

// The forward scan (renderColumn, writing the float image) of a sorted queue.
template <int SECTIONS>
__device__ __forceinline__ void forwardScan(const RasterInputs& in, const ColumnState& c, Queue& q,
                                            ShapeStack<SECTIONS>& stack, const AdjSlot& s, uint32_t bits,
                                            float4* image, int& status) {
  if (SECTIONS > 1 && bits <= 64) {
    ShapeStack<1> one;
    one.clear();
    one.w[0] = stack.word(0);
    one.nz = one.w[0] ? 1u : 0u;
    renderColumn<1>(in, c, q, one, s.idx, status, (int)bits, image);
  } else {
    renderColumn<SECTIONS>(in, c, q, stack, s.idx, status, (int)bits, image);
  }
}

// one column: float image, then gradients
// The column's lines and their gradients stay in the slot (nLines, nBits, delta out);
// the kernel carries them to the pile and the substances for the whole warp at once.
//
// By default the thresholds are generated once, with provenance: the forward scan
// runs on a copy of the sorted queue (the scan consumes its queue) and the gradient
// scan on the queue itself, so nothing outlives the work unit.  generateP makes the
// same thresholds in the same order as buildThresholds (the same decisions and
// arithmetic, with sources recorded beside them) and both sorts are stable under the
// same order, so the forward image is the raster kernel's.  With `regenerate` the
// forward pass generates its own thresholds (buildThresholds) and the gradient pass
// generates them again.
template <int SECTIONS>
__device__ bool adjointColumn(const RasterInputs& in, const gudni_tile_info& ti, int column, const AdjSlot& s,
                              float4* image, const float4* target, bool regenerate, int& nLines, int& nBits,
                              float2& delta, int& status) {
  nLines = 0;
  nBits = 0;
  const ColumnState c = initColumn(in, ti, column, in.job_index);
  if (!c.active) return false;
  AdjQueue q{s.thr, s.hdr, s.prov, s.cap, s.cap, false};
  int n_lines = 0;
  AdjGen g{&q, s.lines, &n_lines, s.cap, &c};
  ShapeStack<SECTIONS> stack;
  stack.clear();
  uint32_t bits = 0, fbits;
  Queue f{s.thrFwd, s.hdrFwd, s.cap, s.cap, false};  // the forward scan's queue
  if (regenerate) {  // the raster kernel's own generate and order
    fbits = buildThresholds<SECTIONS>(in, c, f, stack, s.idx, status);
    if (f.overflow) return true;
    sortQueue(f);
  } else {  // the thresholds with provenance, once; the forward scans a copy
    bits = fbits = generateP<SECTIONS>(in, c, g, stack, s.idx, status);
    if (q.overflow) return true;
    q.sort();
    for (int i = q.start; i < q.cap; ++i) {
      s.thrFwd[i] = s.thr[i];
      s.hdrFwd[i] = s.hdr[i];
    }
    f.start = q.start;
  }
  // The stack the generation left, for the gradient scan: kept in local memory while
  // the forward scan runs (a second stack in registers would spill in the scans).
  volatile uint64_t w0[SECTIONS];
#pragma unroll
  for (int k = 0; k < SECTIONS; ++k) w0[k] = stack.w[k];
  const uint32_t nz0 = stack.nz;
  const int hi0 = stack.hiFlip;
  // the forward: the float image (I rgb, section-area sum) instead of bytes
  forwardScan<SECTIONS>(in, c, f, stack, s, fbits, image, status);
  if (f.overflow) return true;
  if (regenerate) {  // the thresholds again, now with provenance
    stack.clear();
    bits = generateP<SECTIONS>(in, c, g, stack, s.idx, status);
    if (q.overflow) return true;
    q.sort();
  } else {
#pragma unroll
    for (int k = 0; k < SECTIONS; ++k) stack.w[k] = w0[k];
    stack.nz = nz0;
    stack.hiFlip = hi0;
  }
  // the gradients
  for (int i = 0; i < n_lines; ++i) s.lineGrad[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  for (uint32_t b = 0; b < bits; ++b) s.bitGrad[b] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (SECTIONS > 1 && bits <= 64) {  // as the forward scan: a one-word stack
    ShapeStack<1> one;
    one.clear();
    one.w[0] = stack.word(0);
    one.nz = one.w[0] ? 1u : 0u;
    scanP<1>(in, c, q, s, one, (int)bits, image, target, true, status);
  } else {
    scanP<SECTIONS>(in, c, q, s, stack, (int)bits, image, target, true, status);
  }
  if (q.overflow) return true;
  nLines = n_lines;
  nBits = (int)bits;
  delta = make_float2((float)c.deltaX, (float)c.deltaY);
  return false;
}

}  // namespace

}  // namespace gudni
