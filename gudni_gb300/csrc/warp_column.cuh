// Warp-cooperative scan of dense columns.
//
// The reference scans a column in one work item: a serial sweep band by band
// (verticalAdvance, K:1744-1824) and section by section (horizontalAdvance,
// K:1826-1851), a shape-stack colour walk per section (sectionColor, K:1724-1742) and
// one running sum per pixel (renderThresholdArray, K:1978-2028).  In canvas-wide
// dense scenes a column holds hundreds of thresholds and one pixel row hundreds of
// thousands of sections, so the longest lane's chain decides a launch, and 32 such
// chains in one warp diverge and keep 32 queues live at once.
//
// Here the lanes of a warp first generate and sort their own columns as before.  The
// columns whose queues are long (at least `denseMin` entries) are then scanned one at
// a time by the whole warp:
//  * the band step keeps the serial order of operations.  Every lane holds its own
//    copy of the column's shape stack and applies the same flips; the one queue
//    mutation (splitNext) runs on lane 0 between two warp barriers, and the other lanes
//    take its queue state by shuffle;
//  * a band's sections are dealt to the lanes 32 at a time.  Section k sees the band's
//    stack with the flips of thresholds 0..k-1, so lane j applies the flips of the
//    chunk's thresholds ahead of its section, takes the section's colour (with its
//    own opaque-cut memo) and area, then applies the rest of the chunk's flips, after
//    which all copies agree again;
//  * the pixel sums take the sections' products in section order: every lane adds the
//    chunk's products one after another, so each floating-point operation is the
//    serial scan's, and the pixel is the serial scan's bit for bit.
//
// All lanes of the warp call these functions together (full-mask collectives).

#pragma once

#include "raster_device.cuh"

namespace gudni {

// Per-warp scratch in shared memory: one entry per lane.
struct WarpScratch {
  float4* prod;   // a chunk's section products (r, g, b, area)
  uint32_t* bit;  // a chunk's threshold shape bits
};

__device__ __forceinline__ uint64_t shflWord(uint64_t v, int src) {
  const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src);
  const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
  return ((uint64_t)hi << 32) | (uint64_t)lo;
}

// verticalAdvance K:1744-1824 by the whole warp, at a band's end (p.sEndX == kRight).
// Every lane runs the same steps on its copy of the stack; only splitNext writes the
// queue, on lane 0.
template <int SECTIONS>
__device__ __forceinline__ void verticalAdvanceWarp(Queue& q, const ColumnState& c, Parse& p,
                                                    ShapeStack<SECTIONS>& stack, int lane) {
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
      __syncwarp();  // every lane is done reading the queue
      float slice = 0.0f;
      if (lane == 0) slice = splitNext(q, p);
      __syncwarp();  // lane 0's writes are visible
      slice = __shfl_sync(0xffffffffu, slice, 0);
      q.start = __shfl_sync(0xffffffffu, q.start, 0);
      q.overflow = __shfl_sync(0xffffffffu, q.overflow ? 1 : 0, 0) != 0;
      p.numActive = __shfl_sync(0xffffffffu, p.numActive, 0);
      nextBottom = cl_min(nextBreak, slice);
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

// renderThresholdArray K:1978-2028 for one column by the whole warp; the BGRA word of
// each pixel is written by lane 0.
template <int SECTIONS>
__device__ __forceinline__ void renderColumnWarp(const RasterInputs& in, const ColumnState& c, Queue& q,
                                                 ShapeStack<SECTIONS>& stack, const uint32_t* shapeIdx,
                                                 int& status, int shapeBits, int lane, WarpScratch ws) {
  Parse p;
  p.current = 0;
  p.numActive = 0;
  p.sStartX = kLeft;
  p.sStartY = 0.0f;
  p.sEndX = kRight;
  p.sEndY = 0.0f;
  int cursor = 0;
  if (in.stochastic != 0.0f && in.random_field) {  // initRandomField K:1597-1606
    cursor = (int)(__float_as_uint(in.random_field[c.threadUnique & (GUDNI_RANDOM_FIELD_SIZE - 1)]) &
                   (GUDNI_RANDOM_FIELD_SIZE - 1));
  }
  const int px = c.deltaX;
  int py = c.deltaY;
  uint32_t* outp = in.out + (size_t)c.deltaY * (size_t)in.bitmap_w + (size_t)c.deltaX;
  int64_t sections = 0;
  int64_t texels = 0;
  // this lane's section-colour memo (exact, as in renderColumn)
  float4 color = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  bool colorOk = false;
  bool colorPositional = false;
  int colorStop = 0;
  for (p.pixelY = 1.0f; p.pixelY <= c.floatHeight; p.pixelY += 1.0f) {
    if (colorPositional) colorOk = false;
    float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f, acc4 = 0.0f;
    int guard = 0;
    while ((p.sEndX < kRight) || (p.sEndY < p.pixelY)) {
      verticalAdvanceWarp<SECTIONS>(q, c, p, stack, lane);
      if (q.overflow) return;
      const int n = p.numActive;  // the band has n + 1 sections
      if (n + 1 > kSectionCap - guard) {
        status |= kStatusIterLimit;
        return;
      }
      guard += n + 1;
      const float yMid = p.sStartY + ((p.sEndY - p.sStartY) * 0.5f);
      const float height = p.sEndY - p.sStartY;
      float xBefore = kLeft;  // where the chunk's first section starts
      for (int base = 0; base <= n; base += 32) {
        const int count = min(32, n + 1 - base);  // sections in the chunk
        const int flips = min(32, n - base);      // thresholds in the chunk
        const int k = base + lane;
        // horizontalAdvance: section k ends at threshold k's crossing of the band's
        // middle (thresholdMidXLow K:916-926), the band's last one at the right border
        float xEnd = kRight;
        uint32_t bit = 0u;
        if (k < n) {
          const float4 t = q.get(k);
          const uint32_t h = q.getH(k);
          const float x = intersectX(h, t, yMid);
          xEnd = x >= kRight ? kLeft : cl_max(kLeft, x);
          bit = h & kShapeBitMask;
        }
        float xStart = __shfl_up_sync(0xffffffffu, xEnd, 1);
        if (lane == 0) xStart = xBefore;
        ws.bit[lane] = bit;
        __syncwarp();
        for (int j = 0; j < lane && j < flips; ++j) stack.flip(ws.bit[j]);
        float4 prod = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (lane < count) {
          if (!colorOk || stack.hiFlip >= colorStop) {
            color = determineColor(in, stack, shapeIdx, px, py, status, texels, shapeBits, colorPositional,
                                   colorStop);
            colorOk = true;
            stack.clearFlips();
          }
          float area = (xEnd - xStart) * height;
          if (in.stochastic != 0.0f) {  // getRandom K:1608-1613, one step per section
            const int at = (cursor + lane + 1) & (GUDNI_RANDOM_FIELD_SIZE - 1);
            const float random = in.random_field ? in.random_field[at] : 0.0f;
            area = area + (area * random * in.stochastic);
          }
          prod = make_float4(color.x * area, color.y * area, color.z * area, area);
        }
        for (int j = lane; j < flips; ++j) stack.flip(ws.bit[j]);
        ws.prod[lane] = prod;
        __syncwarp();
        for (int j = 0; j < count; ++j) {
          const float4 v = ws.prod[j];
          acc0 += v.x;
          acc1 += v.y;
          acc2 += v.z;
          acc4 += v.w;
        }
        xBefore = __shfl_sync(0xffffffffu, xEnd, 31);
        if (in.stochastic != 0.0f) cursor = (cursor + count) & (GUDNI_RANDOM_FIELD_SIZE - 1);
        sections += count;
        __syncwarp();  // every lane has read the scratch before the next chunk writes it
      }
      p.sEndX = kRight;
      p.current = n + 1;
    }
    if (lane == 0) {
      const float r = acc0 / acc4, g = acc1 / acc4, b = acc2 / acc4;
      *outp = toByte(b * 255.0f) | (toByte(g * 255.0f) << 8) | (toByte(r * 255.0f) << 16) | (255u << 24);
    }
    outp += in.bitmap_w;
    p.sStartX = kLeft;
    p.sStartY = p.pixelY;
    py += 1;
  }
  if (in.counters) {
    if (lane == 0) atomicAdd(reinterpret_cast<unsigned long long*>(&in.counters[0]), (unsigned long long)sections);
    if (texels) atomicAdd(reinterpret_cast<unsigned long long*>(&in.counters[1]), (unsigned long long)texels);
  }
}

constexpr int kUnitOverflow = 1;  // the lane's column overflowed `cap`
constexpr int kUnitByWarp = 2;    // the lane's column was scanned by the whole warp

// The columns of one work unit (column = chunk * 32 + lane; `live` when the lane has
// one): each lane generates and sorts its own column; short queues are scanned by
// their lane, queues of at least `denseMin` entries by the whole warp, one column
// after another.  Returns kUnit* flags for this lane's column.
template <int SECTIONS>
__device__ __forceinline__ int runUnitWarp(const RasterInputs& in, const gudni_tile_info& ti, int column,
                                            bool live, float4* thr, uint32_t* hdr, int cap, uint32_t* idx,
                                            int& status, int lane, int denseMin, WarpScratch ws) {
  ColumnState c;
  c.active = false;
  if (live) c = initColumn(in, ti, column, in.job_index);
  Queue q{thr, hdr, cap, cap, false};
  ShapeStack<SECTIONS> mine;
  mine.clear();
  uint32_t bits = 0;
  bool dense = false;
  if (c.active) {
    bits = buildThresholds<SECTIONS>(in, c, q, mine, idx, status);
    if (!q.overflow) {
      sortQueue(q);
      if (in.counters) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&in.counters[2]), (unsigned long long)q.length());
        atomicMax(reinterpret_cast<unsigned long long*>(&in.counters[3]), (unsigned long long)bits);
      }
      dense = q.length() >= denseMin;
      if (!dense) {
        if (SECTIONS > 1 && bits <= 64) {
          ShapeStack<1> one;
          one.clear();
          one.w[0] = mine.word(0);
          one.nz = one.w[0] ? 1u : 0u;
          renderColumn<1>(in, c, q, one, idx, status, (int)bits);
        } else {
          renderColumn<SECTIONS>(in, c, q, mine, idx, status, (int)bits);
        }
      }
    }
  }
  uint32_t owners = __ballot_sync(0xffffffffu, dense);
  __syncwarp();  // every lane's queue is in memory before the others read it
  while (owners) {
    const int o = __ffs((int)owners) - 1;
    owners &= owners - 1u;
    const ColumnState oc = initColumn(in, ti, __shfl_sync(0xffffffffu, column, o), in.job_index);
    Queue oq;
    oq.thr = reinterpret_cast<float4*>(shflWord(reinterpret_cast<uint64_t>(thr), o));
    oq.hdr = reinterpret_cast<uint32_t*>(shflWord(reinterpret_cast<uint64_t>(hdr), o));
    oq.start = __shfl_sync(0xffffffffu, q.start, o);
    oq.cap = cap;
    oq.overflow = false;
    const uint32_t* oIdx = reinterpret_cast<const uint32_t*>(shflWord(reinterpret_cast<uint64_t>(idx), o));
    const int oBits = __shfl_sync(0xffffffffu, (int)bits, o);
    if (SECTIONS > 1 && oBits <= 64) {
      ShapeStack<1> s;
      s.clear();
      s.w[0] = shflWord(mine.word(0), o);
      s.nz = s.w[0] ? 1u : 0u;
      renderColumnWarp<1>(in, oc, oq, s, oIdx, status, oBits, lane, ws);
    } else {
      ShapeStack<SECTIONS> s;
      s.clear();
#pragma unroll
      for (int w = 0; w < SECTIONS; ++w) s.w[w] = shflWord(mine.word(w), o);
      s.nz = __shfl_sync(0xffffffffu, mine.nz, o);
      renderColumnWarp<SECTIONS>(in, oc, oq, s, oIdx, status, oBits, lane, ws);
    }
    // a split part that found no room: the owner's column goes to the full-capacity
    // pass, as from the per-lane scan
    if (oq.overflow && lane == o) q.overflow = true;
  }
  return (c.active && q.overflow ? kUnitOverflow : 0) | (dense ? kUnitByWarp : 0);
}

}  // namespace gudni
