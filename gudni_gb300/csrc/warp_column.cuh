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

// Path counters for the host tests (empty in the CUDA build): which way splitNextWarp
// went, and how the parts were sorted.
#ifndef GUDNI_WARP_TRACE
#define GUDNI_WARP_TRACE(event)
#endif

namespace gudni {

enum WarpTraceEvent {
  kTraceSplitWarp = 0,   // splitNextWarp across the lanes
  kTraceSplitLane0 = 1,  // splitNextWarp on lane 0
  kTraceSortRounds = 2,  // parts sorted by transposition rounds
  kTraceSortLane0 = 3,   // parts sorted on lane 0
  kTraceTies = 4,        // parts with equal keys reordered
  kTraceEvents = 5
};

// Per-warp scratch in shared memory: one entry per lane.
struct WarpScratch {
  float4* prod;     // a chunk's section products (r, g, b, area)
  uint32_t* bit;    // a chunk's threshold shape bits
  uint32_t* flips;  // a set of shape-bit flips (kWarpFlipWords words)
};

constexpr int kWarpFlipWords = 64;  // 2 per stack word, up to 32 stack words

__device__ __forceinline__ uint64_t shflWord(uint64_t v, int src) {
  const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)v, src);
  const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(v >> 32), src);
  return ((uint64_t)hi << 32) | (uint64_t)lo;
}

// ---- shape-bit flips by the whole warp
//
// A set of flips is an XOR, so its order does not matter: the lanes mark their share
// of the flips in a per-warp bitset (2 words per stack word), then every lane folds the
// set into its copy of the stack.  `hiFlip` (the colour memo's test) takes the highest
// bit the set changes: a bit flipped twice is unchanged, and the memo depends only on
// the bits themselves.

__device__ __forceinline__ void flipClear(uint32_t* d, int words, int lane) {
  for (int w = lane; w < words; w += 32) d[w] = 0u;
  __syncwarp();
}

__device__ __forceinline__ void flipMark(uint32_t* d, uint32_t bit) {
  atomicXor(&d[bit >> 5], 1u << (bit & 31u));
}

template <int SECTIONS>
__device__ __forceinline__ void flipApply(const uint32_t* d, ShapeStack<SECTIONS>& s) {
  __syncwarp();
#pragma unroll
  for (int w = 0; w < SECTIONS; ++w) {
    const uint64_t m = ((uint64_t)d[2 * w + 1] << 32) | (uint64_t)d[2 * w];
    if (m) {
      s.w[w] ^= m;
      s.nz = s.w[w] ? (s.nz | (1u << w)) : (s.nz & ~(1u << w));
      s.hiFlip = max(s.hiFlip, w * 64 + 63 - __clzll((long long)m));
    }
  }
  __syncwarp();  // every lane has read the set before it is cleared again
}

// ---- splitNext by the whole warp

// splitNext on lane 0 (the per-lane code, raster_device.cuh), the other lanes taking
// its queue state.  Nothing may have changed the queue since the last barrier.
__device__ __forceinline__ float splitNextLane0(Queue& q, Parse& p, int lane) {
  if (lane == 0) GUDNI_WARP_TRACE(kTraceSplitLane0);
  __syncwarp();  // every lane is done reading the queue
  float slice = 0.0f;
  if (lane == 0) slice = splitNext(q, p);
  __syncwarp();  // lane 0's writes are visible
  slice = __shfl_sync(0xffffffffu, slice, 0);
  q.start = __shfl_sync(0xffffffffu, q.start, 0);
  q.overflow = __shfl_sync(0xffffffffu, q.overflow ? 1 : 0, 0) != 0;
  p.numActive = __shfl_sync(0xffffffffu, p.numActive, 0);
  return slice;
}

// The parts [lo, lo + m), in the order they were split off, into the order the per-lane
// code gives them: ascending (an entry goes after another only when it is strictly
// below it, thresholdIsBelow K:1079-1094), equal keys latest first.  A stable sort
// first -- odd-even transposition rounds across the lanes until a round swaps
// nothing, which the few line crossings inside one band keep short, or after
// `kSortRounds` rounds an insertion sort on lane 0 (a stable sort's result is unique)
// -- then each run of equal keys is reversed.
constexpr int kSortRounds = 16;

__device__ __forceinline__ bool sameKey(uint32_t ha, float4 ta, uint32_t hb, float4 tb) {
  return !isBelow(ha, ta, hb, tb) && !isBelow(hb, tb, ha, ta);
}

__device__ __forceinline__ void sortPartsWarp(Queue& q, int lo, int m, int lane) {
  bool sorted = false;
  for (int round = 0; round < kSortRounds && !sorted; ++round) {
    bool swapped = false;
    for (int phase = 0; phase < 2; ++phase) {
      for (int a = 2 * lane + phase; a + 1 < m; a += 64) {
        const uint32_t ha = q.hdr[lo + a], hb = q.hdr[lo + a + 1];
        const float4 ta = q.thr[lo + a], tb = q.thr[lo + a + 1];
        if (isBelow(ha, ta, hb, tb)) {
          q.hdr[lo + a] = hb;
          q.thr[lo + a] = tb;
          q.hdr[lo + a + 1] = ha;
          q.thr[lo + a + 1] = ta;
          swapped = true;
        }
      }
      __syncwarp();
    }
    sorted = __ballot_sync(0xffffffffu, swapped) == 0u;
  }
  if (lane == 0) {
    if (sorted) {
      GUDNI_WARP_TRACE(kTraceSortRounds);
    } else {
      GUDNI_WARP_TRACE(kTraceSortLane0);
      for (int i = lo + 1; i < lo + m; ++i) {
        const float4 t = q.thr[i];
        const uint32_t h = q.hdr[i];
        int j = i - 1;
        while (j >= lo && isBelow(q.hdr[j], q.thr[j], h, t)) {
          q.thr[j + 1] = q.thr[j];
          q.hdr[j + 1] = q.hdr[j];
          --j;
        }
        q.thr[j + 1] = t;
        q.hdr[j + 1] = h;
      }
    }
  }
  __syncwarp();
  // equal keys: latest first
  bool tie = false;
  for (int a = lane; a + 1 < m; a += 32) tie = tie || sameKey(q.hdr[lo + a], q.thr[lo + a], q.hdr[lo + a + 1], q.thr[lo + a + 1]);
  if (__ballot_sync(0xffffffffu, tie) != 0u) {
    if (lane == 0) {
      GUDNI_WARP_TRACE(kTraceTies);
      int a = 0;
      while (a < m) {
        int z = a + 1;
        while (z < m && sameKey(q.hdr[lo + z - 1], q.thr[lo + z - 1], q.hdr[lo + z], q.thr[lo + z])) ++z;
        for (int i = a, j = z - 1; i < j; ++i, --j) {
          const uint32_t h = q.hdr[lo + i];
          const float4 t = q.thr[lo + i];
          q.hdr[lo + i] = q.hdr[lo + j];
          q.thr[lo + i] = q.thr[lo + j];
          q.hdr[lo + j] = h;
          q.thr[lo + j] = t;
        }
        a = z;
      }
    }
    __syncwarp();
  }
}

// splitNext K:1069-1077 by the whole warp.  The band's end, the split of the active
// entries and the placing of their kept lower parts run across the lanes, producing
// the per-lane splitNext's queue entry for entry: the parts are sorted and merged
// with the entries of equal top after the active block (the per-lane merge path; with
// no NaN key involved it equals inserting the parts one by one).  Any case outside
// that (the literal path, a NaN key, more than 32 equal-top entries) runs the
// per-lane splitNext on lane 0 before anything is written.  Every lane returns the
// slice point with q.start and p.numActive updated.
__device__ __forceinline__ float splitNextWarp(Queue& q, Parse& p, int lane) {
  const unsigned full = 0xffffffffu;
  const int len = q.length();
  const int s0 = q.start;
  const float top = q.get(0).x;
  // the active block ends at the first entry whose top is above `top`
  int n = len;
  float slicePoint = FLT_MAX;
  for (int b = 1; b < len; b += 32) {
    const int i = b + lane;
    const float t = i < len ? q.get(i).x : 0.0f;
    const uint32_t above = __ballot_sync(full, i < len && t > top);
    if (above) {
      const int f = __ffs((int)above) - 1;
      n = b + f;
      slicePoint = __shfl_sync(full, t, f);
      break;
    }
  }
  // the nearest active bottom below `top`: cl_min keeps the earlier of equal values,
  // so the smallest (value, index), the next top (index -1) first
  float best = FLT_MAX;
  int bestAt = 0x7fffffff;
  for (int i = lane; i < n; i += 32) {
    const float bottom = q.get(i).y;
    if (top < bottom && bottom < best) {
      best = bottom;
      bestAt = i;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    const float ob = __shfl_xor_sync(full, best, off);
    const int oa = __shfl_xor_sync(full, bestAt, off);
    if (ob < best || (ob == best && oa < bestAt)) {
      best = ob;
      bestAt = oa;
    }
  }
  slicePoint = best < slicePoint ? best : slicePoint;
  // the per-lane code's batched case: room below the queue, every active top above
  // the slice point
  bool batched = s0 >= 2 * n;
  for (int b = 0; batched && b < n; b += 32) {
    const int i = b + lane;
    batched = __ballot_sync(full, i < n && !(q.get(i).x < slicePoint)) == 0u;
  }
  if (!batched) return splitNextLane0(q, p, lane);
  // read only: how many lower parts are kept, and whether a sort key is NaN
  int m = 0;
  bool nan = false;
  for (int b = 0; b < n; b += 32) {
    const int i = b + lane;
    bool keep = false, bad = false;
    if (i < n) {
      uint32_t ch = q.getH(i);
      float4 cur = q.get(i);
      if (cur.x < slicePoint && slicePoint < cur.y) {
        uint32_t sh;
        float4 split;
        splitAt(ch, cur, slicePoint, sh, split);
        keep = tKeep(sh, split);
        const float tx = tTopX(sh, split), sl = invSlope(sh, split);
        bad = keep && !(tx == tx && sl == sl);
      }
    }
    m += __popc(__ballot_sync(full, keep));
    nan = nan || __ballot_sync(full, bad) != 0u;
  }
  // the entries of top == slicePoint right after the active block, and the one after
  int g = 0;
  bool mergeable = !nan;
  for (int b = 0; m > 0 && mergeable; b += 32) {
    const int r = s0 + n + b + lane;
    bool eq = false, bad = false;
    if (r < q.cap) {
      const float4 t = q.thr[r];
      eq = t.x == slicePoint;
      if (eq) {
        const uint32_t h = q.hdr[r];
        const float tx = tTopX(h, t), sl = invSlope(h, t);
        bad = !(tx == tx && sl == sl);
      }
    }
    const uint32_t noteq = ~__ballot_sync(full, eq);
    const int run = noteq ? __ffs((int)noteq) - 1 : 32;
    mergeable = __ballot_sync(full, lane < run && bad) == 0u;
    g += run;
    if (g > 32) mergeable = false;
    if (run < 32) {
      const int rEnd = s0 + n + g;
      if (mergeable && rEnd < q.cap) mergeable = q.thr[rEnd].x > slicePoint;
      break;
    }
  }
  if (m > 0 && !mergeable) return splitNextLane0(q, p, lane);
  if (lane == 0) GUDNI_WARP_TRACE(kTraceSplitWarp);
  p.numActive = n;
  __syncwarp();  // every lane is done reading before the queue changes
  // split in place; kept part j (in cursor order) to s0 - n - m + j
  int j0 = 0;
  for (int b = 0; b < n; b += 32) {
    const int i = b + lane;
    bool keep = false;
    uint32_t sh = 0u;
    float4 split = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (i < n) {
      uint32_t ch = q.hdr[s0 + i];
      float4 cur = q.thr[s0 + i];
      if (cur.x < slicePoint && slicePoint < cur.y) {
        splitAt(ch, cur, slicePoint, sh, split);
        q.hdr[s0 + i] = ch;
        q.thr[s0 + i] = cur;
        keep = tKeep(sh, split);
      }
    }
    const uint32_t kept = __ballot_sync(full, keep);
    if (keep) {
      const int j = j0 + __popc(kept & ((1u << lane) - 1u));
      q.hdr[s0 - n - m + j] = sh;
      q.thr[s0 - n - m + j] = split;
    }
    j0 += __popc(kept);
  }
  __syncwarp();
  if (m == 0) return slicePoint;
  // the active block moves down by m (each chunk read before it is written; a chunk's
  // destinations lie below the next chunk's sources)
  for (int b = 0; b < n; b += 32) {
    const int i = b + lane;
    uint32_t h = 0u;
    float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (i < n) {
      h = q.hdr[s0 + i];
      t = q.thr[s0 + i];
    }
    __syncwarp();
    if (i < n) {
      q.hdr[s0 - m + i] = h;
      q.thr[s0 - m + i] = t;
    }
  }
  q.start = s0 - m;
  // the parts, in cursor order at [lo, lo + m), into the per-lane order
  const int lo = s0 - n - m;
  sortPartsWarp(q, lo, m, lane);
  // merge with the g equal-top entries: an entry goes ahead of a part only when the
  // part is strictly below it.  Entry r is preceded by the parts not below it (a
  // prefix of the sorted parts); part k by the entries whose prefix ends at or
  // before k.
  const int out = s0 - m + n;
  uint32_t eh = 0u;
  float4 et = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  int ahead = 0;
  if (lane < g) {
    eh = q.hdr[s0 + n + lane];
    et = q.thr[s0 + n + lane];
    int a = 0, z = m;  // first part strictly below the entry
    while (a < z) {
      const int mid = (a + z) >> 1;
      if (isBelow(q.hdr[lo + mid], q.thr[lo + mid], eh, et)) {
        z = mid;
      } else {
        a = mid + 1;
      }
    }
    ahead = a;
  }
  __syncwarp();  // the entries are read before the parts may land on their places
  if (lane < g) {
    q.hdr[out + lane + ahead] = eh;
    q.thr[out + lane + ahead] = et;
  }
  for (int b = 0; b < m; b += 32) {
    const int k = b + lane;
    int before = 0;
    for (int r = 0; r < g; ++r) before += __shfl_sync(full, ahead, r) <= k ? 1 : 0;
    if (k < m) {
      q.hdr[out + k + before] = q.hdr[lo + k];
      q.thr[out + k + before] = q.thr[lo + k];
    }
  }
  __syncwarp();
  return slicePoint;
}

// verticalAdvance K:1744-1824 by the whole warp, at a band's end (p.sEndX == kRight).
// The stack flips of each step are applied as one set; the queue changes only in
// splitNextWarp.
template <int SECTIONS>
__device__ __forceinline__ void verticalAdvanceWarp(Queue& q, const ColumnState& c, Parse& p,
                                                    ShapeStack<SECTIONS>& stack, int lane, uint32_t* flips) {
  const int n0 = p.numActive;
  const float activeBottom = q.length() > 0 ? q.get(0).y : FLT_MAX;
  const bool dropAll = activeBottom == p.sEndY;
  if (n0 > 0) {
    // every active threshold is passed; when the band ended at their bottom they are
    // dropped, the persistent bottoms passed again (two flips of one bit cancel)
    flipClear(flips, 2 * SECTIONS, lane);
    for (int i = lane; i < n0; i += 32) {
      const uint32_t h = q.getH(i);
      if (!(dropAll && hPersistBottom(h))) flipMark(flips, h & kShapeBitMask);
    }
    flipApply<SECTIONS>(flips, stack);
    if (dropAll) {
      q.start += n0;
      p.numActive = 0;
    }
  }
  const float nextBreak = cl_min(c.floatHeight, p.pixelY);
  float nextBottom;
  if (p.numActive > 0) {
    nextBottom = cl_min(activeBottom, nextBreak);
  } else {
    const float nextTop = q.length() > 0 ? q.get(0).x : FLT_MAX;
    if (nextTop > p.sEndY) {
      nextBottom = cl_min(nextBreak, nextTop);
    } else {
      nextBottom = cl_min(nextBreak, splitNextWarp(q, p, lane));
      // leading zero-height entries are dropped (their persistent tops passed), then
      // the persistent tops of the active entries below the column top are passed
      int lead = p.numActive;
      for (int b = 0; b < p.numActive; b += 32) {
        const int i = b + lane;
        bool flat = true;
        if (i < p.numActive) {
          const float4 t = q.get(i);
          flat = t.x == t.y;
        }
        const uint32_t notFlat = __ballot_sync(0xffffffffu, !flat);
        if (notFlat) {
          lead = b + __ffs((int)notFlat) - 1;
          break;
        }
      }
      flipClear(flips, 2 * SECTIONS, lane);
      for (int i = lane; i < p.numActive; i += 32) {
        const uint32_t h = q.getH(i);
        if (hPersistTop(h) && (i < lead || q.get(i).x > 0.0f)) flipMark(flips, h & kShapeBitMask);
      }
      flipApply<SECTIONS>(flips, stack);
      q.start += lead;
      p.numActive -= lead;
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
      verticalAdvanceWarp<SECTIONS>(q, c, p, stack, lane, ws.flips);
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
