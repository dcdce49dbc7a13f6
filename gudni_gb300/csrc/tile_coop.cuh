// Warp-cooperative generation of a work unit's thresholds (sm_103a).
//
// The reference generates each column's thresholds in its own work item
// (generateThresholds, Kernels.cl:2030-2082): every column walks every strand of its
// tile's shapes, and only the few columns a strand crosses do the tree search and the
// curve halving (buildThresholdArray / traverseTree / spawnThresholds, K:1264-1595).
// Run per lane, a warp of 32 columns walks each strand together and, for a glyph-sized
// strand crossing two or three columns, leaves most lanes idle through the expensive
// part.
//
// Here the 32 lanes of a warp share the unit's generation:
//  * the tile's shape records are staged into shared memory with one bulk copy
//    (cp.async.bulk, completed on an mbarrier);
//  * lanes take the tile's strands 32 at a time (strand table rows: one coalesced
//    load) and each finds, exactly, the interval of the unit's columns its strand's
//    range test passes (the test is monotone in the column position, so two binary
//    searches over the column positions give the columns the per-column test would);
//  * the (strand, column) pairs are dealt to the lanes 32 at a time; a lane runs the
//    per-column code on its pair (strandThresholds: tree search, halving, spawning,
//    y culling) into a three-entry sink;
//  * the thresholds are binned to their columns by warp ballots: lanes holding
//    thresholds of the same column find each other with __match_any_sync, and the
//    prefix of the peers' counts (two ballots of the count bits) places each
//    threshold at its position in the column's push order.  Pairs are dealt in
//    strand order, so that order is the per-column code's order of pushes, and each
//    column's slab ends up holding, entry for entry, the queue the per-column
//    generation builds (newest push first, K:1096-1103);
//  * per column, the enclosure parity of each shape is gathered with shared-memory
//    atomics; the column's shape bits are the tile's shape numbers (the per-column
//    code numbers only the shapes that touch the column, K:1586-1593, in the same
//    order, and the scan depends on the bits only through their order), so the
//    colour walk reads each layer's tag straight from the staged shape records; the
//    lane sorts and scans its queue with the per-column code;
//  * the unit's pixels go to a shared-memory tile and leave as whole rows: one bulk
//    copy per 128-byte row (cp.async.bulk shared -> global) where the row is complete
//    and aligned, else plain stores.
//
// A unit qualifies when its tile has at most 64 shapes and no more than max_shape
// (so no column can reach the MAXSHAPE cut-off and every shape bit fits one stack
// word), every shape has its strands in the strand table, and the tile is no wider
// than the threads per tile; other units run the per-column code on their lanes.
// Overflowing columns go to the full-capacity pass as before.
//
// All lanes of the warp call these functions together (full-mask collectives).

#pragma once

#include "raster_device.cuh"

namespace gudni {

constexpr int kCoopMaxShapes = 64;
constexpr int kCoopStageRows = 32;  // pixel rows staged per unit (one 32-column slab)

// Per-warp shared memory of the cooperative unit.
struct CoopShared {
  gudni_shape shapes[kCoopMaxShapes];  // staged shape records (16-byte aligned: first member)
  uint32_t stage[kCoopStageRows * 32]; // the unit's pixels, 32 per row
  unsigned long long encl[32];         // per column: enclosure parity per tile shape index
  unsigned long long added[32];        // per column: shapes that pushed a threshold
  uint4 sTab[32];                      // the strand batch's table rows
  float2 sY[32];                       // and y ranges
  uint32_t strandBase[kCoopMaxShapes + 1];  // exclusive prefix of strands per shape
  uint32_t strandFirst[kCoopMaxShapes];     // strand-table index of each shape's first strand
  uint32_t colCount[32];               // thresholds pushed per column
  uint32_t pairEnd[32];                // inclusive prefix of the batch's pair counts
  int sShape[32], sX0[32], sNx[32];    // the batch's strands: shape, first column, columns
  unsigned long long mbar;             // completion barrier of the shape copy
};

// The few thresholds one strand spawns in one column (spawnThresholds pushes at most
// three: the two wings and the bridge).
struct PairSink {
  float4 t0, t1, t2;
  uint32_t h0, h1, h2;
  int n;
  bool overflow;
  __device__ __forceinline__ void push(uint32_t h, float4 t) {
    if (n == 0) {
      h0 = h;
      t0 = t;
    } else if (n == 1) {
      h1 = h;
      t1 = t;
    } else if (n == 2) {
      h2 = h;
      t2 = t;
    } else {
      overflow = true;  // cannot happen; the column is then redone by the full pass
      return;
    }
    ++n;
  }
};

// ---- bulk copies (the host build of this header, for the CPU tests, copies plainly)

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__cvta_generic_to_shared(p);
#else
  return (uint32_t)(uintptr_t)p;
#endif
}

__device__ __forceinline__ void mbarInit(unsigned long long* bar) {
#ifdef __CUDA_ARCH__
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemAddr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
#else
  *bar = 0;
#endif
}

// Copy `bytes` (a multiple of 16, both addresses 16-byte aligned) from global to
// shared memory with one bulk copy issued by lane 0; every lane waits for it.  `phase`
// is the barrier's parity (bit 0) and a "bulk copies off" flag (bit 1).  The wait is
// bounded: on timeout the kernel's status records it, the copy still in flight is
// waited for (bounded again), bulk copies are switched off for the rest of the
// launch (the barrier's phase is no longer known) and false is returned, so that the
// caller reads the records from global memory instead.
__device__ __forceinline__ bool bulkLoad(void* dst, const void* src, uint32_t bytes, unsigned long long* bar,
                                        uint32_t& phase, int lane, int& status) {
#ifdef __CUDA_ARCH__
  if (lane == 0) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier reads of dst first
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smemAddr(dst)),
        "l"(src), "r"(bytes), "r"(smemAddr(bar))
        : "memory");
  }
  bool done = false;
  for (int spin = 0; spin < (1 << 22) && !done; ++spin) {
    uint32_t ok = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smemAddr(bar)), "r"(phase)
        : "memory");
    done = ok != 0;
  }
  const bool all = __all_sync(0xffffffffu, done);
  if (!all) {
    status |= kStatusIterLimit;
    phase |= 2u;
    // the copy is still in flight: give it a last bounded wait before the buffer is
    // abandoned for this unit
    for (int spin = 0; spin < (1 << 22) && !done; ++spin) {
      uint32_t ok = 0;
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
          : "=r"(ok)
          : "r"(smemAddr(bar)), "r"(phase)
          : "memory");
      done = ok != 0;
    }
    __syncwarp();
    return false;
  }
  phase ^= 1u;
  __syncwarp();
  return true;
#else
  (void)bar;
  (void)status;
  if (lane == 0) {
    const uint8_t* s = static_cast<const uint8_t*>(src);
    uint8_t* d = static_cast<uint8_t*>(dst);
    for (uint32_t i = 0; i < bytes; ++i) d[i] = s[i];
  }
  phase ^= 1u;
  __syncwarp();
  return true;
#endif
}

// One 128-byte row of the staged tile to global memory (both 16-byte aligned), as a
// bulk copy of this lane's bulk group; the source is read before bulkStoreWait
// returns.
__device__ __forceinline__ void bulkStoreRow(uint32_t* dst, const uint32_t* src) {
#ifdef __CUDA_ARCH__
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], 128;" ::"l"(dst), "r"(smemAddr(src))
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
#else
  for (int i = 0; i < 32; ++i) dst[i] = src[i];
#endif
}

// Every bulk store this lane issued has finished reading shared memory.
__device__ __forceinline__ void bulkStoreWait() {
#ifdef __CUDA_ARCH__
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
#endif
}

// Every bulk store this lane issued is complete.
__device__ __forceinline__ void bulkStoreDrain() {
#ifdef __CUDA_ARCH__
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
#endif
}

// Shared-memory writes of this thread are visible to the bulk-copy (async) proxy.
__device__ __forceinline__ void fenceProxyAsync() {
#ifdef __CUDA_ARCH__
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
#endif
}

// ---- the unit

constexpr int kCoopOverflow = 1;  // the lane's column needs the full-capacity pass
constexpr int kCoopNotTaken = 2;  // the unit does not qualify: run the per-column code

// Inclusive warp scan of v.
__device__ __forceinline__ uint32_t warpScan(uint32_t v, int lane) {
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t o = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) v += o;
  }
  return v;
}

// First i in [lo, hi) with pred(i), else hi (pred false then true over the range).
template <class P>
__device__ __forceinline__ int firstTrue(int lo, int hi, P pred) {
  while (lo < hi) {
    const int mid = lo + ((hi - lo) >> 1);
    if (pred(mid)) {
      hi = mid;
    } else {
      lo = mid + 1;
    }
  }
  return lo;
}

// The unit's staged pixels to the output: whole 128-byte rows by bulk copies when all
// 32 columns were rendered and the rows are 16-byte aligned, else each rendered
// column's pixels by plain stores.  `rendered`: this lane's column was scanned into
// the stage.
__device__ __forceinline__ void storeStagedUnit(const RasterInputs& in, const ColumnState& c, bool rendered,
                                                int lane, CoopShared& sh) {
  const unsigned full = 0xffffffffu;
  fenceProxyAsync();
  __syncwarp();
  const bool all = __all_sync(full, rendered);
  const int rows = __shfl_sync(full, c.intHeight, 0);
  const int x0 = __shfl_sync(full, c.deltaX, 0);
  const int y0 = __shfl_sync(full, c.deltaY, 0);
  uint32_t* row0 = in.out + (size_t)y0 * (size_t)in.bitmap_w + (size_t)x0;
  const bool aligned = ((uintptr_t)row0 & 15u) == 0 && ((size_t)in.bitmap_w * 4u) % 16u == 0;
  if (all && aligned) {
    if (lane < rows) bulkStoreRow(row0 + (size_t)lane * (size_t)in.bitmap_w, sh.stage + lane * 32);
    bulkStoreWait();
  } else if (rendered) {
    uint32_t* o = in.out + (size_t)c.deltaY * (size_t)in.bitmap_w + (size_t)c.deltaX;
    for (int r = 0; r < c.intHeight; ++r) o[(size_t)r * (size_t)in.bitmap_w] = sh.stage[r * 32 + lane];
  }
  __syncwarp();  // the stage is free for the next unit
}

// The columns of unit `chunk` of tile `ti` (column = chunk * 32 + lane), generated by
// the whole warp, then each sorted and scanned by its lane.  thrWarp / hdrWarp are
// the warp's 32 scratch slots (lane L's queue at L * cap).
// `stage`: write the pixels into sh.stage and store them by rows (single-slab units
// of at most 32 rows).  Returns kCoop* flags for this lane; with kCoopNotTaken
// nothing was written.
__device__ __forceinline__ int runUnitCoop(const RasterInputs& in, const gudni_tile_info& ti, int chunk, int lane,
                                           float4* thrWarp, uint32_t* hdrWarp, int cap, int& status,
                                           CoopShared& sh, uint32_t& phase) {
  const unsigned full = 0xffffffffu;
  const int numShapes = (int)ti.shapes.length;
  const int tpt = 1 << in.log2_tpt;
  const int hDepth = ti.hdepth;
  if (!in.strand_table || numShapes > kCoopMaxShapes || numShapes > in.max_shape || hDepth > in.log2_tpt)
    return kCoopNotTaken;
  const int W = 1 << hDepth;  // x-columns of the tile
  const int unitW = W < 32 ? W : 32;
  const int xbase = W >= 32 ? ((chunk * 32) & (W - 1)) : 0;
  const int nslab = W >= 32 ? 1 : (tpt < 32 ? tpt : 32) / W;
  const int column = chunk * 32 + lane;
  const bool live = column < tpt;
  ColumnState c;
  c.active = false;
  c.deltaX = c.deltaY = 0;
  c.floatHeight = 0.0f;
  c.intHeight = 0;
  if (live) c = initColumn(in, ti, column, in.job_index);

  // the tile's shape records: one bulk copy when the source is 16-byte aligned
  const gudni_shape* src = in.shapes + ti.shapes.start;
  bool staged = false;
  if (numShapes > 0 && ((uintptr_t)src & 15u) == 0 && (phase & 2u) == 0)
    staged = bulkLoad(sh.shapes, src, (uint32_t)numShapes * (uint32_t)sizeof(gudni_shape), &sh.mbar, phase, lane,
                      status);
  // per shape: its strands in the strand table
  bool bad = false;
  uint32_t cnt0 = 0, cnt1 = 0;
  for (int n = lane; n < kCoopMaxShapes; n += 32) {
    uint32_t count = 0;
    if (n < numShapes) {
      const gudni_shape s = staged ? sh.shapes[n] : src[n];
      const uint32_t first = s.geo_start < in.n_units ? in.strand_first[s.geo_start] : kNoStrand;
      if (first == kNoStrand || (uint64_t)first + s.num_strands > in.n_strands) bad = true;
      sh.strandFirst[n] = first;
      count = s.num_strands;
    }
    if (n < 32) cnt0 = count; else cnt1 = count;
  }
  if (__any_sync(full, bad)) return kCoopNotTaken;
  const uint32_t inc0 = warpScan(cnt0, lane);
  const uint32_t tot0 = __shfl_sync(full, inc0, 31);
  const uint32_t inc1 = warpScan(cnt1, lane) + tot0;
  sh.strandBase[lane] = inc0 - cnt0;
  sh.strandBase[32 + lane] = inc1 - cnt1;
  const uint32_t S = __shfl_sync(full, inc1, 31);
  if (lane == 0) sh.strandBase[kCoopMaxShapes] = S;
  sh.colCount[lane] = 0u;
  sh.encl[lane] = 0ull;
  sh.added[lane] = 0ull;
  __syncwarp();

  bool sinkOverflow = false;
  for (uint32_t s0 = 0; s0 < S; s0 += 32) {
    // ---- this lane's strand: its shape, table row and interval of unit columns
    const uint32_t s = s0 + (uint32_t)lane;
    int n = 0, x0 = 0, nx = 0;
    uint4 e = make_uint4(0u, 0u, 0u, 0u);
    float2 yr = make_float2(0.0f, 0.0f);
    if (s < S) {
      int lo = 0, hi = numShapes;  // last shape with strandBase <= s
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (sh.strandBase[mid] <= s) {
          lo = mid;
        } else {
          hi = mid;
        }
      }
      n = lo;
      const uint32_t t = sh.strandFirst[n] + (s - sh.strandBase[n]);
      e = in.strand_table[t];
      yr = in.strand_y[t];
      const float lx = __uint_as_float(e.z), rx = __uint_as_float(e.w);
      const int left = ti.left;
      // the range test of column x (checkInRange, K:1360-1363, on the strand table's
      // left and right x): lx - X <= 1 and rx - X > 0 with X = float(left + x); the
      // first holds from some x on, the second up to some x
      const int a = firstTrue(xbase, xbase + unitW, [&](int x) { return lx - (float)(left + x) <= kRight; });
      const int b = firstTrue(a, xbase + unitW, [&](int x) { return !(rx - (float)(left + x) > kLeft); });
      x0 = a;
      nx = b - a;
    }
    const uint32_t pairs = (uint32_t)(nx * nslab);
    const uint32_t pe = warpScan(pairs, lane);
    const uint32_t T = __shfl_sync(full, pe, 31);
    sh.pairEnd[lane] = pe;
    sh.sTab[lane] = e;
    sh.sY[lane] = yr;
    sh.sShape[lane] = n;
    sh.sX0[lane] = x0;
    sh.sNx[lane] = nx;
    __syncwarp();
    // ---- the batch's (strand, column) pairs, 32 at a time, in strand order
    for (uint32_t q0 = 0; q0 < T; q0 += 32) {
      const uint32_t q = q0 + (uint32_t)lane;
      int L = -1, j = 0;
      if (q < T) {
        j = firstTrue(0, 32, [&](int i) { return sh.pairEnd[i] > q; });
        const uint32_t r = q - (j > 0 ? sh.pairEnd[j - 1] : 0u);
        const uint32_t nxj = (uint32_t)sh.sNx[j];
        const int slab = (int)(r / nxj);
        const int x = sh.sX0[j] + (int)(r % nxj);
        L = slab * unitW + (x - xbase);
      }
      const int srcLane = L >= 0 ? L : 0;
      const int dX = __shfl_sync(full, c.deltaX, srcLane);
      const int dY = __shfl_sync(full, c.deltaY, srcLane);
      const float fh = __shfl_sync(full, c.floatHeight, srcLane);
      const int act = __shfl_sync(full, c.active ? 1 : 0, srcLane);
      PairSink sink;
      sink.n = 0;
      sink.overflow = false;
      bool added = false, enclosed = false;
      int shapeN = 0;
      if (L >= 0 && act) {
        shapeN = sh.sShape[j];
        const uint4 ej = sh.sTab[j];
        const float2 yj = sh.sY[j];
        const float2 d = make_float2((float)dX, (float)dY);
        // y culling (as the per-column code): wholly below the column, nothing; wholly
        // above, no intercepts
        if (!(yj.x - d.y >= fh + 1.0f)) {
          const bool above = yj.y - d.y <= -1.0f;
          ColumnState pc;
          pc.floatHeight = fh;
          GenStateOf<PairSink> g{&sink, &pc};
          strandThresholds(g, in.geometry + (size_t)ej.x * 8, ej.y, d, (uint32_t)shapeN, added, enclosed, status,
                           above);
        }
      }
      sinkOverflow = sinkOverflow || sink.overflow;
      // ---- binning: ballots over the lanes that pushed into the same column
      const int cnt = sink.n;
      const unsigned has = __ballot_sync(full, cnt > 0);
      const unsigned b0 = __ballot_sync(full, (cnt & 1) != 0);
      const unsigned b1 = __ballot_sync(full, (cnt & 2) != 0);
      const unsigned peers = __match_any_sync(full, cnt > 0 ? (unsigned)L : 0xFFFFFFFFu) & has;
      const unsigned lower = peers & ((1u << lane) - 1u);
      uint32_t base = 0u;
      if (cnt > 0) base = sh.colCount[L];
      __syncwarp();
      if (cnt > 0) {
        const uint32_t pos = base + (uint32_t)__popc(b0 & lower) + 2u * (uint32_t)__popc(b1 & lower);
        float4* thr = thrWarp + (size_t)L * (size_t)cap;
        uint32_t* hdr = hdrWarp + (size_t)L * (size_t)cap;
        for (int k = 0; k < cnt; ++k) {
          const uint32_t p = pos + (uint32_t)k;
          if (p < (uint32_t)cap) {
            const int at = cap - 1 - (int)p;  // newest push first, as Queue::push
            hdr[at] = k == 0 ? sink.h0 : (k == 1 ? sink.h1 : sink.h2);
            thr[at] = k == 0 ? sink.t0 : (k == 1 ? sink.t1 : sink.t2);
          }
        }
        // the highest peer closes the column's count for this round
        if (lane == 31 - __clz((int)peers))
          sh.colCount[L] = base + (uint32_t)__popc(b0 & peers) + 2u * (uint32_t)__popc(b1 & peers);
      }
      if (L >= 0 && act) {
        if (enclosed) atomicXor(&sh.encl[L], 1ull << shapeN);
        if (added) atomicOr(&sh.added[L], 1ull << shapeN);
      }
      __syncwarp();
    }
  }
  __syncwarp();

  // ---- each lane: its column's shape bits, sort and scan
  // a unit of one slab of at most 32 rows renders into the shared tile
  const int desired = 1 << max(0, (int)ti.vdepth - (in.log2_tpt - hDepth));
  const bool stageUnit = nslab == 1 && desired <= kCoopStageRows;
  int flags = 0;
  bool rendered = false;
  if (c.active) {
    const int count = (int)sh.colCount[lane];
    if (count > cap || sinkOverflow) {
      flags |= kCoopOverflow;
    } else {
      float4* thr = thrWarp + (size_t)lane * (size_t)cap;
      uint32_t* hdr = hdrWarp + (size_t)lane * (size_t)cap;
      // The column's shape bits are the tile's shape numbers n (the headers already
      // carry them): the per-column generation numbers only the shapes that touch
      // the column, in the same order, and the scan depends on the bits only
      // through their order (findTop walks them top down, the colour memo compares
      // positions), so the image is the same.  The initial stack is the enclosure
      // parity of each shape.
      const unsigned long long encl = sh.encl[lane];
      const unsigned long long touched = encl | sh.added[lane];
      const uint64_t word = encl;
      const int bits = __popcll(touched);
      Queue q{thr, hdr, cap - count, cap, false};
      sortQueue(q);
      if (in.counters) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&in.counters[2]), (unsigned long long)q.length());
        atomicMax(reinterpret_cast<unsigned long long*>(&in.counters[3]), (unsigned long long)bits);
      }
      ShapeStack<1> one;
      one.clear();
      one.w[0] = word;
      one.nz = word ? 1u : 0u;
      // tags of bit n: the staged record n (or the tile's records in the shape pile)
      const DirectTags tags{staged ? sh.shapes : src};
      renderColumnT<1, false>(in, c, q, one, tags, status, numShapes, nullptr, stageUnit ? sh.stage + lane : nullptr);
      if (q.overflow) {
        flags |= kCoopOverflow;
      } else {
        rendered = true;
      }
    }
  }
  if (stageUnit) storeStagedUnit(in, c, rendered, lane, sh);
  return flags;
}

}  // namespace gudni
