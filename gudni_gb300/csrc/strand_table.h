// The strand table of a geometry pile (host code; shared by the C ABI and tests).
//
// The pile is the strands of every shape back to back (Raster/Serialize.hs:76-84,
// Enclosure.hs:76-80).  One walk from its first byte records, per strand, its offset
// (8-byte units), size, the left and right x its range test reads (checkInRange,
// Kernels.cl:1360-1363) and the y range of all its points, and, per 16-byte unit of
// the pile, the index of the strand starting there.  The walk stops at the first
// malformed header; shapes starting past that point keep the kernel's checked
// per-strand path.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace gudni {

constexpr uint32_t kNoStrandIndex = 0xFFFFFFFFu;  // no strand starts at this unit

// Coordinates beyond this magnitude disable the kernels' y culling of their strand:
// at and below it the curve intercepts stay finite and inside the strand's y range up
// to rounding far below the culling's one-pixel margin; a NaN or infinite coordinate,
// or finite ones so large that a difference or product overflows, can make an
// intercept NaN or infinite, where the culling's reasoning does not hold.
constexpr float kStrandCullExtent = 2097152.0f;  // 2^21

// y range of every point of one strand (right end, left end and its control, then
// each tree node's point and control).  A strand with a coordinate (x or y) that is
// NaN, infinite or beyond kStrandCullExtent in magnitude gets (-inf, inf), which
// disables the kernels' culling for it.
inline float2 strand_y_range(const uint8_t* strand, uint32_t size) {
  float lo = INFINITY, hi = -INFINITY;
  bool bad = false;
  auto take = [&](size_t at) {  // the point whose x is at byte `at`
    float x, y;
    std::memcpy(&x, strand + at, 4);
    std::memcpy(&y, strand + at + 4, 4);
    if (!(std::fabs(x) <= kStrandCullExtent) || !(std::fabs(y) <= kStrandCullExtent)) bad = true;
    lo = std::min(lo, y);
    hi = std::max(hi, y);
  };
  take(8);
  take(16);
  take(24);
  for (size_t node = 32; node + 16 <= (size_t)size * 8; node += 16) {
    take(node);
    take(node + 8);
  }
  return bad ? make_float2(-INFINITY, INFINITY) : make_float2(lo, hi);
}

// `threads` > 1: the y ranges (independent per strand, most of the time of a large
// pile) are computed on that many host threads after the sequential walk; the table is
// the same.
inline void build_strand_table(const uint8_t* geo, size_t bytes, std::vector<uint4>& table, std::vector<float2>& ys,
                               std::vector<uint32_t>& first, unsigned threads = 1) {
  table.clear();
  ys.clear();
  first.assign(bytes / 16, kNoStrandIndex);
  size_t off = 0;
  while (off + 32 <= bytes) {
    uint16_t size;
    std::memcpy(&size, geo + off, 2);
    if (size < 4 || (size & 1u) != 0 || off + (size_t)size * 8 > bytes) break;
    if (table.size() >= 0xFFFFFFF0ull || off / 8 > 0xFFFFFFFFull) break;
    uint32_t lx, rx;
    std::memcpy(&rx, geo + off + 8, 4);
    std::memcpy(&lx, geo + off + 16, 4);
    if (off % 16 == 0) first[off / 16] = (uint32_t)table.size();
    table.push_back(make_uint4((uint32_t)(off / 8), size, lx, rx));
    off += (size_t)size * 8;
  }
  ys.resize(table.size());
  auto range = [&](size_t a, size_t b) {
    for (size_t i = a; i < b; ++i) ys[i] = strand_y_range(geo + (size_t)table[i].x * 8, table[i].y);
  };
  const size_t n = table.size();
  threads = (unsigned)std::max<size_t>(1, std::min<size_t>(threads, n / 16384));
  if (threads <= 1) {
    range(0, n);
    return;
  }
  std::vector<std::thread> pool;
  for (unsigned t = 1; t < threads; ++t) pool.emplace_back(range, n * t / threads, n * (t + 1) / threads);
  range(0, n / threads);
  for (auto& th : pool) th.join();
}

}  // namespace gudni
