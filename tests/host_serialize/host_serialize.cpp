// TEST INFRASTRUCTURE -- not part of the product and never loaded by it.
//
// The device serializer's passes (gudni_gb300/csrc/serialize_device.cuh) run on the
// CPU by an executor of plain loops, as a standalone program built with
// AddressSanitizer and UBSan: every index a pass computes is checked against the
// exact size of the buffer it reads or writes, buffers start filled with a garbage
// byte (device memory is not cleared), and the items of each pass run in a seeded
// random order (the GPU runs them in any order), so a pass that reads another item's
// output, or memory nobody wrote, changes the result.
//
//   host_serialize <scene file> <result file> <seed>
//
// Both files are lists of named arrays: u32 name length, name, u64 byte count, bytes.

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "serialize_device.cuh"

namespace ser = gudni::ser;

struct HostExec {
  std::vector<std::vector<uint8_t>> slot = std::vector<std::vector<uint8_t>>(ser::kSlots);
  uint64_t rng;

  template <class T>
  T* alloc(ser::Slot s, uint64_t n) {
    std::vector<uint8_t>& v = slot[s];
    v.assign((size_t)(n ? n * sizeof(T) : 1), 0xA5);
    v.shrink_to_fit();
    return reinterpret_cast<T*>(v.data());
  }
  uint64_t next() {  // splitmix64
    uint64_t z = (rng += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  template <class Pass>
  int forEach(uint64_t n, const Pass& pass) {
    std::vector<uint64_t> order(n);
    for (uint64_t i = 0; i < n; ++i) order[i] = i;
    for (uint64_t i = n; i > 1; --i) std::swap(order[i - 1], order[next() % i]);
    for (uint64_t i : order) pass(i);
    return 0;
  }
  int scan(const uint64_t* in, uint64_t* out, uint64_t n) {
    uint64_t acc = 0;
    for (uint64_t i = 0; i < n; ++i) {
      const uint64_t v = in[i];
      out[i] = acc;
      acc += v;
    }
    out[n] = acc;
    return 0;
  }
  int read(void* dst, const void* src, size_t bytes) {
    std::memcpy(dst, src, bytes);
    return 0;
  }
  int copy(void* dst, const void* src, size_t bytes) {
    std::memcpy(dst, src, bytes);
    return 0;
  }
  int upload(void* dst, const void* src, size_t bytes) {
    std::memcpy(dst, src, bytes);
    return 0;
  }
};

using Arrays = std::map<std::string, std::vector<uint8_t>>;

static bool load(const char* path, Arrays& a) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  uint32_t len;
  while (std::fread(&len, 4, 1, f) == 1) {
    std::string name(len, '\0');
    uint64_t bytes;
    if (std::fread(&name[0], 1, len, f) != len || std::fread(&bytes, 8, 1, f) != 1) break;
    std::vector<uint8_t>& v = a[name];
    v.resize(bytes);
    if (bytes && std::fread(v.data(), 1, bytes, f) != bytes) break;
  }
  std::fclose(f);
  return true;
}

static void put(FILE* f, const char* name, const void* data, uint64_t bytes) {
  const uint32_t len = (uint32_t)std::strlen(name);
  std::fwrite(&len, 4, 1, f);
  std::fwrite(name, 1, len, f);
  std::fwrite(&bytes, 8, 1, f);
  if (bytes) std::fwrite(data, 1, bytes, f);
}

template <class T>
static const T* arr(Arrays& a, const char* name) {
  auto it = a.find(name);
  if (it == a.end() || it->second.empty()) return nullptr;
  return reinterpret_cast<const T*>(it->second.data());
}

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  Arrays a;
  if (!load(argv[1], a)) return 2;
  const int32_t* hdr = arr<int32_t>(a, "header");  // canvas w, h, substances, pictures
  const gudni_spec* spec = arr<gudni_spec>(a, "spec");
  if (!hdr || !spec) return 2;
  gudni_scene_desc d;
  std::memset(&d, 0, sizeof(d));
  d.canvas_w = hdr[0];
  d.canvas_h = hdr[1];
  d.n_substances = hdr[2];
  d.n_pictures = hdr[3];
  d.substance_kind = arr<int32_t>(a, "substance_kind");
  d.substance_color = arr<float>(a, "substance_color");
  d.substance_picture = arr<int32_t>(a, "substance_picture");
  d.substance_picture_xform = arr<float>(a, "substance_picture_xform");
  d.substance_radial = arr<gudni_radial>(a, "substance_radial");
  d.substance_shape_start = arr<int32_t>(a, "substance_shape_start");
  d.shape_compound = arr<int32_t>(a, "shape_compound");
  d.shape_outline_start = arr<int32_t>(a, "shape_outline_start");
  d.outline_pair_start = arr<int32_t>(a, "outline_pair_start");
  d.pairs = arr<float>(a, "pairs");
  d.picture_size = arr<int32_t>(a, "picture_size");
  d.picture_offset = arr<int32_t>(a, "picture_offset");

  FILE* out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  ser::Scene sc;
  int64_t n_pairs = 0;
  std::vector<float4> subs;
  std::vector<gudni_picture_use> uses;
  std::vector<gudni_radial> rads;
  std::vector<uint64_t> tags;
  const char* why = ser::checkScene(&d, *spec, sc, n_pairs);
  if (!why) why = ser::buildSubstances(&d, subs, uses, rads, tags);
  if (why) {
    put(out, "error", why, std::strlen(why));
    std::fclose(out);
    return 0;
  }
  sc.substance_shape_start = d.substance_shape_start;
  sc.substance_tag = tags.data();
  sc.shape_compound = d.shape_compound;
  sc.shape_outline_start = d.shape_outline_start;
  sc.outline_pair_start = d.outline_pair_start;
  sc.pairs = d.pairs;
  ser::Limits lim{spec->max_tile_size, spec->threads_per_tile, spec->max_tiles_per_call, spec->max_shape,
                  (int64_t)spec->max_strands_per_tile};
  HostExec ex;
  ex.rng = std::strtoull(argv[3], nullptr, 10);
  ser::Result r;
  const int rc = ser::serialize(ex, sc, lim, r);
  if (rc) {
    put(out, "error", "serializer failed", 17);
    std::fclose(out);
    return 0;
  }
  put(out, "geometry", r.geometry, r.geometry_bytes);
  put(out, "strand_table", r.strand_table, r.n_strands * sizeof(uint4));
  put(out, "strand_y", r.strand_y, r.n_strands * sizeof(float2));
  put(out, "strand_first", r.strand_first, r.geometry_bytes / 16 * 4);
  put(out, "shapes", r.shapes, r.n_shapes * sizeof(gudni_shape));
  put(out, "tiles", r.tiles, r.n_tiles * sizeof(gudni_tile_info));
  put(out, "tile_jobs", r.tile_jobs, r.n_tiles * 4);
  put(out, "substances", subs.data(), subs.size() * sizeof(float4));
  put(out, "picture_uses", uses.data(), uses.size() * sizeof(gudni_picture_use));
  put(out, "radials", rads.data(), rads.size() * sizeof(gudni_radial));
  put(out, "stats", r.stats, sizeof(r.stats));
  put(out, "n_jobs", &r.n_jobs, 8);
  std::fclose(out);
  return 0;
}
