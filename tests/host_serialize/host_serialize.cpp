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
//   host_serialize <scene file> <result file> <seed> [provenance]
//
// Both files are lists of named arrays: u32 name length, name, u64 byte count, bytes.
//
// Compiled by nvcc (as CUDA source) the same program runs the passes as the library's
// kernels (pass_kernel, scan_kernel) with a device executor, so the GPU's result can be
// compared with the CPU's file byte for byte.

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
  std::vector<uint8_t> fetch(const void* src, size_t bytes) {
    const uint8_t* p = static_cast<const uint8_t*>(src);
    return std::vector<uint8_t>(p, p + bytes);
  }
  const void* place(const void* host, size_t) { return host; }
};

#if defined(__CUDACC__)
// The passes as kernels on the default stream, each slot one device allocation.
struct DeviceExec {
  void* ptr[ser::kSlots] = {};
  size_t cap[ser::kSlots] = {};
  std::vector<void*> extra;
  uint64_t rng;
  int sm_count = 1;
  ~DeviceExec() {
    for (void* p : ptr) cudaFree(p);
    for (void* p : extra) cudaFree(p);
  }
  template <class T>
  T* alloc(ser::Slot s, uint64_t n) {
    const size_t bytes = (size_t)(n ? n * sizeof(T) : 1);
    if (bytes > cap[s]) {
      cudaFree(ptr[s]);
      ptr[s] = nullptr;
      cap[s] = 0;
      if (cudaMalloc(&ptr[s], bytes) != cudaSuccess) return nullptr;
      cap[s] = bytes;
    }
    cudaMemset(ptr[s], 0xA5, bytes);
    return static_cast<T*>(ptr[s]);
  }
  template <class Pass>
  int forEach(uint64_t n, const Pass& pass) {
    if (n == 0) return 0;
    const uint64_t blocks = (n + ser::kPassBlock - 1) / ser::kPassBlock;
    const int grid = (int)(blocks < (uint64_t)sm_count * 8 ? blocks : (uint64_t)sm_count * 8);
    ser::pass_kernel<Pass><<<grid, ser::kPassBlock>>>(pass, n);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
  }
  int scan(const uint64_t* in, uint64_t* out, uint64_t n) {
    ser::scan_kernel<<<1, ser::kScanBlock>>>(in, out, n);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
  }
  int read(void* dst, const void* src, size_t bytes) {
    return cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? 0 : -1;
  }
  int copy(void* dst, const void* src, size_t bytes) {
    return cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToDevice) == cudaSuccess ? 0 : -1;
  }
  int upload(void* dst, const void* src, size_t bytes) {
    return cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess ? 0 : -1;
  }
  std::vector<uint8_t> fetch(const void* src, size_t bytes) {
    std::vector<uint8_t> v(bytes);
    if (bytes) cudaMemcpy(v.data(), src, bytes, cudaMemcpyDeviceToHost);
    return v;
  }
  // a device copy of a host array the passes read
  const void* place(const void* host, size_t bytes) {
    if (!host || !bytes) return host;
    void* d = nullptr;
    if (cudaMalloc(&d, bytes) != cudaSuccess) return nullptr;
    cudaMemcpy(d, host, bytes, cudaMemcpyHostToDevice);
    extra.push_back(d);
    return d;
  }
};
using Exec = DeviceExec;
#else
using Exec = HostExec;
#endif

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

// host_serialize --strands <pile file> <result file> <seed>: the strand table of a
// geometry pile by the device passes (strandTable).
static int strands_main(char** argv) {
  FILE* f = std::fopen(argv[2], "rb");
  if (!f) return 2;
  std::vector<uint8_t> pile;
  uint8_t buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) pile.insert(pile.end(), buf, buf + got);
  std::fclose(f);
  Exec ex;
  ex.rng = std::strtoull(argv[4], nullptr, 10);
#if defined(__CUDACC__)
  cudaDeviceGetAttribute(&ex.sm_count, cudaDevAttrMultiProcessorCount, 0);
#endif
  const uint8_t* geo = static_cast<const uint8_t*>(ex.place(pile.data(), pile.size()));
  ser::StrandTableOut t;
  const int rc = ser::strandTable(ex, pile.empty() ? nullptr : geo, pile.size(), t);
  FILE* out = std::fopen(argv[3], "wb");
  if (!out) return 2;
  if (rc) {
    put(out, "error", "strand table failed", 19);
  } else {
    const std::vector<uint8_t> tb = ex.fetch(t.table, t.n_strands * sizeof(uint4));
    const std::vector<uint8_t> ys = ex.fetch(t.ys, t.n_strands * sizeof(float2));
    const std::vector<uint8_t> fi = ex.fetch(t.first, pile.size() / 16 * 4);
    put(out, "strand_table", tb.data(), tb.size());
    put(out, "strand_y", ys.data(), ys.size());
    put(out, "strand_first", fi.data(), fi.size());
  }
  std::fclose(out);
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 5 && std::strcmp(argv[1], "--strands") == 0) return strands_main(argv);
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
  Exec ex;
  ex.rng = std::strtoull(argv[3], nullptr, 10);
#if defined(__CUDACC__)
  cudaDeviceGetAttribute(&ex.sm_count, cudaDevAttrMultiProcessorCount, 0);
#endif
  auto bytes_of = [&](const char* name) -> size_t {
    auto it = a.find(name);
    return it == a.end() ? 0 : it->second.size();
  };
  sc.substance_shape_start = (const int32_t*)ex.place(d.substance_shape_start, bytes_of("substance_shape_start"));
  sc.substance_tag = (const uint64_t*)ex.place(tags.data(), tags.size() * 8);
  sc.shape_compound = (const int32_t*)ex.place(d.shape_compound, bytes_of("shape_compound"));
  sc.shape_outline_start = (const int32_t*)ex.place(d.shape_outline_start, bytes_of("shape_outline_start"));
  sc.outline_pair_start = (const int32_t*)ex.place(d.outline_pair_start, bytes_of("outline_pair_start"));
  sc.pairs = (const float*)ex.place(d.pairs, bytes_of("pairs"));
  ser::Limits lim{spec->max_tile_size, spec->threads_per_tile, spec->max_tiles_per_call, spec->max_shape,
                  (int64_t)spec->max_strands_per_tile};
  ser::Result r;
  const bool provenance = argc > 4 && std::atoi(argv[4]) != 0;
  const int rc = ser::serialize(ex, sc, lim, r, provenance);
  if (rc) {
    put(out, "error", "serializer failed", 17);
    std::fclose(out);
    return 0;
  }
  auto put_fetched = [&](const char* name, const void* src, size_t bytes) {
    const std::vector<uint8_t> v = ex.fetch(src, bytes);
    put(out, name, v.data(), bytes);
  };
  put_fetched("geometry", r.geometry, r.geometry_bytes);
  put_fetched("strand_table", r.strand_table, r.n_strands * sizeof(uint4));
  put_fetched("strand_y", r.strand_y, r.n_strands * sizeof(float2));
  put_fetched("strand_first", r.strand_first, r.geometry_bytes / 16 * 4);
  put_fetched("shapes", r.shapes, r.n_shapes * sizeof(gudni_shape));
  put_fetched("tiles", r.tiles, r.n_tiles * sizeof(gudni_tile_info));
  put_fetched("tile_jobs", r.tile_jobs, r.n_tiles * 4);
  if (provenance) {
    put_fetched("point_offsets", r.point_offsets, r.n_points * 4);
    put_fetched("point_sources", r.point_sources, r.n_points * 12);
    put_fetched("point_weights", r.point_weights, r.n_points * 12);
  }
  put(out, "substances", subs.data(), subs.size() * sizeof(float4));
  put(out, "picture_uses", uses.data(), uses.size() * sizeof(gudni_picture_use));
  put(out, "radials", rads.data(), rads.size() * sizeof(gudni_radial));
  put(out, "stats", r.stats, sizeof(r.stats));
  put(out, "n_jobs", &r.n_jobs, 8);
  std::fclose(out);
  return 0;
}
