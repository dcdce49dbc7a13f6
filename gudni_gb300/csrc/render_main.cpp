// gudni_render: a native host for the raster path, through the C ABI only.
//
//   gudni_render <scene file> <out.ppm> [--device-serializer] [--frames N]
//   gudni_render <scene file> --describe
//
// The scene file is a flattened scene (gudni_scene_desc) with its spec, picture pile
// and random field, written by gudni_gb300.scene.write_scene_file: a list of named
// arrays (u32 name length, name, u64 byte count, bytes).  The frame is serialized by
// the host serializer (gudni_serialize, then gudni_upload_common + gudni_raster_frame
// with host buffers) or, with --device-serializer, on the device
// (gudni_upload_pictures + gudni_serialize_device + gudni_raster_tiles_device), and
// written as a binary PPM (the BGRA words' colour channels).  One JSON line reports
// the median times over N frames.  --describe reads the file and prints its counts
// without touching a GPU.
//
// Exit codes: 0 done, 1 bad arguments or file, 2 serializer refused the scene, 3 no
// CUDA device or context, 4 a raster call failed.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "gudni_cuda.h"
#include "gudni_serialize.h"

namespace {

using Arrays = std::map<std::string, std::vector<uint8_t>>;

bool read_scene_file(const char* path, Arrays& a) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  bool ok = true;
  uint32_t len;
  while (std::fread(&len, 4, 1, f) == 1) {
    if (len > 256) {
      ok = false;
      break;
    }
    std::string name(len, '\0');
    uint64_t bytes = 0;
    if (std::fread(&name[0], 1, len, f) != len || std::fread(&bytes, 8, 1, f) != 1 || bytes > (1ull << 40)) {
      ok = false;
      break;
    }
    std::vector<uint8_t>& v = a[name];
    v.resize(bytes);
    if (bytes && std::fread(v.data(), 1, bytes, f) != bytes) {
      ok = false;
      break;
    }
  }
  std::fclose(f);
  return ok;
}

template <class T>
const T* array_of(const Arrays& a, const char* name, size_t* count = nullptr) {
  auto it = a.find(name);
  if (count) *count = it == a.end() ? 0 : it->second.size() / sizeof(T);
  if (it == a.end() || it->second.empty()) return nullptr;
  return reinterpret_cast<const T*>(it->second.data());
}

// Every index array the descriptor points into, checked against its own length, so a
// truncated file is refused here rather than read past its end.
bool scene_from(const Arrays& a, gudni_scene_desc& d, gudni_spec& spec, std::string& why) {
  size_t n_hdr = 0, n_spec = 0;
  const int32_t* hdr = array_of<int32_t>(a, "header", &n_hdr);  // canvas w, h, substances, pictures
  const gudni_spec* sp = array_of<gudni_spec>(a, "spec", &n_spec);
  if (!hdr || n_hdr < 4 || !sp || n_spec < 1) {
    why = "missing header or spec";
    return false;
  }
  spec = *sp;
  std::memset(&d, 0, sizeof(d));
  d.canvas_w = hdr[0];
  d.canvas_h = hdr[1];
  d.n_substances = hdr[2];
  d.n_pictures = hdr[3];
  if (const float* bg = array_of<float>(a, "background")) std::memcpy(d.background, bg, 16);
  size_t n_kind, n_color, n_pict, n_xform, n_rad, n_sub_start, n_comp, n_os, n_ops, n_pairs, n_psize, n_poff;
  d.substance_kind = array_of<int32_t>(a, "substance_kind", &n_kind);
  d.substance_color = array_of<float>(a, "substance_color", &n_color);
  d.substance_picture = array_of<int32_t>(a, "substance_picture", &n_pict);
  d.substance_picture_xform = array_of<float>(a, "substance_picture_xform", &n_xform);
  d.substance_radial = array_of<gudni_radial>(a, "substance_radial", &n_rad);
  d.substance_shape_start = array_of<int32_t>(a, "substance_shape_start", &n_sub_start);
  d.shape_compound = array_of<int32_t>(a, "shape_compound", &n_comp);
  d.shape_outline_start = array_of<int32_t>(a, "shape_outline_start", &n_os);
  d.outline_pair_start = array_of<int32_t>(a, "outline_pair_start", &n_ops);
  d.pairs = array_of<float>(a, "pairs", &n_pairs);
  d.picture_size = array_of<int32_t>(a, "picture_size", &n_psize);
  d.picture_offset = array_of<int32_t>(a, "picture_offset", &n_poff);
  const size_t ns = d.n_substances < 0 ? 0 : (size_t)d.n_substances;
  const size_t np = d.n_pictures < 0 ? 0 : (size_t)d.n_pictures;
  if (d.n_substances < 0 || d.n_pictures < 0 || n_kind < ns || n_color < 4 * ns || n_pict < ns || n_xform < 3 * ns ||
      n_rad < ns || (ns && n_sub_start < ns + 1) || n_psize < 2 * np || n_poff < np) {
    why = "substance or picture arrays shorter than their counts";
    return false;
  }
  auto in_range = [](const int32_t* v, size_t n, int64_t lo, int64_t hi) {
    for (size_t i = 0; i < n; ++i)
      if (v[i] < lo || v[i] > hi || (i && v[i] < v[i - 1])) return false;
    return true;
  };
  if (ns && !in_range(d.substance_shape_start, ns + 1, 0, (int64_t)n_comp)) {
    why = "substance shape starts out of order or beyond the shapes";
    return false;
  }
  const int64_t shapes = ns ? d.substance_shape_start[ns] : 0;
  if (shapes && (n_os < (size_t)shapes + 1 || !in_range(d.shape_outline_start, (size_t)shapes + 1, 0,
                                                         (int64_t)n_ops - 1))) {
    why = "shape outline starts out of order or beyond the outlines";
    return false;
  }
  const int64_t outlines = shapes ? d.shape_outline_start[shapes] : 0;
  if (outlines && (n_ops < (size_t)outlines + 1 || !in_range(d.outline_pair_start, (size_t)outlines + 1, 0,
                                                              (int64_t)(n_pairs / 4)))) {
    why = "outline pair starts out of order or beyond the pairs";
    return false;
  }
  return true;
}

// The BGRA words' colour channels as a binary PPM.
bool write_ppm(const char* path, const uint32_t* bgra, int w, int h) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return false;
  std::fprintf(f, "P6\n%d %d\n255\n", w, h);
  std::vector<uint8_t> row((size_t)w * 3);
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const uint32_t p = bgra[(size_t)y * w + x];
      row[3 * x + 0] = (uint8_t)(p >> 16);
      row[3 * x + 1] = (uint8_t)(p >> 8);
      row[3 * x + 2] = (uint8_t)p;
    }
    std::fwrite(row.data(), 1, row.size(), f);
  }
  return std::fclose(f) == 0;
}

double median(std::vector<double> v) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  return v[v.size() / 2];
}

int log2_of(int v) {
  int d = 0;
  while ((1 << d) < v) ++d;
  return d;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <scene file> <out.ppm> [--device-serializer] [--frames N]\n"
                         "       %s <scene file> --describe\n", argv[0], argv[0]);
    return 1;
  }
  const bool describe = std::strcmp(argv[2], "--describe") == 0;
  bool on_device = false;
  int frames = 1;
  for (int i = 3; i < argc; ++i) {
    if (std::strcmp(argv[i], "--device-serializer") == 0) {
      on_device = true;
    } else if (std::strcmp(argv[i], "--frames") == 0 && i + 1 < argc) {
      frames = std::max(1, std::atoi(argv[++i]));
    } else {
      std::fprintf(stderr, "unknown argument %s\n", argv[i]);
      return 1;
    }
  }
  Arrays arrays;
  gudni_scene_desc scene;
  gudni_spec spec;
  std::string why;
  if (!read_scene_file(argv[1], arrays) || !scene_from(arrays, scene, spec, why)) {
    std::fprintf(stderr, "cannot read scene %s: %s\n", argv[1], why.empty() ? "unreadable" : why.c_str());
    return 1;
  }
  size_t n_picture_bytes = 0, n_random = 0, n_pairs = 0, n_shapes = 0;
  const uint8_t* pictures = array_of<uint8_t>(arrays, "pictures", &n_picture_bytes);
  const float* random_field = array_of<float>(arrays, "random_field", &n_random);
  array_of<float>(arrays, "pairs", &n_pairs);
  array_of<int32_t>(arrays, "shape_compound", &n_shapes);
  if (random_field && n_random < GUDNI_RANDOM_FIELD_SIZE) random_field = nullptr;
  if (describe) {
    std::printf("{\"canvas\": [%d, %d], \"substances\": %d, \"shapes\": %zu, \"pairs\": %zu, \"pictures\": %d, "
                "\"picture_bytes\": %zu, \"random_field\": %s, \"tile\": %d, \"threads_per_tile\": %d}\n",
                scene.canvas_w, scene.canvas_h, scene.n_substances, n_shapes, n_pairs / 4, scene.n_pictures,
                n_picture_bytes, random_field ? "true" : "false", spec.max_tile_size, spec.threads_per_tile);
    return 0;
  }

  gudni_ctx* ctx = gudni_create(&spec, 0);
  if (!ctx) {
    std::fprintf(stderr, "gudni_create: %s\n", gudni_last_error(nullptr));
    return 3;
  }
  const int w = scene.canvas_w, h = scene.canvas_h;
  std::vector<uint32_t> image((size_t)w * h, 0u);
  std::vector<double> ser_ms, ren_ms;
  int rc = 0;
  using clock = std::chrono::steady_clock;
  auto ms_since = [](clock::time_point t) {
    return std::chrono::duration<double, std::milli>(clock::now() - t).count();
  };
  if (!on_device) {
    for (int f = 0; f < frames && rc == 0; ++f) {
      const auto t0 = clock::now();
      gudni_frame* fr = gudni_serialize(&scene, &spec);
      if (!fr) {
        std::fprintf(stderr, "gudni_serialize: %s\n", gudni_serialize_error());
        gudni_destroy(ctx);
        return 2;
      }
      ser_ms.push_back(ms_since(t0));
      const auto t1 = clock::now();
      rc = gudni_upload_common(ctx, gudni_frame_geometry(fr), gudni_frame_geometry_bytes(fr), gudni_frame_substances(fr),
                               gudni_frame_n_substances(fr), pictures, n_picture_bytes, gudni_frame_picture_uses(fr),
                               gudni_frame_n_picture_uses(fr), gudni_frame_radials(fr), gudni_frame_n_radials(fr),
                               random_field);
      std::vector<gudni_job_desc> jobs(gudni_frame_n_jobs(fr));
      for (size_t j = 0; j < jobs.size(); ++j) {
        jobs[j].shapes = gudni_frame_job_shapes(fr, j);
        jobs[j].n_shapes = gudni_frame_job_n_shapes(fr, j);
        jobs[j].tiles = gudni_frame_job_tiles(fr, j);
        jobs[j].n_tiles = gudni_frame_job_n_tiles(fr, j);
        jobs[j].columns_to_alloc = gudni_frame_job_columns(fr, j);
      }
      if (rc == 0)
        rc = gudni_raster_frame(ctx, jobs.data(), jobs.size(), w, h, log2_of(spec.threads_per_tile), f,
                                scene.background, image.data());
      ren_ms.push_back(ms_since(t1));
      gudni_frame_free(fr);
    }
  } else {
    uint32_t* d_out = nullptr;
    rc = gudni_upload_pictures(ctx, pictures, n_picture_bytes);
    if (rc == 0) rc = gudni_upload_random_field(ctx, random_field);
    if (rc == 0 && cudaMalloc(&d_out, image.size() * 4) != cudaSuccess) {
      std::fprintf(stderr, "cannot allocate the output bitmap\n");
      gudni_destroy(ctx);
      return 3;
    }
    for (int f = 0; f < frames && rc == 0; ++f) {
      const auto t0 = clock::now();
      gudni_device_frame df;
      rc = gudni_serialize_device(ctx, &scene, 0, &df);
      if (rc) break;
      ser_ms.push_back(ms_since(t0));
      const auto t1 = clock::now();
      rc = gudni_raster_tiles_device(ctx, df.shapes, df.n_shapes, df.tiles, df.tile_jobs, df.n_tiles, w, h,
                                     log2_of(spec.threads_per_tile), f, scene.background, d_out, nullptr);
      if (rc == 0) rc = gudni_sync_status(ctx);
      ren_ms.push_back(ms_since(t1));
    }
    if (rc == 0 && cudaMemcpy(image.data(), d_out, image.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = -4;
    cudaFree(d_out);
  }
  if (rc) {
    std::fprintf(stderr, "raster: %s (%d)\n", gudni_last_error(ctx), rc);
    gudni_destroy(ctx);
    return rc == GUDNI_ERR_BAD_INPUT ? 2 : 4;
  }
  gudni_destroy(ctx);
  if (!write_ppm(argv[2], image.data(), w, h)) {
    std::fprintf(stderr, "cannot write %s\n", argv[2]);
    return 1;
  }
  std::printf("{\"canvas\": [%d, %d], \"serializer\": \"%s\", \"frames\": %d, \"serialize_ms\": %.3f, "
              "\"upload_and_raster_ms\": %.3f}\n",
              w, h, on_device ? "device" : "host", frames, median(ser_ms), median(ren_ms));
  return 0;
}
