// Host serializer: flattened scene -> reference-compatible piles.
//
// Restates the reference's Haskell host path on the CPU (file:line citations on each
// function).  Float arithmetic is IEEE single precision with no contraction
// (built with -ffp-contract=off), as GHC evaluates Float expressions.

#include "gudni_serialize.h"

#if defined(_OPENMP)
#include <omp.h>
#endif

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <utility>
#include <string>
#include <vector>

#include "serialize_device.cuh"

namespace {

thread_local std::string g_error;

// An allocator whose resize leaves new elements uninitialized (default-initialized):
// the parallel serializer writes every byte of the piles it sizes, so the zero fill a
// std::vector resize performs would be a second, serial pass over them.
template <class T>
struct NoFill : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoFill<U>;
  };
  NoFill() = default;
  template <class U>
  NoFill(const NoFill<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept {
    ::new (static_cast<void*>(p)) U;
  }
  template <class U, class... Args>
  void construct(U* p, Args&&... args) {
    ::new (static_cast<void*>(p)) U(std::forward<Args>(args)...);
  }
};
template <class T>
using Pile = std::vector<T, NoFill<T>>;

struct P2 { float x, y; };
struct Bez { P2 a, c, b; };  // start, control, end (Figure/Bezier.hs Bez)

// ---------------------------------------------------------------- deknob
// Raster/Deknob.hs:35-108

constexpr float kSplit = 0.5f;        // sPLIT, Deknob.hs:36-37
constexpr float kIota = 0.0001f;      // iota for SubSpace, Figure/Space.hs:101-102

inline P2 between(float t, P2 v0, P2 v1) {  // Deknob.hs:40-41
  float u = 1.0f - t;
  return P2{v0.x * u + v1.x * t, v0.y * u + v1.y * t};
}

// findSplit (Deknob.hs:61-79): bisect the parameter while one half keeps bulging in
// the knob's direction.  Returns (mid0, onCurve, mid1); *t_out receives the split
// parameter.
Bez find_split(bool left, const Bez& z, float* t_out) {
  float bottom = 0.0f, top = 1.0f, t = kSplit;
  for (;;) {
    P2 mid0 = between(t, z.a, z.c);
    P2 mid1 = between(t, z.c, z.b);
    P2 on = between(t, mid0, mid1);
    *t_out = t;
    if (top - bottom <= kIota) return Bez{mid0, on, mid1};
    bool mid1_stays = left ? (mid1.x < on.x) : (mid1.x > on.x);
    if (mid1_stays) {
      float ts = t + ((top - t) / 2.0f);
      bottom = t;
      t = ts;
      continue;
    }
    bool mid0_stays = left ? (mid0.x < on.x) : (mid0.x > on.x);
    if (mid0_stays) {
      float bs = bottom + ((t - bottom) / 2.0f);
      top = t;
      t = bs;
      continue;
    }
    return Bez{mid0, on, mid1};
  }
}

// Provenance of a serialized point: a fixed linear combination of at most three
// points of the flattened scene (index = 2 * pair + 0 for the on-curve point, + 1 for
// the off-curve point).  Used to carry gradients from the geometry pile back to the
// scene's control points.
struct Prov {
  int32_t src[3];
  float w[3];
};
inline Prov prov1(int32_t a) { return Prov{{a, -1, -1}, {1.0f, 0.0f, 0.0f}}; }
struct BezProv { Prov a, c, b; };

// fixKnob (Deknob.hs:85-100)
void fix_knob(const Bez& z, std::vector<Bez>& out, const BezProv* zp, std::vector<BezProv>* outp) {
  bool left = z.c.x < z.a.x && z.c.x < z.b.x;
  bool right = !left && (z.c.x > z.a.x && z.c.x > z.b.x);
  if (left || right) {
    float t = kSplit;
    Bez s = find_split(left, z, &t);
    out.push_back(Bez{z.a, s.a, s.c});
    out.push_back(Bez{s.c, s.b, z.b});
    if (outp) {
      // mid0 = (1-t) a + t c, mid1 = (1-t) c + t b, on = (1-t)^2 a + 2t(1-t) c + t^2 b
      const int32_t ia = zp->a.src[0], ic = zp->c.src[0], ib = zp->b.src[0];
      const float u = 1.0f - t;
      Prov mid0{{ia, ic, -1}, {u, t, 0.0f}};
      Prov mid1{{ic, ib, -1}, {u, t, 0.0f}};
      Prov on{{ia, ic, ib}, {u * u, 2.0f * t * u, t * t}};
      outp->push_back(BezProv{zp->a, mid0, on});
      outp->push_back(BezProv{on, mid1, zp->b});
    }
  } else {
    out.push_back(z);
    if (outp) outp->push_back(*zp);
  }
}

// ---------------------------------------------------------------- reorder table
// Raster/ReorderTable.hs:32-110

int perfect_tree_partition(int n) {  // ReorderTable.hs:44-56
  int x = 1;
  while (x <= n / 2) x *= 2;  // powerLess
  if ((x / 2) - 1 <= n - x) return x - 1;
  return n - (x / 2);
}

struct INode { int idx; int left; int right; };  // -1 = leaf

int build_itree(const std::vector<int>& xs, int lo, int hi, std::vector<INode>& nodes) {
  int l = hi - lo;
  if (l <= 0) return -1;
  int half = perfect_tree_partition(l);
  int id = (int)nodes.size();
  nodes.push_back(INode{xs[lo + half], -1, -1});
  int a = build_itree(xs, lo, lo + half, nodes);
  int b = build_itree(xs, lo + half + 1, hi, nodes);
  nodes[id].left = a;
  nodes[id].right = b;
  return id;
}

std::vector<int> make_tree_row(int size) {  // ReorderTable.hs:81-87
  std::vector<int> internal;
  for (int i = 0; i < size / 2; ++i) internal.push_back(i);
  std::vector<INode> nodes;
  int root = build_itree(internal, 0, (int)internal.size(), nodes);
  std::vector<int> half_tree;
  std::vector<int> level;
  if (root >= 0) level.push_back(root);
  while (!level.empty()) {  // breadth-first, left to right
    std::vector<int> next;
    for (int n : level) {
      half_tree.push_back(nodes[n].idx);
      if (nodes[n].left >= 0) next.push_back(nodes[n].left);
      if (nodes[n].right >= 0) next.push_back(nodes[n].right);
    }
    level.swap(next);
  }
  std::vector<int> tree;
  for (int h : half_tree) {
    tree.push_back(2 * h);
    tree.push_back(2 * h + 1);
  }
  return tree;
}

std::vector<int> reorder_for_extents(int size) {  // ReorderTable.hs:92-99
  std::vector<int> row;
  if (size < 3) return row;
  row.push_back(size - 1);
  row.push_back(0);
  row.push_back(1);
  if (size > 3) {
    for (int v : make_tree_row(size - 3)) row.push_back(v + 2);
  }
  return row;
}

constexpr int kMaxSectionSize = 32;                  // mAXsECTIONsIZE, Constants.hs:67
constexpr int kMaxStrandCurves = kMaxSectionSize / 2;  // Strand.hs:178

struct ReorderTable {
  std::vector<std::vector<int>> rows;  // indexed by size/2, buildReorderTable (:103-104)
  ReorderTable() {
    for (int k = 0; k <= kMaxSectionSize / 2; ++k) rows.push_back(reorder_for_extents(2 * k + 1));
  }
};

const ReorderTable& reorder_table() {
  static ReorderTable t;
  return t;
}

// ---------------------------------------------------------------- strands
// Raster/Strand.hs:67-206

inline int cmp_x(const Bez& z) {  // compareHorizontal
  return (z.a.x < z.b.x) ? -1 : ((z.a.x > z.b.x) ? 1 : 0);
}

inline bool connectable(const Bez& a, const Bez& b) {  // Strand.hs:77-81
  int ha = cmp_x(a), hb = cmp_x(b);
  return ha == hb && ha != 0;
}

struct ProvSink {
  Pile<int32_t> src;     // 3 per serialized point
  Pile<float> w;         // 3 per serialized point
  Pile<uint32_t> where;  // float index of the point's x in the geometry pile
};

// Append the serialized strands of one outline (curve pairs) to `geo`; returns the
// number of strands.  splitShape / outlineToStrands, Strand.hs:153-178.  With `prov`,
// also records the provenance of every point written (pair indices from `pair0`).
uint32_t outline_to_strands(const float* pairs, int n_pairs, Pile<uint8_t>& geo, ProvSink* prov = nullptr,
                            int32_t pair0 = 0) {
  if (n_pairs < 2) return 0;
  // pairsToBeziers (overNeighbors makeBezier), then replaceKnobs
  std::vector<Bez> beziers;
  std::vector<BezProv> bprov;
  beziers.reserve(n_pairs + 8);
  for (int i = 0; i < n_pairs; ++i) {
    int j = (i + 1) % n_pairs;
    Bez z{P2{pairs[4 * i], pairs[4 * i + 1]}, P2{pairs[4 * i + 2], pairs[4 * i + 3]},
          P2{pairs[4 * j], pairs[4 * j + 1]}};
    BezProv zp{prov1(2 * (pair0 + i)), prov1(2 * (pair0 + i) + 1), prov1(2 * (pair0 + j))};
    fix_knob(z, beziers, &zp, prov ? &bprov : nullptr);
  }
  // splitIntoStrands: the fold's final accumulator comes first, then the strands in
  // the order they were closed (Strand.hs:98-102).
  std::vector<std::pair<int, int>> runs;  // [start, end) into beziers
  int acc_start = 0;
  for (int i = 1; i < (int)beziers.size(); ++i) {
    if (!connectable(beziers[i - 1], beziers[i])) {
      runs.emplace_back(acc_start, i);
      acc_start = i;
    }
  }
  runs.insert(runs.begin(), std::make_pair(acc_start, (int)beziers.size()));

  const ReorderTable& table = reorder_table();
  uint32_t count = 0;
  std::vector<P2> pts;
  std::vector<Prov> ppts;
  std::vector<Bez> chunk;
  std::vector<BezProv> pchunk;
  for (auto& run : runs) {
    // splitTooLarge 16 (Strand.hs:105-109)
    for (int s = run.first; s < run.second; s += kMaxStrandCurves) {
      int e = std::min(run.second, s + kMaxStrandCurves);
      chunk.assign(beziers.begin() + s, beziers.begin() + e);
      if (prov) pchunk.assign(bprov.begin() + s, bprov.begin() + e);
      // reverseIfBackwards (Strand.hs:137-143)
      if (chunk.front().a.x > chunk.back().b.x) {
        std::reverse(chunk.begin(), chunk.end());
        for (auto& z : chunk) std::swap(z.a, z.b);
        if (prov) {
          std::reverse(pchunk.begin(), pchunk.end());
          for (auto& z : pchunk) std::swap(z.a, z.b);
        }
      }
      // beziersToPoints (Strand.hs:130-134)
      pts.clear();
      ppts.clear();
      for (size_t k = 0; k < chunk.size(); ++k) {
        pts.push_back(chunk[k].a);
        pts.push_back(chunk[k].c);
        if (prov) {
          ppts.push_back(pchunk[k].a);
          ppts.push_back(pchunk[k].c);
        }
      }
      pts.push_back(chunk.back().b);
      if (prov) ppts.push_back(pchunk.back().b);
      const int len = (int)pts.size();
      const std::vector<int>& row = table.rows[len / 2];
      // header: u16 size in 8-byte units, u16 0, u32 0 (Strand.hs:201-206)
      uint16_t size = (uint16_t)((8 + 8 * len) / 8);
      uint8_t hdr[8] = {0};
      std::memcpy(hdr, &size, 2);
      geo.insert(geo.end(), hdr, hdr + 8);
      for (int i = 0; i < len; ++i) {
        const P2& p = pts[row[i]];
        if (prov) {
          const Prov& q = ppts[row[i]];
          prov->src.insert(prov->src.end(), q.src, q.src + 3);
          prov->w.insert(prov->w.end(), q.w, q.w + 3);
          prov->where.push_back((uint32_t)(geo.size() / 4));
        }
        uint8_t b[8];
        std::memcpy(b, &p.x, 4);
        std::memcpy(b + 4, &p.y, 4);
        geo.insert(geo.end(), b, b + 8);
      }
      ++count;
    }
  }
  return count;
}

// ---------------------------------------------------------------- tile tree
// Raster/TileTree.hs:40-204

struct BoxF { float left, top, right, bottom; };

struct ShapeEntry {
  uint64_t tag;
  uint32_t geo_start;
  uint32_t num_strands;
  BoxF box;
};

struct Tile {
  int left, top, right, bottom;
  int hdepth, vdepth;
  std::vector<int> shapes;  // insertion order (the reference prepends)
  uint64_t strand_count = 0;
  int shape_count = 0;
};

enum NodeKind { VTREE, HTREE, VLEAF, HLEAF };

struct Node {
  NodeKind kind;
  float cut;
  int a, b;   // children (top/bottom or left/right)
  int tile;   // leaf tile index
};

int adjusted_log(int x) {  // TileTree.hs:74-75
  if (x < 1) return 0;
  int d = 0;
  while ((1LL << d) < (long long)x) ++d;
  return d;
}

class TileTree {
 public:
  TileTree(int tile_size, int canvas_w, int canvas_h, int max_shape, int64_t max_strands,
           const std::vector<ShapeEntry>* shapes)
      : max_shape_(max_shape), max_strands_(max_strands), shapes_(shapes) {
    int canvas_depth = adjusted_log(std::max(canvas_w, canvas_h));
    tile_depth_ = adjusted_log(tile_size);
    int side = 1 << canvas_depth;
    root_ = go_v(canvas_depth, 0, 0, side, side);
  }

  void add(int shape) { insert_v(root_, shape); }

  template <class F>
  void traverse(F&& f) { trav_v(root_, f); }

  int splits() const { return splits_; }

 private:
  int new_leaf(NodeKind kind, int hd, int vd, int l, int t, int r, int b) {
    Tile tile;
    tile.left = l; tile.top = t; tile.right = r; tile.bottom = b;
    tile.hdepth = hd; tile.vdepth = vd;
    tiles_.push_back(std::move(tile));
    nodes_.push_back(Node{kind, 0.0f, -1, -1, (int)tiles_.size() - 1});
    return (int)nodes_.size() - 1;
  }
  int new_node(NodeKind kind, float cut, int a, int b) {
    nodes_.push_back(Node{kind, cut, a, b, -1});
    return (int)nodes_.size() - 1;
  }
  // buildTileTree goV / goH (TileTree.hs:95-109)
  int go_v(int depth, int l, int t, int r, int b) {
    if (depth > tile_depth_) {
      int cut = t + (1 << (depth - 1));
      int top = go_h(depth, l, t, r, cut);
      int bot = go_h(depth, l, cut, r, b);
      return new_node(VTREE, (float)cut, top, bot);
    }
    return new_leaf(VLEAF, depth, depth, l, t, r, b);
  }
  int go_h(int depth, int l, int t, int r, int b) {
    if (depth > tile_depth_) {
      int cut = l + (1 << (depth - 1));
      int left = go_v(depth - 1, l, t, cut, b);
      int right = go_v(depth - 1, cut, t, r, b);
      return new_node(HTREE, (float)cut, left, right);
    }
    return new_leaf(HLEAF, depth, depth, l, t, r, b);
  }

  // checkTileSpace (TileTree.hs:167-172)
  bool has_space(const Tile& tile, int s) const {
    uint64_t with_added = tile.strand_count + (*shapes_)[s].num_strands;
    return tile.shape_count < max_shape_ - 1 && (int64_t)with_added < max_strands_;
  }
  void insert_tile(Tile& tile, int s) {  // insertShapeTile (TileTree.hs:154-164)
    tile.shapes.push_back(s);
    tile.strand_count += (*shapes_)[s].num_strands;
    tile.shape_count += 1;
  }

  void insert_h(int n, int s) {  // insertShapeH (TileTree.hs:117-134)
    const BoxF& box = (*shapes_)[s].box;
    if (nodes_[n].kind == HTREE) {
      float cut = nodes_[n].cut;
      int a = nodes_[n].a, b = nodes_[n].b;
      if (box.left < cut) insert_v(a, s);
      if (box.right > cut) insert_v(b, s);
      return;
    }
    Tile& tile = tiles_[nodes_[n].tile];
    if (has_space(tile, s) || (tile.right - tile.left) <= 8) {  // mINtILEsIZE
      insert_tile(tile, s);
      return;
    }
    h_split(n);
    insert_h(n, s);
  }

  void insert_v(int n, int s) {  // insertShapeV (TileTree.hs:136-151)
    const BoxF& box = (*shapes_)[s].box;
    if (nodes_[n].kind == VTREE) {
      float cut = nodes_[n].cut;
      int a = nodes_[n].a, b = nodes_[n].b;
      if (box.top < cut) insert_h(a, s);
      if (box.bottom > cut) insert_h(b, s);
      return;
    }
    Tile& tile = tiles_[nodes_[n].tile];
    if (has_space(tile, s) || (tile.bottom - tile.top) <= 8) {
      insert_tile(tile, s);
      return;
    }
    v_split(n);
    insert_v(n, s);
  }

  // hSplit (TileTree.hs:175-181): node n becomes an HTree over two VLeafs and the
  // old contents are re-inserted in their original order.
  void h_split(int n) {
    Tile old = std::move(tiles_[nodes_[n].tile]);
    int cut = old.left + ((old.right - old.left) / 2);
    int l = new_leaf(VLEAF, old.hdepth - 1, old.vdepth, old.left, old.top, cut, old.bottom);
    int r = new_leaf(VLEAF, old.hdepth - 1, old.vdepth, cut, old.top, old.right, old.bottom);
    nodes_[n] = Node{HTREE, (float)cut, l, r, -1};
    ++splits_;
    for (int s : old.shapes) insert_h(n, s);
  }
  // vSplit (TileTree.hs:184-190)
  void v_split(int n) {
    Tile old = std::move(tiles_[nodes_[n].tile]);
    int cut = old.top + ((old.bottom - old.top) / 2);
    int t = new_leaf(HLEAF, old.hdepth, old.vdepth - 1, old.left, old.top, old.right, cut);
    int b = new_leaf(HLEAF, old.hdepth, old.vdepth - 1, old.left, cut, old.right, old.bottom);
    nodes_[n] = Node{VTREE, (float)cut, t, b, -1};
    ++splits_;
    for (int s : old.shapes) insert_v(n, s);
  }

  // traverseTileTree (TileTree.hs:193-204)
  template <class F>
  void trav_v(int n, F& f) {
    if (nodes_[n].kind == VTREE) {
      trav_h(nodes_[n].a, f);
      trav_h(nodes_[n].b, f);
    } else {
      f(tiles_[nodes_[n].tile]);
    }
  }
  template <class F>
  void trav_h(int n, F& f) {
    if (nodes_[n].kind == HTREE) {
      trav_v(nodes_[n].a, f);
      trav_v(nodes_[n].b, f);
    } else {
      f(tiles_[nodes_[n].tile]);
    }
  }

  int max_shape_;
  int64_t max_strands_;
  const std::vector<ShapeEntry>* shapes_;
  int tile_depth_ = 0;
  int root_ = -1;
  int splits_ = 0;
  std::vector<Node> nodes_;
  std::vector<Tile> tiles_;
};

}  // namespace

// ---------------------------------------------------------------- frame

struct gudni_frame {
  ProvSink prov;
  Pile<uint8_t> geometry;
  std::vector<float> substances;
  std::vector<gudni_picture_use> picture_uses;
  std::vector<gudni_radial> radials;
  struct Job {
    std::vector<gudni_shape> shapes;
    std::vector<gudni_tile_info> tiles;
    int32_t columns = 0;
  };
  std::vector<Job> jobs;
  int64_t stats[8] = {0};
};

namespace {

uint64_t make_tag(int kind, int compound, uint64_t substance_id) {  // ShapeInfo.hs:89-99
  uint64_t type = kind == GUDNI_SUBSTANCE_SOLID     ? GUDNI_TAG_SOLID
                  : kind == GUDNI_SUBSTANCE_PICTURE ? GUDNI_TAG_PICTURE
                                                    : GUDNI_TAG_RADIAL;
  uint64_t comb = compound == GUDNI_COMPOUND_SUBTRACT ? GUDNI_TAG_SUBTRACT : GUDNI_TAG_ADD;
  return type | comb | (substance_id & GUDNI_TAG_ID_MASK);
}

bool validate(const gudni_scene_desc* s, const gudni_spec* spec) {
  if (!s || !spec) { g_error = "null scene or spec"; return false; }
  if (s->canvas_w <= 0 || s->canvas_h <= 0) { g_error = "canvas must be positive"; return false; }
  if (spec->max_tile_size <= 0 || spec->max_tiles_per_call <= 0 || spec->threads_per_tile <= 0) {
    g_error = "spec sizes must be positive";
    return false;
  }
  if (s->n_substances < 0) { g_error = "negative substance count"; return false; }
  if (s->n_substances > 0 && (!s->substance_kind || !s->substance_shape_start)) {
    g_error = "missing substance arrays";
    return false;
  }
  return true;
}

}  // namespace

extern "C" {

const char* gudni_serialize_error(void) { return g_error.c_str(); }

gudni_frame* gudni_serialize(const gudni_scene_desc* s, const gudni_spec* spec) {
  g_error.clear();
  if (!validate(s, spec)) return nullptr;
  std::unique_ptr<gudni_frame> f(new gudni_frame());
  f->geometry.reserve(1 << 16);

  const float cw = (float)s->canvas_w, ch = (float)s->canvas_h;
  std::vector<ShapeEntry> entries;
  TileTree tree(spec->max_tile_size, s->canvas_w, s->canvas_h, spec->max_shape,
                (int64_t)spec->max_strands_per_tile, &entries);

  uint32_t picture_usage = 0;
  for (int sub = 0; sub < s->n_substances; ++sub) {
    // onSubstance (Serialize.hs:226-264): one id and one substance record per SRep.
    const uint64_t substance_id = (uint64_t)sub;
    const int kind = s->substance_kind[sub];
    float rec[4] = {0, 0, 0, 0};
    if (kind == GUDNI_SUBSTANCE_SOLID) {
      if (!s->substance_color) { g_error = "solid substance without colour"; return nullptr; }
      std::memcpy(rec, s->substance_color + 4 * sub, 16);
    } else if (kind == GUDNI_SUBSTANCE_PICTURE) {
      if (!s->substance_picture || !s->substance_picture_xform || !s->picture_size ||
          !s->picture_offset) {
        g_error = "picture substance without picture arrays";
        return nullptr;
      }
      int pid = s->substance_picture[sub];
      if (pid < 0 || pid >= s->n_pictures) { g_error = "picture index out of range"; return nullptr; }
      gudni_picture_use use;
      use.translate_x = s->substance_picture_xform[3 * sub + 0];
      use.translate_y = s->substance_picture_xform[3 * sub + 1];
      use.scale = s->substance_picture_xform[3 * sub + 2];
      use.size_x = s->picture_size[2 * pid];
      use.size_y = s->picture_size[2 * pid + 1];
      use.mem_offset = s->picture_offset[pid];
      f->picture_uses.push_back(use);
      uint32_t id = picture_usage++;
      std::memcpy(&rec[0], &id, 4);  // pokeM (ref :: PictId), then a zero word
    } else if (kind == GUDNI_SUBSTANCE_RADIAL) {
      if (!s->substance_radial) { g_error = "radial substance without gradient"; return nullptr; }
      uint32_t id = (uint32_t)f->radials.size();
      f->radials.push_back(s->substance_radial[sub]);
      std::memcpy(&rec[0], &id, 4);
    } else {
      g_error = "unknown substance kind";
      return nullptr;
    }
    f->substances.insert(f->substances.end(), rec, rec + 4);

    for (int sh = s->substance_shape_start[sub]; sh < s->substance_shape_start[sub + 1]; ++sh) {
      // onShape (Serialize.hs:148-177)
      int o0 = s->shape_outline_start[sh], o1 = s->shape_outline_start[sh + 1];
      BoxF box{std::numeric_limits<float>::infinity(), std::numeric_limits<float>::infinity(),
               -std::numeric_limits<float>::infinity(), -std::numeric_limits<float>::infinity()};
      for (int o = o0; o < o1; ++o) {
        for (int p = s->outline_pair_start[o]; p < s->outline_pair_start[o + 1]; ++p) {
          const float* q = s->pairs + 4 * p;
          for (int k = 0; k < 2; ++k) {  // boxOf (CurvePair c o) includes the control point
            float x = q[2 * k], y = q[2 * k + 1];
            box.left = box.left <= x ? box.left : x;
            box.top = box.top <= y ? box.top : y;
            box.right = box.right <= x ? x : box.right;
            box.bottom = box.bottom <= y ? y : box.bottom;
          }
        }
      }
      // excludeBox (Serialize.hs:97-104)
      if (box.left >= cw || box.top >= ch || box.right <= 0.0f || box.bottom <= 0.0f) {
        f->stats[1]++;
        continue;
      }
      size_t start_bytes = f->geometry.size();
      uint32_t strands = 0;
      for (int o = o0; o < o1; ++o) {
        int p0 = s->outline_pair_start[o];
        strands += outline_to_strands(s->pairs + 4 * p0, s->outline_pair_start[o + 1] - p0,
                                      f->geometry, &f->prov, p0);
      }
      ShapeEntry e;
      e.tag = make_tag(kind, s->shape_compound[sh], substance_id);
      e.geo_start = (uint32_t)(start_bytes / 16);  // appendGeoRef, Serialize.hs:83
      e.num_strands = strands;
      e.box = box;
      entries.push_back(e);
      tree.add((int)entries.size() - 1);
      f->stats[0]++;
      f->stats[2] += strands;
    }
  }

  // buildRasterJobs / accumulateRasterJobs (CallKernels.hs:244-255, Job.hs:132-178).
  // The reference passes (threadsPerTile, tilesPerCall) into parameters named
  // (maxTilesPerJob, threadsPerTile); both equal the device's maximum work-group size
  // there.  Here the tile count per job is max_tiles_per_call and each tile takes
  // threads_per_tile column slots.
  std::vector<gudni_frame::Job> built;
  built.emplace_back();
  int count = 0;
  tree.traverse([&](const Tile& tile) {
    if (count >= spec->max_tiles_per_call) {
      built.emplace_back();
      count = 0;
    }
    gudni_frame::Job& job = built.back();
    gudni_tile_info ti;
    ti.left = tile.left; ti.top = tile.top; ti.right = tile.right; ti.bottom = tile.bottom;
    ti.hdepth = (int16_t)tile.hdepth;
    ti.vdepth = (int16_t)tile.vdepth;
    ti.column_allocation = job.columns;
    ti.shapes.start = (uint32_t)job.shapes.size();
    ti.shapes.length = (uint32_t)tile.shapes.size();
    // the tile's list is newest-first (prepend), so emit in reverse insertion order
    for (auto it = tile.shapes.rbegin(); it != tile.shapes.rend(); ++it) {
      const ShapeEntry& e = entries[*it];
      job.shapes.push_back(gudni_shape{e.tag, e.geo_start, e.num_strands});
    }
    job.tiles.push_back(ti);
    job.columns += spec->threads_per_tile;
    ++count;
    f->stats[3]++;
    f->stats[5] = std::max<int64_t>(f->stats[5], tile.shape_count);
    f->stats[6] = std::max<int64_t>(f->stats[6], (int64_t)tile.strand_count);
    f->stats[7] += tile.shape_count;
  });
  f->stats[4] = tree.splits();
  // finalState ^. bsCurrentJob : finalState ^. bsJobs -- the last job first
  f->jobs.assign(built.rbegin(), built.rend());
  return f.release();
}

}  // extern "C"

namespace {

// The serializer's data-parallel passes (serialize_device.cuh) on host threads: every
// pass an OpenMP loop over its items (each item writes its own outputs), scans
// sequential.  Pile results land in the frame's own vectors.
struct ThreadExec {
  gudni_frame* f;
  int threads;
  std::vector<Pile<uint8_t>> slot = std::vector<Pile<uint8_t>>(gudni::ser::kSlots);

  template <class V>
  void* grow(V& v, uint64_t bytes) {
    v.resize((size_t)((bytes + sizeof(typename V::value_type) - 1) / sizeof(typename V::value_type)) + 1);
    return v.data();
  }
  template <class T>
  T* alloc(gudni::ser::Slot s, uint64_t n) {
    const uint64_t bytes = n * sizeof(T);
    switch (s) {
      case gudni::ser::kGeometry: return static_cast<T*>(grow(f->geometry, bytes));
      case gudni::ser::kPointSources: return static_cast<T*>(grow(f->prov.src, bytes));
      case gudni::ser::kPointWeights: return static_cast<T*>(grow(f->prov.w, bytes));
      case gudni::ser::kPointOffsets: return static_cast<T*>(grow(f->prov.where, bytes));
      default: {
        Pile<uint8_t>& v = slot[s];
        // 16-byte units keep every record type aligned
        if (v.size() < bytes + 16) v.resize((size_t)bytes + 16);
        return reinterpret_cast<T*>(v.data());
      }
    }
  }
  template <class Pass>
  int forEach(uint64_t n, const Pass& pass) {
    if (n < 2048 || threads <= 1) {
      for (uint64_t i = 0; i < n; ++i) pass(i);
      return 0;
    }
    const long long count = (long long)n;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 64)
    for (long long i = 0; i < count; ++i) pass((uint64_t)i);
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
    std::memmove(dst, src, bytes);
    return 0;
  }
  int copy(void* dst, const void* src, size_t bytes) {
    std::memmove(dst, src, bytes);
    return 0;
  }
  int upload(void* dst, const void* src, size_t bytes) {
    std::memmove(dst, src, bytes);
    return 0;
  }
};

}  // namespace

extern "C" {

gudni_frame* gudni_serialize_parallel(const gudni_scene_desc* s, const gudni_spec* spec, int threads) {
  g_error.clear();
  if (!validate(s, spec)) return nullptr;
  gudni::ser::Scene sc;
  int64_t n_pairs = 0;
  std::unique_ptr<gudni_frame> f(new gudni_frame());
  std::vector<float4> subs;
  std::vector<uint64_t> tags;
  const char* why = gudni::ser::checkScene(s, *spec, sc, n_pairs);
  if (!why) why = gudni::ser::buildSubstances(s, subs, f->picture_uses, f->radials, tags);
  if (why) {
    g_error = why;
    return nullptr;
  }
  f->substances.resize(subs.size() * 4);
  if (!subs.empty()) std::memcpy(f->substances.data(), subs.data(), subs.size() * sizeof(float4));
  sc.substance_shape_start = s->substance_shape_start;
  sc.substance_tag = tags.data();
  sc.shape_compound = s->shape_compound;
  sc.shape_outline_start = s->shape_outline_start;
  sc.outline_pair_start = s->outline_pair_start;
  sc.pairs = s->pairs;
  const gudni::ser::Limits lim{spec->max_tile_size, spec->threads_per_tile, spec->max_tiles_per_call,
                               spec->max_shape, (int64_t)spec->max_strands_per_tile};
#if defined(_OPENMP)
  const int all_threads = omp_get_max_threads();
#else  // built without OpenMP: the passes' loops run on the calling thread
  const int all_threads = 1;
#endif
  ThreadExec ex{f.get(), threads > 0 ? threads : all_threads};
  gudni::ser::Result r;
  const int rc = gudni::ser::serialize(ex, sc, lim, r, true);
  if (rc) {
    g_error = rc == -2 ? "scene too large" : "serializer failed";
    return nullptr;
  }
  f->geometry.resize((size_t)r.geometry_bytes);
  f->prov.src.resize((size_t)r.n_points * 3);
  f->prov.w.resize((size_t)r.n_points * 3);
  f->prov.where.resize((size_t)r.n_points);
  // the concatenated piles back into jobs: each job's tiles and shapes are contiguous
  f->jobs.resize((size_t)r.n_jobs);
  size_t t = 0;
  for (size_t j = 0; j < f->jobs.size(); ++j) {
    gudni_frame::Job& job = f->jobs[j];
    const size_t t0 = t;
    while (t < r.n_tiles && r.tile_jobs[t] == (int32_t)j) ++t;
    const uint32_t base = t0 < t ? r.tiles[t0].shapes.start : 0;
    uint64_t n = 0;
    for (size_t k = t0; k < t; ++k) {
      gudni_tile_info ti = r.tiles[k];
      ti.shapes.start -= base;
      n += ti.shapes.length;
      job.tiles.push_back(ti);
    }
    job.shapes.assign(r.shapes + base, r.shapes + base + n);
    job.columns = (int32_t)((t - t0) * (size_t)spec->threads_per_tile);
  }
  std::memcpy(f->stats, r.stats, sizeof(f->stats));
  return f.release();
}

void gudni_frame_free(gudni_frame* f) { delete f; }

size_t gudni_frame_geometry_bytes(const gudni_frame* f) { return f->geometry.size(); }
const uint8_t* gudni_frame_geometry(const gudni_frame* f) { return f->geometry.data(); }
size_t gudni_frame_n_substances(const gudni_frame* f) { return f->substances.size() / 4; }
const float* gudni_frame_substances(const gudni_frame* f) { return f->substances.data(); }
size_t gudni_frame_n_picture_uses(const gudni_frame* f) { return f->picture_uses.size(); }
const gudni_picture_use* gudni_frame_picture_uses(const gudni_frame* f) { return f->picture_uses.data(); }
size_t gudni_frame_n_radials(const gudni_frame* f) { return f->radials.size(); }
const gudni_radial* gudni_frame_radials(const gudni_frame* f) { return f->radials.data(); }
size_t gudni_frame_n_jobs(const gudni_frame* f) { return f->jobs.size(); }
size_t gudni_frame_job_n_shapes(const gudni_frame* f, size_t j) { return f->jobs[j].shapes.size(); }
const gudni_shape* gudni_frame_job_shapes(const gudni_frame* f, size_t j) { return f->jobs[j].shapes.data(); }
size_t gudni_frame_job_n_tiles(const gudni_frame* f, size_t j) { return f->jobs[j].tiles.size(); }
const gudni_tile_info* gudni_frame_job_tiles(const gudni_frame* f, size_t j) { return f->jobs[j].tiles.data(); }
int32_t gudni_frame_job_columns(const gudni_frame* f, size_t j) { return f->jobs[j].columns; }
size_t gudni_frame_n_points(const gudni_frame* f) { return f->prov.where.size(); }
const int32_t* gudni_frame_point_sources(const gudni_frame* f) { return f->prov.src.data(); }
const float* gudni_frame_point_weights(const gudni_frame* f) { return f->prov.w.data(); }
const uint32_t* gudni_frame_point_offsets(const gudni_frame* f) { return f->prov.where.data(); }

void gudni_frame_stats(const gudni_frame* f, int64_t out[8]) {
  for (int i = 0; i < 8; ++i) out[i] = f->stats[i];
}

}  // extern "C"
