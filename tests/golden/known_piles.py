"""TEST INFRASTRUCTURE -- known-answer piles for the serializer, derived by hand from
the reference's Haskell host.

The reference pins no serializer output (it has no tests, and GHC is not available
to run it here), so the serializer restatements (gudni_gb300/csrc/serialize.cpp, and
the device passes of serialize_device.cuh) are pinned here against a second,
independent restatement written step by step from the Haskell source, in numpy
float32 (SubSpace is Float):

* strands: pairsToBeziers, replaceKnobs / fixKnob / findSplit, splitIntoStrands (the
  last run first: `acc V.cons strands`), splitTooLarge at mAXsECTIONsIZE / 2 = 16
  curves, reverseIfBackwards, beziersToPoints, reorder through buildReorderTable,
  and the Strand poke (u16 size in 8-byte units, u16 0, u32 0, then the points)
  -- Raster/Strand.hs:88-206, Raster/Deknob.hs:37-108, Raster/ReorderTable.hs:30-118,
  Raster/Enclosure.hs:62-80;
* shapes: excludeBox, the bounding box of every on- and off-curve point, appendGeoRef
  (geo_start in 16-byte units), makeShapeTag -- Raster/Serialize.hs:76-177,
  Figure/Outline.hs:123-133, Raster/ShapeInfo.hs:89-99;
* the tile tree: buildTileTree, addShapeToTree with checkTileSpace (fewer than
  mAXsHAPE - 1 shapes and fewer than max strands per tile), hSplit / vSplit
  re-inserting the old shapes oldest first, mINtILEsIZE 8 -- Raster/TileTree.hs:81-204;
* jobs: traverseTileTree order, accumulateRasterJobs (a tile's shapes newest first,
  column allocation in steps of threads per tile), the last job first --
  Raster/Job.hs:132-178, OpenCL/CallKernels.hs:244-255.

The scenes are given as flattened scenes (one shape per substance, each shape one
or more outlines of curve pairs), the form both serializers take; the ShapeTree
walk that produces them is not part of what is pinned.  Run as a script to write
known_piles.json (hex of the geometry pile and of every job's shape and tile
records); tests/test_known_piles.py checks both serializers against it and checks
that this derivation still produces it.
"""
from __future__ import annotations

import json
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
F32 = np.float32
ITA = F32(0.0001)          # iota for SubSpace, Figure/Space.hs:101-102
SPLIT = F32(0.5)           # sPLIT, Deknob.hs:37
MAX_SECTION = 32           # mAXsECTIONsIZE, Constants.hs:67
MAX_SHAPE = 127            # mAXsHAPE, Constants.hs:58
MIN_TILE = 8               # mINtILEsIZE, Constants.hs:66
SOLID, ADD = 0x8000000000000000, 0x2000000000000000


# ---------------------------------------------------------------- strands
def between(t, a, b):
    """(a ^* (1-t)) ^+^ (b ^* t), per component in float32 (Deknob.hs)."""
    one = F32(1.0)
    return (a[0] * (one - t) + b[0] * t, a[1] * (one - t) + b[1] * t)


def curve_point(t, v0, c, v1):
    m0 = between(t, v0, c)
    m1 = between(t, c, v1)
    return m0, between(t, m0, m1), m1


def find_split(stays, t, v0, c, v1):
    bottom, top = F32(0.0), F32(1.0)
    while True:
        m0, on, m1 = curve_point(t, v0, c, v1)
        if top - bottom <= ITA:
            return m0, on, m1
        if stays(m1, on):
            bottom, t = t, F32(t + (top - t) / F32(2.0))
        elif stays(m0, on):
            top, t = t, F32(bottom + (t - bottom) / F32(2.0))
        else:
            return m0, on, m1


def left_of(a, b):
    return a[0] < b[0]


def right_of(a, b):
    return a[0] > b[0]


def fix_knob(bez):
    v0, c, v1 = bez
    for stays in (left_of, right_of):
        if stays(c, v0) and stays(c, v1):
            m0, on, m1 = find_split(stays, SPLIT, v0, c, v1)
            return [(v0, m0, on), (on, m1, v1)]
    return [bez]


def cmp(a, b):
    return int(a > b) - int(a < b)


def connectable(a, b):
    ha, hb = cmp(a[0][0], a[2][0]), cmp(b[0][0], b[2][0])
    return ha == hb and ha != 0


def split_into_strands(beziers):
    acc, strands = [], []
    for b in beziers:
        if not acc:
            acc = [b]
        elif connectable(acc[-1], b):
            acc.append(b)
        else:
            strands.append(acc)
            acc = [b]
    return [acc] + strands


def split_too_large(n, v):
    return [v[i:i + n] for i in range(0, len(v), n)] if len(v) > n else [v]


def reverse_if_backwards(v):
    if v[0][0][0] > v[-1][2][0]:
        return [(b[2], b[1], b[0]) for b in reversed(v)]
    return v


def beziers_to_points(v):
    pts = []
    for b in v:
        pts += [b[0], b[1]]
    return pts + [v[-1][2]]


def perfect_tree_partition(n):
    x = 1
    while x <= n // 2:
        x *= 2
    return x - 1 if (x // 2) - 1 <= n - x else n - (x // 2)


def build_itree(xs):
    if not xs:
        return None
    half = perfect_tree_partition(len(xs))
    return (xs[half], build_itree(xs[:half]), build_itree(xs[half + 1:]))


def breadth(node):
    out, level = [], [node]
    while level:
        nxt = []
        for nd in level:
            if nd is not None:
                out.append(nd[0])
                nxt += [nd[1], nd[2]]
        level = nxt
    return out


def make_tree_row(size):
    half = breadth(build_itree(list(range(size // 2))))
    row = []
    for x in half:
        row += [2 * x, 2 * x + 1]
    return row


def reorder_for_extents(size):
    if size < 3:
        return []
    return [size - 1, 0, 1] + ([i + 2 for i in make_tree_row(size - 3)] if size > 3 else [])


def reorder(pts):
    row = reorder_for_extents(len(pts))  # the table row of len(pts) // 2 is built for 2 * (len // 2) + 1
    return [pts[i] for i in row]


def outline_strands(pairs):
    """pairs: [(on_x, on_y, off_x, off_y)] of one outline -> list of point lists."""
    if len(pairs) < 2:
        return []
    pts = [((F32(p[0]), F32(p[1])), (F32(p[2]), F32(p[3]))) for p in pairs]
    beziers = [(pts[i][0], pts[i][1], pts[(i + 1) % len(pts)][0]) for i in range(len(pts))]
    beziers = [b for bez in beziers for b in fix_knob(bez)]
    out = []
    for strand in split_into_strands(beziers):
        for part in split_too_large(MAX_SECTION // 2, strand):
            out.append(reorder(beziers_to_points(reverse_if_backwards(part))))
    return out


def poke_strand(points) -> bytes:
    size = (8 + 8 * len(points)) // 8
    b = struct.pack("<HHI", size, 0, 0)
    for x, y in points:
        b += struct.pack("<ff", float(x), float(y))
    return b


# ---------------------------------------------------------------- tile tree
class Tile:
    def __init__(self, hdepth, vdepth, box):
        self.hdepth, self.vdepth, self.box = hdepth, vdepth, box  # box: [left, top, right, bottom]
        self.shapes = []  # newest first
        self.strands = 0


def adjusted_log(x):
    return 0 if x < 1 else int(np.ceil(np.log2(x)))


def build_tile_tree(tile_size, w, h):
    depth, tdepth = adjusted_log(max(w, h)), adjusted_log(tile_size)

    def go_v(d, box):
        cut = box[1] + 2 ** (d - 1)
        if d > tdepth:
            return ["V", cut, go_h(d, [box[0], box[1], box[2], cut]), go_h(d, [box[0], cut, box[2], box[3]])]
        return ["VL", Tile(d, d, box)]

    def go_h(d, box):
        cut = box[0] + 2 ** (d - 1)
        if d > tdepth:
            return ["H", cut, go_v(d - 1, [box[0], box[1], cut, box[3]]), go_v(d - 1, [cut, box[1], box[2], box[3]])]
        return ["HL", Tile(d, d, box)]

    return go_v(depth, [0, 0, 2 ** depth, 2 ** depth])


def add_shape(tree, entry, max_strands):
    """entry: dict(box=(l, t, r, b) float32, strands=n, ...)."""
    def put(tile, e):
        tile.shapes.insert(0, e)
        tile.strands += e["strands"]

    def ins_h(node, e):
        if node[0] == "H":
            if e["box"][0] < F32(node[1]):
                node[2] = ins_v(node[2], e)
            if e["box"][2] > F32(node[1]):
                node[3] = ins_v(node[3], e)
            return node
        tile = node[1]
        if fits_e(tile, e) or tile.box[2] - tile.box[0] <= MIN_TILE:
            put(tile, e)
            return node
        return ins_h(h_split(tile), e)

    def ins_v(node, e):
        if node[0] == "V":
            if e["box"][1] < F32(node[1]):
                node[2] = ins_h(node[2], e)
            if e["box"][3] > F32(node[1]):
                node[3] = ins_h(node[3], e)
            return node
        tile = node[1]
        if fits_e(tile, e) or tile.box[3] - tile.box[1] <= MIN_TILE:
            put(tile, e)
            return node
        return ins_v(v_split(tile), e)

    def fits_e(tile, e):
        return len(tile.shapes) < MAX_SHAPE - 1 and tile.strands + e["strands"] < max_strands

    def h_split(tile):
        cut = tile.box[0] + (tile.box[2] - tile.box[0]) // 2
        node = ["H", cut, ["VL", Tile(tile.hdepth - 1, tile.vdepth, [tile.box[0], tile.box[1], cut, tile.box[3]])],
                ["VL", Tile(tile.hdepth - 1, tile.vdepth, [cut, tile.box[1], tile.box[2], tile.box[3]])]]
        for e in reversed(tile.shapes):
            node = ins_h(node, e)
        return node

    def v_split(tile):
        cut = tile.box[1] + (tile.box[3] - tile.box[1]) // 2
        node = ["V", cut, ["HL", Tile(tile.hdepth, tile.vdepth - 1, [tile.box[0], tile.box[1], tile.box[2], cut])],
                ["HL", Tile(tile.hdepth, tile.vdepth - 1, [tile.box[0], cut, tile.box[2], tile.box[3]])]]
        for e in reversed(tile.shapes):
            node = ins_v(node, e)
        return node

    return ins_v(tree, entry)


def traverse(node, fn):
    if node[0] in ("V", "H"):
        traverse(node[2], fn)
        traverse(node[3], fn)
    else:
        fn(node[1])


# ---------------------------------------------------------------- a frame
def derive(shapes, canvas_w, canvas_h, tile_size, threads_per_tile, tiles_per_job, max_strands):
    """shapes: [[outline pairs, ...] per shape], each the only shape of its substance
    (id = its index), solid, added.  Returns the geometry pile and the jobs (shape and
    tile records as bytes), last job first."""
    geo = b""
    tree = build_tile_tree(tile_size, canvas_w, canvas_h)
    for sid, outlines in enumerate(shapes):
        allp = np.asarray([p for o in outlines for p in o], np.float32)
        xs, ys = np.concatenate([allp[:, 0], allp[:, 2]]), np.concatenate([allp[:, 1], allp[:, 3]])
        box = (xs.min(), ys.min(), xs.max(), ys.max())
        if box[0] >= canvas_w or box[1] >= canvas_h or box[2] <= 0 or box[3] <= 0:  # excludeBox
            continue
        strands = [s for o in outlines for s in outline_strands(o)]
        start = len(geo) // 16
        for s in strands:
            geo += poke_strand(s)
        entry = {"box": box, "strands": len(strands), "tag": SOLID | ADD | sid, "geo": start}
        tree = add_shape(tree, entry, max_strands)
    jobs = [{"shapes": b"", "tiles": b"", "n_shapes": 0, "columns": 0, "count": 0}]

    def acc(tile):
        job = jobs[-1]
        if job["count"] >= tiles_per_job:
            jobs.append({"shapes": b"", "tiles": b"", "n_shapes": 0, "columns": 0, "count": 0})
            job = jobs[-1]
        first = job["n_shapes"]
        for e in tile.shapes:  # newest first
            job["shapes"] += struct.pack("<QII", e["tag"], e["geo"], e["strands"])
        job["n_shapes"] += len(tile.shapes)
        b = tile.box
        job["tiles"] += struct.pack("<iiiihhiII", b[0], b[1], b[2], b[3], tile.hdepth, tile.vdepth, job["columns"],
                                    first, len(tile.shapes))
        job["columns"] += threads_per_tile
        job["count"] += 1

    traverse(tree, acc)
    return geo, [{"shapes": j["shapes"], "tiles": j["tiles"]} for j in reversed(jobs)]


# ---------------------------------------------------------------- the scenes
def scenes():
    """name -> (shapes, canvas_w, canvas_h, tile, threads per tile, tiles per job, strands per tile)."""
    out = {}
    # simpleKnob (benchmarks/GudniTests.hs:247-255) placed on a small canvas: a curve
    # whose control point bulges right of both ends (split by findSplit) and a
    # straight return (its control the midpoint)
    out["knob"] = ([[[(5, 3, 15, 13), (5, 23, 5, 13)]]], 24, 28, 16, 16, 64, 4094)
    # a left bulging knob with an off-axis control, and a shape of two outlines
    out["left_knob_two_outlines"] = ([[[(20, 2, 1, 9.5), (20, 17, 20.5, 9.5)]],
                                      [[(2, 2, 6, 1), (10, 2, 10, 6), (10, 10, 6, 11), (2, 10, 1.5, 6)],
                                       [(4, 4, 4, 6), (4, 8, 6, 8), (8, 8, 8, 6), (8, 4, 6, 4)]]],
                                     24, 20, 16, 16, 64, 4094)
    # one outline of 21 curves rising left to right, then a vertical drop and a
    # straight return: strands of 16 and 5 curves (splitTooLarge), the vertical
    # segment alone, and the return reversed
    zig = [(2 + 2 * i, 20 + (3 if i % 2 else -3) * 0.5, 3 + 2 * i, 10 + (i % 3)) for i in range(21)]
    zig += [(44, 30, 44, 35), (44, 40, 23, 40)]
    out["long_strands"] = ([[zig]], 48, 48, 16, 16, 64, 4094)
    # 130 small rectangles over one corner: the first leaf fills to mAXsHAPE - 1
    # shapes, splits vertically and horizontally down to 8 pixels, re-inserting its
    # shapes oldest first; tiles past the canvas are listed with no shapes; jobs of
    # 2 tiles, the last job first
    rects = []
    for i in range(130):
        x0, y0 = 1 + (i % 13) * 2.1, 1 + (i // 13) * 2.7
        rects.append([[(x0, y0, x0 + 0.5, y0), (x0 + 1, y0, x0 + 1, y0 + 0.5), (x0 + 1, y0 + 1, x0 + 0.5, y0 + 1),
                       (x0, y0 + 1, x0, y0 + 0.5)]])
    out["crowded_leaf"] = (rects, 40, 36, 32, 32, 2, 4094)
    # a strand limit that splits leaves: 30 long thin shapes of 6 strands each
    thin = []
    for i in range(30):
        y = 2 + i
        thin.append([[(1, y, 10, y - 0.4), (20, y, 30, y + 0.4), (38, y, 38, y + 0.3), (38, y + 0.6, 20, y + 0.9),
                      (1, y + 0.6, 1, y + 0.3)]])
    out["strand_limit"] = (thin, 40, 40, 32, 32, 64, 40)
    return out


def flat_scene(shapes, w, h):
    """The same scene as a gudni_gb300 FlatScene (one solid substance per shape)."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from gudni_gb300 import lib as L
    from gudni_gb300 import scene as S
    n = len(shapes)
    pairs, outline_start, shape_outline_start = [], [], []
    for outlines in shapes:
        shape_outline_start.append(len(outline_start))
        for o in outlines:
            outline_start.append(len(pairs))
            pairs += list(o)
    outline_start.append(len(pairs))
    shape_outline_start.append(len(outline_start) - 1)
    rng = np.random.default_rng(0)
    return S.FlatScene(
        canvas_w=w, canvas_h=h, background=np.asarray([1, 1, 1, 1], np.float32),
        substance_kind=np.zeros(n, np.int32), substance_color=rng.random((n, 4), dtype=np.float32),
        substance_picture=np.zeros(n, np.int32),
        substance_picture_xform=np.tile(np.asarray([0, 0, 1], np.float32), (n, 1)),
        substance_radial=np.zeros(n, dtype=L.RADIAL_DTYPE), substance_shape_start=np.arange(n + 1, dtype=np.int32),
        shape_compound=np.full(n, S.ADD, np.int32), shape_outline_start=np.asarray(shape_outline_start, np.int32),
        outline_pair_start=np.asarray(outline_start, np.int32), pairs=np.asarray(pairs, np.float32).reshape(-1, 4),
        pictures=np.zeros(0, np.uint8), picture_size=np.zeros((0, 2), np.int32),
        picture_offset=np.zeros(0, np.int32))


def derive_all():
    out = {}
    for name, (shapes, w, h, tile, tpt, per_job, max_strands) in scenes().items():
        geo, jobs = derive(shapes, w, h, tile, tpt, per_job, max_strands)
        out[name] = {"canvas": [w, h], "tile": tile, "threads_per_tile": tpt, "tiles_per_job": per_job,
                     "max_strands_per_tile": max_strands, "geometry": geo.hex(),
                     "jobs": [{"shapes": j["shapes"].hex(), "tiles": j["tiles"].hex()} for j in jobs]}
    return out


if __name__ == "__main__":
    with open(os.path.join(HERE, "known_piles.json"), "w") as f:
        json.dump(derive_all(), f, indent=1)
    print("wrote known_piles.json")
