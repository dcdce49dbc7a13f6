"""Host serializer: strand layout, reorder table, tile tree and job packing
(Raster/Strand.hs, ReorderTable.hs, TileTree.hs, Job.hs)."""
import numpy as np
import pytest

from gudni_gb300 import lib as L
from gudni_gb300 import scene as S
from gudni_gb300 import scenes as G


def strands_of(frame):
    """Decode the geometry pile into per-strand point lists (reordered order)."""
    geo = frame.geometry
    out = []
    off = 0
    while off < geo.size:
        size = int(np.frombuffer(geo[off:off + 2].tobytes(), np.uint16)[0])
        pts = np.frombuffer(geo[off + 8: off + 8 * size].tobytes(), np.float32).reshape(-1, 2)
        out.append((size, pts))
        off += 8 * size
    return out


def inorder(pts):
    """Undo the reorder: right point, left point + control, then the BFS tree of
    (point, control) pairs -> left-to-right point sequence."""
    right, left, ctl = pts[0], pts[1], pts[2]
    tree = pts[3:].reshape(-1, 2, 2)
    seq = []

    def walk(i):
        if i >= len(tree):
            return
        walk(2 * i + 1)
        seq.append(tree[i][0])
        seq.append(tree[i][1])
        walk(2 * i + 2)

    walk(0)
    return np.array([left, ctl] + seq + [right])


def test_single_straight_square_layout():
    sq = S.segments_to_outline([S.straight(0, 0), S.straight(4, 0), S.straight(4, 4), S.straight(0, 4)])
    frame = S.serialize(S.Scene((1, 1, 1, 1), S.solid((1, 0, 0, 1), S.shape([sq]))), 8, 8, L.make_spec(8, 8, 64))
    strands = strands_of(frame)
    # the two vertical edges are strands of their own; the horizontal edges are strands
    assert len(strands) == 4
    for size, pts in strands:
        assert size % 2 == 0 and size == 1 + pts.shape[0]
        xs = inorder(pts)[0::2, 0]
        assert np.all(np.diff(xs) >= 0), "strand on-curve points must run left to right"
    shapes = frame.jobs[0].shapes
    assert shapes[0]["num_strands"] == 4 and shapes[0]["geo_start"] == 0
    assert shapes[0]["tag"] == (L.TAG_SOLID | L.TAG_ADD | 0)


def test_reorder_tree_recovers_sequence():
    """A 15-curve x-monotone run becomes one strand whose tree reproduces the run."""
    xs = np.arange(16, dtype=np.float32) * 2
    seg = [S.curved(x, 10 + (i % 3), x + 1, 12 + (i % 2)) for i, x in enumerate(xs[:-1])]
    seg.append(S.straight(xs[-1], 30))
    seg.append(S.straight(0, 30))
    frame = S.serialize(S.Scene((1, 1, 1, 1), S.solid((0, 0, 0, 1), S.shape([S.segments_to_outline(seg)]))),
                        40, 40, L.make_spec(64, 64, 64))
    strands = strands_of(frame)
    longest = max(strands, key=lambda s: s[0])
    seq = inorder(longest[1])
    on = seq[0::2]
    assert np.all(np.diff(on[:, 0]) > 0)
    assert longest[0] == 2 * 15 + 2


def test_knob_is_split():
    knob = S.segments_to_outline([S.curved(0, 0, 10, 10), S.straight(0, 20)])
    frame = S.serialize(S.Scene((1, 1, 1, 1), S.solid((0, 0, 0, 1), S.shape([knob]))), 32, 32, L.make_spec(32, 32, 64))
    for size, pts in strands_of(frame):
        seq = inorder(pts)
        on = seq[0::2, 0]
        ctl = seq[1::2, 0]
        for a, c, b in zip(on[:-1], ctl, on[1:]):
            assert min(a, b) <= c <= max(a, b) or a == b, "no control point may bulge past its curve"


@pytest.mark.parametrize("w,h,tile,tpt", [(512, 512, 32, 32), (100, 70, 16, 32), (33, 65, 8, 8)])
def test_tiles_cover_canvas_once(w, h, tile, tpt):
    flat = G.random_shapes(seed=5, width=w, height=h, n_shapes=30)
    frame = S.serialize_flat(flat, L.make_spec(tile, tpt, 256, 127, 8))
    cover = np.zeros((h, w), np.int32)
    cd = frame.compute_depth
    for job in frame.jobs:
        for t in job.tiles:
            for column in range(tpt):
                hd, vd = int(t["hdepth"]), int(t["vdepth"])
                diff = max(0, vd - (cd - hd))
                ix = ((1 << hd) - 1) & column
                iy = (column >> hd) << diff
                dx, dy = ix + t["left"], iy + t["top"]
                if iy < t["bottom"] - t["top"] and dx < w and dy < h:
                    hh = min(1 << diff, h - dy)
                    cover[dy:dy + hh, dx] += 1
    assert np.all(cover == 1)


def test_tile_split_and_jobs():
    flat = G.random_shapes(seed=0)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 1024, 127, 8, max_tiles_per_call=1024))
    # 64 random shapes hold ~1700 strands, above max_strands_per_tile=1022, so tiles
    # split down to the 8x8 minimum (TileTree.hs:130, 147)
    assert frame.stats["splits"] > 0
    sizes = {(int(t["right"] - t["left"]), int(t["bottom"] - t["top"])) for j in frame.jobs for t in j.tiles}
    assert (8, 8) in sizes
    assert all(len(j.tiles) <= 1024 for j in frame.jobs)
    # the last job built comes first; column allocations restart per job
    for j in frame.jobs:
        assert j.tiles[0]["column_allocation"] == 0
        assert j.columns == len(j.tiles) * 32


def test_excluded_shapes():
    inside = S.segments_to_outline([S.straight(1, 1), S.straight(5, 1), S.straight(5, 5)])
    outside = S.segments_to_outline([S.straight(50, 50), S.straight(60, 50), S.straight(60, 60)])
    tree = S.overlap([S.solid((1, 0, 0, 1), S.shape([inside])), S.solid((0, 1, 0, 1), S.shape([outside]))])
    frame = S.serialize(S.Scene((1, 1, 1, 1), tree), 16, 16, L.make_spec(16, 16, 64))
    assert frame.stats["shapes"] == 1 and frame.stats["excluded"] == 1
    assert len(frame.substances) == 2  # a substance record per SRep, kept or not


def test_subtract_tags_and_order():
    a = S.shape([S.segments_to_outline([S.straight(0, 0), S.straight(8, 0), S.straight(8, 8)])])
    b = S.shape([S.segments_to_outline([S.straight(1, 1), S.straight(4, 1), S.straight(4, 4)])])
    frame = S.serialize(S.Scene((1, 1, 1, 1), S.solid((1, 0, 0, 1), S.cSubtract(a, b))), 16, 16,
                        L.make_spec(16, 16, 64))
    tags = frame.jobs[0].shapes["tag"]
    # b is visited first (above) with the subtract tag; tile lists are newest-first
    assert list(tags & L.TAG_COMPOUND_MASK) == [L.TAG_ADD, L.TAG_SUBTRACT]


def test_bad_input_rejected():
    flat = G.random_shapes(seed=1, width=64, height=64, n_shapes=3)
    flat.substance_kind[0] = 9
    with pytest.raises(ValueError):
        S.serialize_flat(flat, L.make_spec(16, 16, 64))
