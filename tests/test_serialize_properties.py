"""Structural properties of the serialized piles that the raster kernels rely on
(the reference's serializer cannot run here, so these pin the restatement's output
by its invariants): strand headers and sizes, x-monotone strands with their ends in
the header slots, binary-search-tree order of the strand trees (searchTree,
Kernels.cl:1337-1357), and tiles that list every shape whose points reach into them."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402


def strands_of(frame, shape):
    geo = frame.geometry
    off = int(shape["geo_start"]) * 16
    out = []
    for _ in range(int(shape["num_strands"])):
        size = int(np.frombuffer(geo[off:off + 2].tobytes(), np.uint16)[0])
        pts = np.frombuffer(geo[off + 8:off + size * 8].tobytes(), np.float32).reshape(-1, 2)
        out.append((size, pts))
        off += size * 8
    return out


def inorder(i, n):
    return [] if i >= n else inorder(2 * i + 1, n) + [i] + inorder(2 * i + 2, n)


FRAMES = {
    "random": lambda: S.serialize_flat(G.random_shapes(seed=12, width=300, height=200, n_shapes=40),
                                       L.make_spec(32, 32, 4096, 127, 8)),
    "glyphs": lambda: S.serialize_flat(G.glyph_page(seed=6, width=480, height=270, n_glyphs=150, n_shapes=25),
                                       L.make_spec(32, 32, 4096, 511, 8)),
}


@pytest.mark.parametrize("name", sorted(FRAMES))
def test_strand_layout(name):
    frame = FRAMES[name]()
    seen = 0
    for job in frame.jobs:
        for shape in job.shapes:
            for size, pts in strands_of(frame, shape):
                assert size >= 4 and size % 2 == 0                 # 2k+2 eight-byte units, k >= 1 curves
                assert len(pts) == size - 1                         # 2k+1 points after the header
                right, left, tree = pts[0], pts[1], pts[3:].reshape(-1, 2, 2)
                # the tree's on-curve points in order lie between the ends, x never
                # decreasing (a vertical segment keeps x equal)
                xs = [tree[i, 0, 0] for i in inorder(0, len(tree))]
                on = [left[0]] + xs + [right[0]]
                assert all(a <= b for a, b in zip(on, on[1:])), on
                seen += 1
    assert seen > 50


@pytest.mark.parametrize("name", sorted(FRAMES))
def test_tiles_list_every_shape_reaching_them(name):
    frame = FRAMES[name]()
    for job in frame.jobs:
        boxes = []
        for shape in job.shapes:
            pts = np.concatenate([p for _, p in strands_of(frame, shape)])
            boxes.append((pts[:, 0].min(), pts[:, 1].min(), pts[:, 0].max(), pts[:, 1].max()))
        # shapes are deduplicated per job by their geometry start
        for t in job.tiles:
            listed = {int(job.shapes[i]["geo_start"]) for i in range(t["shape_start"], t["shape_start"] + t["shape_length"])}
            for k, (x0, y0, x1, y1) in enumerate(boxes):
                inside = x0 < t["right"] - 1e-3 and x1 > t["left"] + 1e-3 and y0 < t["bottom"] - 1e-3 and y1 > t["top"] + 1e-3
                if inside:
                    assert int(job.shapes[k]["geo_start"]) in listed, (dict(zip(t.dtype.names, t.tolist())), k)


def test_jobs_partition_the_tiles():
    spec = L.make_spec(32, 32, 4096, 511, 8, max_tiles_per_call=40)
    frame = S.serialize_flat(G.glyph_page(seed=6, width=480, height=270, n_glyphs=150, n_shapes=25), spec)
    assert len(frame.jobs) > 3
    total = 0
    for job in frame.jobs:
        assert 0 < len(job.tiles) <= spec.max_tiles_per_call
        for t in job.tiles:
            assert t["shape_start"] + t["shape_length"] <= len(job.shapes)
        total += len(job.tiles)
    assert total == frame.n_tiles
    boxes = np.concatenate([np.stack([j.tiles["left"], j.tiles["top"], j.tiles["right"], j.tiles["bottom"]], 1)
                            for j in frame.jobs])
    depths = np.concatenate([np.stack([j.tiles["hdepth"], j.tiles["vdepth"]], 1) for j in frame.jobs])
    assert np.all(boxes[:, 2] - boxes[:, 0] == 1 << depths[:, 0].astype(np.int64))
    assert np.all(boxes[:, 3] - boxes[:, 1] == 1 << depths[:, 1].astype(np.int64))
    assert np.all(boxes[:, 2] - boxes[:, 0] <= spec.max_tile_size)
    # the tile tree's leaves cover its square exactly once
    side = 1 << L.compute_depth(max(frame.canvas_w, frame.canvas_h))
    cover = np.zeros((side, side), np.int32)
    for x0, y0, x1, y1 in boxes:
        assert 0 <= x0 < x1 <= side and 0 <= y0 < y1 <= side
        cover[y0:y1, x0:x1] += 1
    assert np.all(cover == 1)
