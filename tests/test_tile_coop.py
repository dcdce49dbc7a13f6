"""The warp-cooperative work units (gudni_gb300/csrc/tile_coop.cuh) on the CPU: the
product's device code compiled for the host and run on an emulated 32-lane warp
(tests/host_column/warp_emu.h, lanes resuming in a seeded random order at every
collective), against the oracle, bit for bit.  The units' strands and (strand, column)
pairs are dealt to the lanes, the thresholds binned to the columns by ballots and
match masks; the per-column queue this builds must be the per-column generation's,
entry for entry, for every tile shape the tile tree makes (full tiles, split leaves
whose columns stack in slabs, canvas edges), every substance, tiles the units do not
take (more than 64 shapes, more than max_shape), overflowing columns and non-finite
coordinates."""
import ctypes as C
import os
import shutil
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.skipif(shutil.which("g++") is None or not os.path.isdir("/usr/local/cuda/include"),
                                reason="needs g++ and the CUDA headers")


def host_render_coop(frame, seed=1, capacity=None):
    """The frame through the cooperative units on the emulated warp; returns the image
    and the number of units taken cooperatively."""
    from host_column.build import load
    lib = load()
    cap = capacity or frame.spec.max_thresholds
    out = np.zeros((frame.canvas_h, frame.canvas_w), np.uint32)
    bg = np.ascontiguousarray(frame.background, np.float32)
    p = L.ptr
    taken = 0
    for ji, job in enumerate(frame.jobs):
        ov, tk = C.c_int(0), C.c_int(0)
        st = lib.host_column_raster_job_coop(p(frame.geometry), frame.geometry.size, p(frame.substances),
                                             len(frame.substances), p(frame.pictures), frame.pictures.size,
                                             p(frame.picture_uses), len(frame.picture_uses), p(frame.radials),
                                             len(frame.radials), p(job.shapes), len(job.shapes), p(job.tiles),
                                             len(job.tiles), frame.compute_depth, frame.canvas_w, frame.canvas_h,
                                             ji, bg.ctypes.data, p(frame.random_field),
                                             frame.spec.stochastic_factor, cap, frame.spec.max_thresholds,
                                             frame.spec.max_shape, seed, out.ctypes.data, C.byref(ov), C.byref(tk))
        assert st == 0 and ov.value == 0, (st, ov.value)
        taken += tk.value
    return out, taken


def check(frame, min_taken=1, **kw):
    got, taken = host_render_coop(frame, **kw)
    want = O.render_frame(frame)
    assert taken >= min_taken, taken
    assert np.array_equal(got, want), f"{int((got != want).sum())} of {got.size} pixels differ"
    return taken


@pytest.mark.parametrize("tile,tpt", [(32, 32), (32, 64), (16, 64), (8, 32), (16, 16), (32, 256)])
def test_random_scene_every_unit_shape(tile, tpt):
    """Single-slab units (32 columns of one slab, staged rows) and units whose columns
    stack in several slabs (narrow tiles, many threads per tile)."""
    flat = G.random_shapes(seed=5, width=150, height=110, n_shapes=30)
    check(S.serialize_flat(flat, L.make_spec(tile, tpt, 4096, 127, 8)))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_glyph_page_all_substances(seed):
    """Glyphs, local shapes, subtract, pictures and radial gradients, canvas edges that
    cut tiles; the lanes resume in a different order per seed."""
    flat = G.glyph_page(seed=4, width=330, height=190, n_glyphs=110, n_shapes=20)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 127, 8))
    assert len(frame.radials) and len(frame.picture_uses)
    check(frame, min_taken=20, seed=seed)


def test_leaves_split_by_the_strand_limit():
    """A low strand limit splits leaves down to 8 pixels: units of split leaves hold
    several slabs of short columns."""
    flat = G.glyph_page(seed=7, width=200, height=120, n_glyphs=90, n_shapes=10)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 127, 8, max_strands_per_tile=60))
    tiles = np.concatenate([j.tiles for j in frame.jobs])
    assert (tiles["hdepth"] < 5).any()
    check(frame, min_taken=5)


def test_tiles_beyond_the_units_run_per_column():
    """Tiles with more than 64 shapes (and a max_shape below the tile's shape count) are
    not taken; the per-column code renders them, and the image is the same."""
    flat = G.random_shapes(seed=9, width=96, height=64, n_shapes=90, seg_lo=4, seg_hi=8)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 8192, 255, 4))
    got, taken = host_render_coop(frame)
    assert np.array_equal(got, O.render_frame(frame))
    small = S.serialize_flat(G.random_shapes(seed=9, width=64, height=64, n_shapes=40, seg_lo=4, seg_hi=8),
                             L.make_spec(32, 32, 8192, 31, 1))
    assert np.array_equal(host_render_coop(small)[0], O.render_frame(small))


def test_overflowing_columns_take_the_full_pass():
    """A working capacity below the longest column: those columns are redone at full
    capacity, the others are kept."""
    flat = G.random_shapes(seed=11, width=128, height=96, n_shapes=24)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 127, 8))
    check(frame, capacity=24)


def test_dense_columns_one_word():
    """Up to 64 canvas-wide shapes per tile: long queues, many shape bits, the colour
    memo and the batched insertion of split parts."""
    flat = G.random_shapes(seed=13, width=96, height=80, n_shapes=60)
    check(S.serialize_flat(flat, L.make_spec(32, 32, 4096, 127, 8)))


def test_non_finite_and_extreme_coordinates():
    """NaN and infinite control points (a NaN range test takes no column; a NaN key
    sends the queue to the bubble sort) and coordinates near float max."""
    from test_host_column import _extreme
    flat = G.random_shapes(seed=77, width=96, height=80, n_shapes=10)
    flat.pairs = flat.pairs.copy()
    flat.pairs[3, 1] = np.nan
    flat.pairs[17, 2] = np.inf
    flat.pairs[40, 0] = np.nan
    check(S.serialize_flat(flat, L.make_spec(16, 32, 4096, 127, 8)))
    near_max = S.serialize_flat(_extreme(16, 8, 1, 6, [3.4e38, -3.4e38, 3.4e38]), L.make_spec(8, 8, 4096, 127, 2))
    check(near_max)


def test_tiny_and_empty_scenes():
    frame = S.serialize(S.Scene((0.2, 0.4, 0.6, 1.0), S.EMPTY), 37, 23, L.make_spec(16, 16, 64))
    got, _ = host_render_coop(frame)
    assert np.array_equal(got, O.render_frame(frame))
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import fixture_scenes as F
    for name in ("tiny_square", "knob", "hourglass", "six_point_rectangle", "two_brackets", "open_squares",
                 "textured", "radial", "thin_rectangles"):
        frame = F.build(name)
        got, _ = host_render_coop(frame)
        assert np.array_equal(got, O.render_frame(frame)), name
