"""CUDA raster path against the golden fixtures (reference kernels) and the oracle,
through the C ABI.  Parity bar: <=1 LSB per channel and >=99.9% of pixels exact; the
kernels are expected to be bit-exact and the tests report the exact fraction."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)

import fixture_scenes as F  # noqa: E402
from conftest import assert_parity  # noqa: E402
from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402
from gudni_gb300.raster import RasterError, Rasterizer  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN, "golden.json")) as f:
    INDEX = json.load(f)


def render(frame, **kw):
    with Rasterizer(frame.spec) as r:
        return r.queue_jobs(frame, **kw)


@pytest.mark.parametrize("name", F.ALL)
def test_golden_fixtures(name):
    frame = F.build(name)
    got = render(frame)
    entry = INDEX[name]
    if "image_file" in entry:
        want = np.load(os.path.join(GOLDEN, entry["image_file"]))
    else:
        want = O.render_frame(frame)
    assert_parity(got, want)
    assert np.array_equal(got, want), f"{(got != want).sum()} pixels differ (within tolerance)"


@pytest.mark.parametrize("tpt,tile", [(32, 32), (64, 32), (128, 32), (16, 16), (256, 16)])
def test_random_scene_threads_per_tile(tpt, tile):
    flat = G.random_shapes(seed=40 + tpt, width=160, height=120, n_shapes=30)
    frame = S.serialize_flat(flat, L.make_spec(tile, tpt, 4096, 127, 8))
    assert_parity(render(frame), O.render_frame(frame))


def test_glyph_page_small_all_substances():
    flat = G.glyph_page(seed=4, width=480, height=270, n_glyphs=150, n_shapes=25)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 511, 8))
    assert len(frame.radials) > 0 and len(frame.picture_uses) > 0
    assert_parity(render(frame), O.render_frame(frame))


def test_many_shapes_wide_stack():
    """More shapes per column than one 64-bit stack word (max_shape 1023)."""
    flat = G.random_shapes(seed=77, width=96, height=80, n_shapes=300, seg_lo=4, seg_hi=10)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 8192, 1023, 16))
    assert_parity(render(frame), O.render_frame(frame))


def test_fallback_pass_matches(monkeypatch):
    """Columns overflowing the small working capacity are re-run at full capacity."""
    monkeypatch.setenv("GUDNI_WORKING_CAPACITY", "8")
    frame = F.build("random_128x96")
    got = render(frame)
    want = np.load(os.path.join(GOLDEN, INDEX["random_128x96"]["image_file"]))
    assert np.array_equal(got, want)


def test_threshold_overflow_is_an_error():
    frame = F.build("random_128x96")
    frame.spec = L.make_spec(32, 32, 16, 127, 8)  # capacity far below the ~230 needed
    with Rasterizer(frame.spec) as r:
        with pytest.raises(RasterError) as e:
            r.queue_jobs(frame)
        assert e.value.code == -2
        # the context stays usable
        frame2 = F.build("tiny_square")
        frame2.spec = frame.spec
        r.queue_jobs(frame2)


def test_corrupt_strand_is_bad_input_not_a_fault():
    frame = F.build("knob")
    frame.geometry = frame.geometry.copy()
    frame.geometry[0:2] = np.frombuffer(np.uint16(7).tobytes(), np.uint8)  # odd strand size
    with Rasterizer(frame.spec) as r:
        with pytest.raises(RasterError) as e:
            r.queue_jobs(frame)
        assert e.value.code == -1
        good = F.build("knob")
        assert np.array_equal(r.queue_jobs(good), np.load(os.path.join(GOLDEN, "knob.npy")))


def test_shape_pointing_past_geometry_is_bad_input():
    frame = F.build("hourglass")
    frame.jobs[0].shapes = frame.jobs[0].shapes.copy()
    frame.jobs[0].shapes["geo_start"] = 1 << 20
    with Rasterizer(frame.spec) as r:
        with pytest.raises(RasterError) as e:
            r.queue_jobs(frame)
        assert e.value.code == -1


def test_empty_scene_is_background():
    frame = S.serialize(S.Scene((0.2, 0.4, 0.6, 1.0), S.EMPTY), 37, 23, L.make_spec(16, 16, 64))
    got = render(frame)
    assert np.array_equal(got, O.render_frame(frame))
    b, g, r = got[0, 0] & 0xFF, (got[0, 0] >> 8) & 0xFF, (got[0, 0] >> 16) & 0xFF
    assert (r, g, b) == (51, 102, 153)


@pytest.mark.parametrize("n_shapes,max_shape", [(64, 127), (65, 127), (31, 31), (32, 31)])
def test_shape_numbers_as_bits_at_the_limits(n_shapes, max_shape):
    """One 32x32 tile of canvas-wide shapes at the limits of the per-column kernel's
    shape numbering (a tile of at most 64 shapes and no more than max_shape numbers its
    shapes' bits by their place in the tile; 65 shapes, or more than max_shape, take the
    per-column bit index): the oracle's image, bit for bit."""
    flat = G.random_shapes(seed=100 + n_shapes, width=32, height=32, n_shapes=n_shapes, seg_lo=4, seg_hi=8)
    sections = 1 if max_shape < 64 else 2
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, max_shape, sections, max_strands_per_tile=1 << 24))
    assert np.concatenate([j.tiles for j in frame.jobs])["shape_length"].max() == n_shapes
    assert np.array_equal(render(frame), O.render_frame(frame))


def test_one_pixel_canvas():
    frame = F.build("tiny_square")
    tiny = S.serialize(F.tiny_square(), 1, 1, frame.spec)
    assert np.array_equal(render(tiny), O.render_frame(tiny))


def test_device_pointer_path():
    import torch
    frame = F.build("random_odd_tiles")
    want = np.load(os.path.join(GOLDEN, "random_odd_tiles.npy"))
    dev = torch.device("cuda:0")
    out = torch.zeros(frame.canvas_h * frame.canvas_w, dtype=torch.int32, device=dev)
    with Rasterizer(frame.spec) as r:
        r.upload_common(frame)
        keep = []
        for j, job in enumerate(frame.jobs):
            sh = torch.from_numpy(job.shapes.view(np.uint8).copy()).to(dev)
            ti = torch.from_numpy(job.tiles.view(np.uint8).copy()).to(dev)
            keep += [sh, ti]
            r.raster_job_device(frame, j, sh.data_ptr(), ti.data_ptr(), out.data_ptr(),
                                stream=L.current_stream_handle())
        r.sync_status()
        torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32).reshape(frame.canvas_h, frame.canvas_w)
    assert np.array_equal(got, want)


def _poly(points, color):
    o = S.segments_to_outline([S.straight(x, y) for x, y in points])
    return S.solid(color, S.shape([o]))


def test_shapes_far_above_and_below_the_columns():
    """Shapes whose strands lie wholly above or below most columns (the generation's
    y culling and its enclosure-only path): a tall canvas-spanning diamond and a
    rectangle reaching far past the canvas, over and under smaller shapes."""
    items = [
        _poly([(-50, -4000), (130, 60), (-50, 4000), (-60, 60)], (0.9, 0.2, 0.1, 0.7)),
        _poly([(20, -9000), (100, -9000), (100, 9000), (20, 9000)], (0.1, 0.6, 0.3, 0.6)),
        _poly([(10, 10), (40, 12), (30, 50)], (0.2, 0.2, 0.9, 1.0)),
        _poly([(60, 90), (110, 70), (90, 110)], (0.8, 0.8, 0.1, 0.5)),
    ]
    scene = S.Scene((1, 1, 1, 1), S.overlap(items))
    for tile, tpt in ((32, 32), (16, 64), (8, 32)):
        frame = S.serialize(scene, 128, 120, L.make_spec(tile, tpt, 4096, 127, 8))
        assert_parity(render(frame), O.render_frame(frame))


def test_non_finite_control_points_match_the_oracle():
    """NaN and +inf coordinates reach the kernels' comparisons (the culling and the
    batched insertion fall back to the literal path there); the image must still
    match the oracle's.  (A -inf x makes the reference's unbounded de Casteljau loop,
    Kernels.cl:1233-1258, run forever; the kernels stop after 96 halvings and report
    GUDNI_ERR_ITER_LIMIT, so there is no image to compare.)"""
    flat = G.random_shapes(seed=77, width=96, height=80, n_shapes=10)
    flat.pairs = flat.pairs.copy()
    flat.pairs[3, 1] = np.nan
    flat.pairs[17, 2] = np.inf
    frame = S.serialize_flat(flat, L.make_spec(16, 32, 4096, 127, 8))
    assert_parity(render(frame), O.render_frame(frame))


@pytest.mark.parametrize("tile,tpt", [(32, 32), (8, 64)])
def test_dense_canvas_wide_shapes(tile, tpt):
    """220 canvas-wide shapes on 160x120 (the batched mix's generator at its dense
    end): hundreds of thresholds and shape bits per column, so the multi-word stack,
    the batched and merged insertion of split parts and the opaque-cut memo all run."""
    flat = G.random_shapes(seed=91, width=160, height=120, n_shapes=220)
    frame = S.serialize_flat(flat, L.make_spec(tile, tpt, 4096, 255, 4, max_strands_per_tile=1 << 24))
    got = render(frame)
    want = O.render_frame(frame)
    assert_parity(got, want)
    assert np.array_equal(got, want)


def test_resident_pictures_across_frames():
    """A picture pile uploaded once (gudni_upload_pictures) and frames that upload only
    their own piles (gudni_upload_frame): two frames with different usages of one
    texture render exactly as through gudni_upload_common, and within the parity bar of
    the oracle.  A pile too small for the uploaded frame's usages makes the frame stale
    (not ready) and is refused for a new frame (bad input)."""
    import dataclasses
    spec = L.make_spec(32, 32, 4096, 511, 8)
    first = G.glyph_page(seed=4, width=320, height=180, n_glyphs=80, n_shapes=12, texture_frac=0.5)
    xf = first.substance_picture_xform.copy()
    xf[:, 0] += np.float32(13.0)
    xf[:, 1] -= np.float32(7.0)
    xf[:, 2] *= np.float32(1.5)
    second = dataclasses.replace(first, substance_picture_xform=xf)
    lib = S.PictureLibrary({1: G.noise_texture(seed=10, size=64), 0: first.pictures.reshape(1024, 1024, 4)})
    images = []
    with Rasterizer(spec) as r:
        r.upload_pictures(lib)
        r.upload_random_field(S.default_random_field())
        for flat in (first, second):
            frame = S.serialize_flat(lib.bind(flat), spec)
            assert len(frame.picture_uses) > 0
            r.upload_frame(frame)
            got = r.raster_frame(frame, upload_common=False)
            assert np.array_equal(got, render(S.serialize_flat(flat, spec)))
            assert_parity(got, O.render_frame(dataclasses.replace(frame, pictures=lib.pile)))
            images.append(got)
        assert not np.array_equal(images[0], images[1])
        r.upload_pictures(lib.pile[:16])
        with pytest.raises(RasterError) as err:
            r.raster_frame(frame, upload_common=False)
        assert err.value.code == -6
        with pytest.raises(RasterError) as err:
            r.upload_frame(frame)
        assert err.value.code == -1
        r.upload_pictures(lib)
        r.upload_frame(frame)
        r.upload_pictures(lib)  # the frame's usages still fit: it stays uploaded
        assert np.array_equal(r.raster_frame(frame, upload_common=False), images[1])


@pytest.mark.parametrize("source", [0, 1])
def test_stochastic_jitter_sources(source):
    """A non-zero STOCHASTIC_FACTOR with the reference's random field (source 0) and
    with the counter-based jitter (source 1, gudni_set_random_source): the image
    matches the oracle's bit for bit and differs from the unjittered one."""
    flat = G.glyph_page(seed=8, width=200, height=150, n_glyphs=50, n_shapes=12)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 127, 8, stochastic_factor=0.37))
    plain = O.render_frame(S.serialize_flat(flat, L.make_spec(32, 32, 4096, 127, 8)))
    seed = 987654321
    with Rasterizer(frame.spec) as r:
        r.set_random_source(source, seed)
        got = r.queue_jobs(frame)
    want = O.render_frame(frame, random_source=source, random_seed=seed)
    assert not np.array_equal(want, plain)
    assert np.array_equal(got, want), f"{int((got != want).sum())} pixels differ"


def test_device_strand_table():
    """The strand table built on the device from the uploaded pile
    (gudni_set_device_strand_table) renders the same images as the host-built one,
    and a pile damaged in the middle gives the same result either way."""
    flat = G.glyph_page(seed=4, width=480, height=270, n_glyphs=150, n_shapes=25)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 511, 8))

    def both(fr):
        outs = []
        for on in (False, True):
            with Rasterizer(fr.spec) as r:
                r.set_device_strand_table(on)
                try:
                    outs.append(("image", r.queue_jobs(fr), r.raster_frame(fr)))
                except RasterError as e:
                    outs.append(("error", e.code, None))
        return outs

    (k0, a0, b0), (k1, a1, b1) = both(frame)
    assert k0 == k1 == "image"
    assert np.array_equal(a0, a1) and np.array_equal(b0, b1) and np.array_equal(a0, b0)
    import dataclasses
    geo = frame.geometry.copy()
    at = (geo.size // 2) // 16 * 16
    geo[at:at + 2] = np.frombuffer(np.uint16(7).tobytes(), np.uint8)  # an odd size mid-pile
    (k0, a0, b0), (k1, a1, b1) = both(dataclasses.replace(frame, geometry=geo))
    assert k0 == k1
    if k0 == "image":
        assert np.array_equal(a0, a1) and np.array_equal(b0, b1)
    else:
        assert a0 == a1


def test_non_finite_coordinates_follow_the_oracle():
    """Single infinite control-point coordinates (a NaN sort key; a strand above the
    column with NaN intercepts) and finite ones near float max (an intercept that
    overflows): the kernels' image is the oracle's."""
    sys.path.insert(0, HERE)
    from test_host_column import _extreme, non_finite_cases
    near_max = S.serialize_flat(_extreme(16, 8, 1, 6, [3.4e38, -3.4e38, 3.4e38]), L.make_spec(8, 8, 4096, 127, 2))
    for frame in non_finite_cases() + [near_max]:
        assert np.array_equal(render(frame), O.render_frame(frame))


DENSE_CASES = {
    # (width, height, shapes, seed, tile, threads per tile, max_shape, stack words)
    "dense_160x120": (160, 120, 220, 91, 32, 32, 255, 4),
    "dense_96x64_onepixel": (96, 64, 400, 7, 8, 64, 511, 8),
    "dense_64x48_wide_stack": (64, 48, 600, 5, 8, 64, 1023, 16),
}


@pytest.mark.parametrize("dense_min", [32, 128])
@pytest.mark.parametrize("case", sorted(DENSE_CASES))
def test_dense_columns_by_a_warp(case, dense_min):
    """The warp-cooperative scan of dense columns (gudni_set_dense_columns): canvas-wide
    random shapes from the batched mix's generator, with hundreds of thresholds and
    shape bits per column and tens of thousands of sections per pixel, scanned by all
    32 lanes of a warp with real shuffles, ballots and __syncwarp; the image is the
    oracle's and the per-lane kernel's, bit for bit."""
    w, h, n, seed, tile, tpt, max_shape, sections = DENSE_CASES[case]
    flat = G.random_shapes(seed=seed, width=w, height=h, n_shapes=n)
    frame = S.serialize_flat(flat, L.make_spec(tile, tpt, 8192, max_shape, sections, max_strands_per_tile=1 << 24))
    with Rasterizer(frame.spec) as r:
        lane = r.queue_jobs(frame)
        r.set_dense_columns(dense_min)
        warp = r.queue_jobs(frame)
        again = r.raster_frame(frame)
    want = O.render_frame(frame)
    assert np.array_equal(lane, want), f"per-lane: {int((lane != want).sum())} pixels differ"
    assert np.array_equal(warp, want), f"warp: {int((warp != want).sum())} pixels differ"
    assert np.array_equal(again, want)


def test_dense_columns_on_the_512_golden():
    """The 512x512 64-shape workload through the warp-cooperative scan matches the
    image the reference kernels rendered (its digest in the golden index)."""
    frame = F.build("random_512_cfg")
    with Rasterizer(frame.spec) as r:
        r.set_dense_columns(32)
        got = r.queue_jobs(frame)
    import hashlib
    digest = hashlib.sha256(np.ascontiguousarray(got).tobytes()).hexdigest()
    assert digest == INDEX["random_512_cfg"]["image_sha256"]


COOP_CASES = {
    # name: (builder, spec)
    "glyph_page_32x32": (lambda: G.glyph_page(seed=4, width=480, height=270, n_glyphs=150, n_shapes=25),
                         dict(max_tile_size=32, threads_per_tile=32, max_thresholds=4096, max_shape=127,
                              stack_sections=8)),
    "split_leaves": (lambda: G.glyph_page(seed=7, width=200, height=120, n_glyphs=90, n_shapes=10),
                     dict(max_tile_size=32, threads_per_tile=32, max_thresholds=4096, max_shape=127,
                          stack_sections=8, max_strands_per_tile=60)),
    "random_16x64": (lambda: G.random_shapes(seed=5, width=150, height=110, n_shapes=30),
                     dict(max_tile_size=16, threads_per_tile=64, max_thresholds=4096, max_shape=127,
                          stack_sections=8)),
    "random_32x256": (lambda: G.random_shapes(seed=6, width=160, height=96, n_shapes=40),
                      dict(max_tile_size=32, threads_per_tile=256, max_thresholds=4096, max_shape=127,
                           stack_sections=8)),
    "dense_one_word": (lambda: G.random_shapes(seed=13, width=96, height=80, n_shapes=60),
                       dict(max_tile_size=32, threads_per_tile=32, max_thresholds=4096, max_shape=127,
                            stack_sections=8)),
    "beyond_64_shapes": (lambda: G.random_shapes(seed=9, width=96, height=64, n_shapes=90, seg_lo=4, seg_hi=8),
                         dict(max_tile_size=32, threads_per_tile=32, max_thresholds=8192, max_shape=255,
                              stack_sections=4)),
}


@pytest.mark.parametrize("case", sorted(COOP_CASES))
def test_cooperative_units_match_per_column_generation(case):
    """The warp-cooperative units (gudni_set_cooperative_units, the default): strands
    and (strand, column) pairs dealt to the lanes, thresholds binned by ballots and
    match masks, shape records staged by a bulk copy, pixels stored by rows from a
    shared tile.  The image is the per-column kernel's and the oracle's bit for bit,
    through the frame entry point and through a job at a time, twice in a row on one
    context (the shared tile and the barrier phase carry over)."""
    build, spec = COOP_CASES[case]
    frame = S.serialize_flat(build(), L.make_spec(**spec))
    want = O.render_frame(frame)
    with Rasterizer(frame.spec) as r:
        r.set_cooperative_units(False)
        per_column = r.raster_frame(frame)
        r.set_cooperative_units(True)
        coop = [r.raster_frame(frame), r.queue_jobs(frame), r.raster_frame(frame)]
    assert np.array_equal(per_column, want), f"per-column: {int((per_column != want).sum())} pixels differ"
    for got in coop:
        assert np.array_equal(got, want), f"cooperative: {int((got != want).sum())} pixels differ"


def test_cooperative_units_overflow_to_the_full_pass(monkeypatch):
    """A small working capacity sends long columns of cooperative units to the
    full-capacity pass; the image does not change."""
    monkeypatch.setenv("GUDNI_WORKING_CAPACITY", "24")
    frame = F.build("random_128x96")
    want = np.load(os.path.join(GOLDEN, INDEX["random_128x96"]["image_file"]))
    with Rasterizer(frame.spec) as r:
        assert np.array_equal(r.raster_frame(frame), want)


def test_cooperative_units_chosen_per_launch():
    """gudni_set_cooperative_units(ctx, -1): each launch picks the cooperative units
    or the per-column kernel by its number of work units; whichever it picks, the
    image is the per-column kernel's (job by job and as one frame launch)."""
    small = F.build("random_128x96")
    big = S.serialize_flat(G.random_shapes(seed=0, width=512, height=512, n_shapes=64),
                           L.make_spec(32, 256, 4096, 127, 8))
    for frame in (small, big):
        with Rasterizer(frame.spec) as r:
            want = r.raster_frame(frame)
            r.set_cooperative_units(None)
            assert np.array_equal(r.raster_frame(frame), want)
            assert np.array_equal(r.queue_jobs(frame), want)
