"""The product's device column machine, compiled for the host CPU
(tests/host_column), against the oracle: the exact-arithmetic transformations of the
CUDA path (strand-table range test and y culling, batched and merged insertion of
split parts, opaque-cut colour memo, one-word and multi-word stacks) checked without a
GPU, on sparse, dense and degenerate scenes; and the warp-cooperative scan of dense
columns (warp_column.cuh) on an emulated 32-lane warp (tests/host_column/warp_emu.h)."""
import ctypes as C
import dataclasses
import os
import shutil
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.skipif(shutil.which("g++") is None or not os.path.isdir("/usr/local/cuda/include"),
                                reason="needs g++ and the CUDA headers")


def host_render(frame, capacity=None) -> np.ndarray:
    from host_column.build import load
    lib = load()
    capacity = capacity or frame.spec.max_thresholds
    out = np.zeros((frame.canvas_h, frame.canvas_w), np.uint32)
    bg = np.ascontiguousarray(frame.background, np.float32)
    p = L.ptr
    for ji, job in enumerate(frame.jobs):
        ov = C.c_int(0)
        st = lib.host_column_raster_job(p(frame.geometry), frame.geometry.size, p(frame.substances),
                                        len(frame.substances), p(frame.pictures), frame.pictures.size,
                                        p(frame.picture_uses), len(frame.picture_uses), p(frame.radials),
                                        len(frame.radials), p(job.shapes), len(job.shapes), p(job.tiles),
                                        len(job.tiles), frame.compute_depth, frame.canvas_w, frame.canvas_h, ji,
                                        bg.ctypes.data, p(frame.random_field), frame.spec.stochastic_factor,
                                        capacity, frame.spec.max_shape,
                                        out.ctypes.data, C.byref(ov))
        assert st == 0 and ov.value == 0, (st, ov.value)
    return out


def check(frame):
    got, want = host_render(frame), O.render_frame(frame)
    assert np.array_equal(got, want), f"{int((got != want).sum())} of {got.size} pixels differ"


@pytest.mark.parametrize("tile,tpt", [(32, 32), (16, 64), (8, 32)])
def test_random_scene(tile, tpt):
    check(S.serialize_flat(G.random_shapes(seed=5, width=160, height=120, n_shapes=40),
                           L.make_spec(tile, tpt, 4096, 127, 8)))


@pytest.mark.parametrize("tile,tpt", [(32, 32), (8, 64)])
def test_dense_canvas_wide_shapes(tile, tpt):
    """Hundreds of thresholds and shape bits per column: multi-word stack, batched and
    merged insertion of split parts."""
    flat = G.random_shapes(seed=91, width=160, height=120, n_shapes=220)
    check(S.serialize_flat(flat, L.make_spec(tile, tpt, 4096, 255, 4, max_strands_per_tile=1 << 24)))


@pytest.mark.parametrize("n_shapes,max_shape", [(64, 127), (65, 127), (31, 31), (32, 31), (40, 63)])
def test_shape_numbers_as_bits_at_the_limits(n_shapes, max_shape):
    """One 32x32 tile of canvas-wide shapes at the limits of the per-column kernel's
    shape numbering: a tile of at most 64 shapes and no more than max_shape numbers its
    shapes' bits by their place in the tile (64 shapes: bit 63 in use), one more shape
    (65), or a tile above max_shape (32 shapes, max_shape 31: the reference drops the
    shapes past max_shape bits), takes the per-column bit index; the image is the
    oracle's either way."""
    flat = G.random_shapes(seed=100 + n_shapes, width=32, height=32, n_shapes=n_shapes, seg_lo=4, seg_hi=8)
    sections = 1 if max_shape < 64 else 2
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, max_shape, sections, max_strands_per_tile=1 << 24))
    tiles = np.concatenate([j.tiles for j in frame.jobs])
    assert tiles["shape_length"].max() == n_shapes
    check(frame)


def test_very_dense_small_canvas():
    """The batched mix's densest corner: a small canvas crossed by many shapes."""
    flat = G.random_shapes(seed=9, width=48, height=40, n_shapes=300, seg_lo=8, seg_hi=32)
    check(S.serialize_flat(flat, L.make_spec(8, 64, 8192, 511, 8, max_strands_per_tile=1 << 24)))


def test_glyph_page_all_substances():
    flat = G.glyph_page(seed=4, width=480, height=270, n_glyphs=150, n_shapes=25)
    check(S.serialize_flat(flat, L.make_spec(32, 32, 4096, 511, 8)))


@pytest.mark.parametrize("factor", [0.25, 0.37])
def test_stochastic_jitter(factor):
    """A non-zero STOCHASTIC_FACTOR: the area jitter reads the random field from the
    same per-column cursor, advanced once per section (K:1597-1613)."""
    spec = L.make_spec(32, 32, 4096, 127, 8, stochastic_factor=factor)
    frame = S.serialize_flat(G.glyph_page(seed=8, width=200, height=150, n_glyphs=50, n_shapes=12), spec)
    assert np.any(frame.random_field != 0)
    plain = O.render_frame(S.serialize_flat(G.glyph_page(seed=8, width=200, height=150, n_glyphs=50, n_shapes=12),
                                            L.make_spec(32, 32, 4096, 127, 8)))
    got, want = host_render(frame), O.render_frame(frame)
    assert not np.array_equal(want, plain)  # the jitter changes the image
    assert np.array_equal(got, want), f"{int((got != want).sum())} of {got.size} pixels differ"


@pytest.mark.parametrize("seed,tile,tpt,max_shape", [(12345, 32, 32, 127), (2 ** 63 + 7, 16, 64, 511)])
def test_counter_jitter(seed, tile, tpt, max_shape):
    """The counter-based jitter source (GUDNI_RANDOM_COUNTER, the scan instantiated
    with kCounterJitter) matches the oracle bit for bit, one-word and multi-word
    stacks; the image differs from the random field's and from another seed's."""
    from host_column.build import load
    lib = load()
    spec = L.make_spec(tile, tpt, 4096, max_shape, 8, stochastic_factor=0.37)
    frame = S.serialize_flat(G.glyph_page(seed=8, width=200, height=150, n_glyphs=50, n_shapes=12), spec)
    field = O.render_frame(frame)
    want = O.render_frame(frame, random_source=1, random_seed=seed)
    other = O.render_frame(frame, random_source=1, random_seed=seed + 1)
    assert not np.array_equal(want, field) and not np.array_equal(want, other)
    lib.host_set_random_source(1, seed)
    try:
        got = host_render(frame)
    finally:
        lib.host_set_random_source(0, 0)
    assert np.array_equal(got, want), f"{int((got != want).sum())} of {got.size} pixels differ"
    assert np.array_equal(host_render(frame), field)  # the field source again


def test_non_finite_points():
    flat = G.random_shapes(seed=77, width=96, height=80, n_shapes=10)
    flat.pairs = flat.pairs.copy()
    flat.pairs[3, 1] = np.nan
    flat.pairs[17, 2] = np.inf
    check(S.serialize_flat(flat, L.make_spec(16, 32, 4096, 127, 8)))


def host_adjoint(frame, target, capacity=1024, regenerate=False):
    from host_column.build import load
    lib = load()
    lib.host_column_set_adjoint_regenerate(1 if regenerate else 0)
    img = np.zeros((frame.canvas_h, frame.canvas_w, 4), np.float32)
    gg = np.zeros(frame.geometry.size // 4, np.float32)
    gs = np.zeros((len(frame.substances), 4), np.float32)
    tgt = np.ascontiguousarray(target, np.float32)
    bg = np.ascontiguousarray(frame.background, np.float32)
    p = L.ptr
    for ji, job in enumerate(frame.jobs):
        ov = C.c_int(0)
        st = lib.host_column_adjoint_job(p(frame.geometry), frame.geometry.size, p(frame.substances),
                                         len(frame.substances), p(frame.pictures), frame.pictures.size,
                                         p(frame.picture_uses), len(frame.picture_uses), p(frame.radials),
                                         len(frame.radials), p(job.shapes), len(job.shapes), p(job.tiles),
                                         len(job.tiles), frame.compute_depth, frame.canvas_w, frame.canvas_h, ji,
                                         bg.ctypes.data, capacity, frame.spec.max_shape, tgt.ctypes.data,
                                         img.ctypes.data, gg.ctypes.data, gs.ctypes.data, C.byref(ov))
        assert st == 0 and ov.value == 0, (st, ov.value)
    return img, gg, gs


def _rel(got, want):
    got, want = np.asarray(got, np.float64).ravel(), np.asarray(want, np.float64).ravel()
    big = np.abs(want) > 0.01 * np.abs(want).max()
    return (float(np.linalg.norm(got - want) / np.linalg.norm(want)),
            float(np.max(np.abs(got[big] - want[big]) / np.abs(want[big]))))


@pytest.mark.parametrize("name", ["random", "dense", "glyphs"])
def test_adjoint_column_code_matches_fp64_reference(name):
    """The adjoint's per-column device code (adjoint_device.cuh) on the host: float image
    equal to the FP64 reference's forward, gradients within 1e-3 of it."""
    rng = np.random.default_rng(1)
    if name == "random":
        make = lambda: G.random_shapes(seed=9, width=160, height=120, n_shapes=24)  # noqa: E731
        spec = L.make_spec(32, 32, 4096, 127, 8)
    elif name == "dense":
        make = lambda: G.random_shapes(seed=91, width=96, height=80, n_shapes=120)  # noqa: E731
        spec = L.make_spec(16, 64, 4096, 255, 4, max_strands_per_tile=1 << 24)
    else:
        make = lambda: G.glyph_page(seed=3, width=256, height=192, n_glyphs=60, n_shapes=30)  # noqa: E731
        spec = L.make_spec(32, 32, 4096, 127, 8)
    frame = S.serialize_flat(make(), spec)
    t = make()
    t.pairs = (t.pairs + rng.normal(0, 2.0, t.pairs.shape)).astype(np.float32)
    target = O.render_float(S.serialize_flat(t, spec))
    _, g_geo, g_sub, img_ref = O.loss_and_gradient(frame, target)
    img, gg, gs = host_adjoint(frame, target)
    np.testing.assert_allclose(img, img_ref, rtol=1e-6, atol=1e-6)
    for got, want, what in ((gg, g_geo, "geometry"), (gs, g_sub, "substances")):
        norm, worst = _rel(got, want)
        assert norm <= 1e-3 and worst <= 1e-3, (what, norm, worst)


@pytest.mark.parametrize("name", ["random", "dense", "glyphs"])
def test_adjoint_generated_once_equals_regenerated(name):
    """The adjoint's two modes on the host: thresholds generated once with provenance
    (the forward scanning a copy of the sorted queue) and the raster generation for the
    forward with a second generation for the gradients give the same float image and
    the same gradients, bit for bit -- generateP and buildThresholds make the same
    queue."""
    if name == "random":
        flat, spec = G.random_shapes(seed=21, width=150, height=110, n_shapes=30), L.make_spec(32, 32, 4096, 127, 8)
    elif name == "dense":
        flat = G.random_shapes(seed=92, width=96, height=80, n_shapes=120)
        spec = L.make_spec(16, 64, 4096, 255, 4, max_strands_per_tile=1 << 24)
    else:
        flat = G.glyph_page(seed=4, width=256, height=192, n_glyphs=60, n_shapes=30)
        spec = L.make_spec(32, 128, 4096, 127, 8)
    frame = S.serialize_flat(flat, spec)
    target = np.random.default_rng(2).random((frame.canvas_h, frame.canvas_w, 4)).astype(np.float32)
    once = host_adjoint(frame, target, capacity=4096)
    twice = host_adjoint(frame, target, capacity=4096, regenerate=True)
    for a, b in zip(once, twice):
        np.testing.assert_array_equal(a, b)


def test_adjoint_column_code_generated_scenes():
    """Generated scenes, tile shapes and targets through the adjoint's column code: the
    float image equals the FP64 reference's forward within 1e-6, and the gradients
    agree with its gradients to a relative norm of 1e-3 and, element by element (those
    above 1 % of the largest), to 1e-2; zero where the reference's are zero.  (Over 400
    such scenes the worst seen were 7e-5 and 2.7e-3.)"""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=40, deadline=None, derandomize=True)
    @hyp.given(seed=st.integers(0, 10 ** 6), w=st.integers(1, 96), h=st.integers(1, 80), n=st.integers(1, 40),
               tile=st.sampled_from([8, 16, 32]), tpt_mul=st.sampled_from([1, 2, 4]), glyph=st.booleans(),
               sigma=st.sampled_from([0.5, 2.0]))
    def run(seed, w, h, n, tile, tpt_mul, glyph, sigma):
        def make():
            if glyph:
                return G.glyph_page(seed=seed, width=max(w, 40), height=max(h, 30), n_glyphs=max(n // 2, 1),
                                    n_shapes=max(n // 4, 1))
            return G.random_shapes(seed=seed, width=w, height=h, n_shapes=n)
        spec = L.make_spec(tile, tile * tpt_mul, 4096, 127, 8)
        frame = S.serialize_flat(make(), spec)
        t = make()
        t.pairs = (t.pairs + np.random.default_rng(seed).normal(0, sigma, t.pairs.shape)).astype(np.float32)
        target = O.render_float(S.serialize_flat(t, spec))
        _, g_geo, g_sub, img_ref = O.loss_and_gradient(frame, target)
        img, gg, gs = host_adjoint(frame, target, capacity=4096)
        np.testing.assert_allclose(img, img_ref, rtol=1e-6, atol=1e-6)
        for got, want, what in ((gg, g_geo, "geometry"), (gs, g_sub, "substances")):
            if not np.any(want):
                assert not np.any(got), what
                continue
            norm, worst = _rel(got, want)
            assert norm <= 1e-3 and worst <= 1e-2, (what, norm, worst)

    run()


def test_strand_table_threads_give_the_same_table():
    """The C ABI builds the strand table's y ranges on several host threads; the table
    is the one-thread table, entry for entry."""
    from host_column.build import load
    lib = load()
    flat = G.glyph_page(seed=2, width=960, height=540, n_glyphs=600, n_shapes=200)
    geo = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 127, 8)).geometry
    outs = []
    for threads in (1, 4, 16):
        cap = geo.size // 16
        table = np.zeros((cap, 4), np.uint32)
        ys = np.zeros((cap, 2), np.float32)
        first = np.zeros(geo.size // 16, np.uint32)
        n = lib.host_strand_table(geo.ctypes.data, geo.size, threads, table.ctypes.data, ys.ctypes.data,
                                  first.ctypes.data, cap)
        assert n >= 2 * 16384  # large enough for the threads to split it
        outs.append((table[:n].tobytes(), ys[:n].tobytes(), first.tobytes()))
    assert outs[0] == outs[1] == outs[2]


@pytest.mark.parametrize("extra", [1, 3])
def test_nearly_full_queues(extra):
    """Slabs only just large enough for the longest column: the merge sort and the
    batched insertion lack free space below the queue and take their literal paths;
    the image must not change."""
    flat = G.random_shapes(seed=301, width=96, height=80, n_shapes=150)
    frame = S.serialize_flat(flat, L.make_spec(8, 64, 8192, 255, 4, max_strands_per_tile=1 << 24))
    st = {}
    want = O.render_frame(frame, stats=st)
    assert np.array_equal(host_render(frame, st["max_queue"] + extra), want)


# ------------------------------------------------------------------ warp-cooperative scan
def host_render_warp(frame, dense_min=0, seed=1, capacity=None):
    """The warp-cooperative fast pass (warp_column.cuh) on an emulated warp; columns
    that overflow `capacity` are re-run at max_thresholds by the per-lane path, as the
    full-capacity pass does.  Returns the image and the number of columns the whole
    warp scanned."""
    from host_column.build import load
    lib = load()
    cap = capacity or frame.spec.max_thresholds
    out = np.zeros((frame.canvas_h, frame.canvas_w), np.uint32)
    bg = np.ascontiguousarray(frame.background, np.float32)
    p = L.ptr
    by_warp = 0
    for ji, job in enumerate(frame.jobs):
        ov, bw = C.c_int(0), C.c_int(0)
        st = lib.host_column_raster_job_warp(p(frame.geometry), frame.geometry.size, p(frame.substances),
                                             len(frame.substances), p(frame.pictures), frame.pictures.size,
                                             p(frame.picture_uses), len(frame.picture_uses), p(frame.radials),
                                             len(frame.radials), p(job.shapes), len(job.shapes), p(job.tiles),
                                             len(job.tiles), frame.compute_depth, frame.canvas_w, frame.canvas_h,
                                             ji, bg.ctypes.data, p(frame.random_field),
                                             frame.spec.stochastic_factor, cap, frame.spec.max_thresholds,
                                             frame.spec.max_shape, dense_min, seed, out.ctypes.data, C.byref(ov),
                                             C.byref(bw))
        assert st == 0 and ov.value == 0, (st, ov.value)
        by_warp += bw.value
    return out, by_warp


def warp_trace():
    """Counts of the warp band step's paths since the last call: split across the
    lanes, split on lane 0, parts sorted by rounds, parts sorted on lane 0, equal
    keys reordered."""
    from host_column.build import load
    t = (C.c_longlong * 5)()
    load().host_warp_trace(t)
    return {"split_warp": t[0], "split_lane0": t[1], "sort_rounds": t[2], "sort_lane0": t[3], "ties": t[4]}


def check_warp(frame, min_by_warp, **kw):
    warp_trace()
    got, by_warp = host_render_warp(frame, **kw)
    trace = warp_trace()
    want = O.render_frame(frame)
    assert by_warp >= min_by_warp
    assert np.array_equal(got, want), f"{int((got != want).sum())} of {got.size} pixels differ"
    return trace


@pytest.mark.parametrize("seed", [1, 2])
def test_warp_scan_random_scene(seed):
    """Every column scanned by the whole warp; the lanes resume in a different order
    at each barrier (seeded), so a read of another lane's write without a barrier
    between would change pixels."""
    frame = S.serialize_flat(G.random_shapes(seed=5, width=64, height=48, n_shapes=12),
                             L.make_spec(32, 32, 4096, 127, 8))
    trace = check_warp(frame, 128, dense_min=0, seed=seed)
    assert trace["split_warp"] > 0


def test_warp_scan_dense_multiword_stack():
    """Canvas-wide shapes: bands of dozens of sections (several chunks of 32), a
    multi-word stack, the band step's splits, sorts and merges across the lanes."""
    frame = S.serialize_flat(G.random_shapes(seed=91, width=40, height=30, n_shapes=120),
                             L.make_spec(8, 64, 4096, 255, 4, max_strands_per_tile=1 << 24))
    trace = check_warp(frame, 1000, dense_min=0, seed=3)
    assert trace["split_warp"] > 10000 and trace["sort_rounds"] > 10000 and trace["sort_lane0"] > 0


def test_warp_scan_equal_keys():
    """Every outline drawn twice (two colours): split parts with equal keys, which the
    per-lane order puts latest first."""
    rng = G._rng(44)
    specs = []
    for sp in G.random_shape_specs(rng, 48, 40, 30, 8, 20):
        twin = dataclasses.replace(sp, leaves=[[a.copy() for a in leaf] for leaf in sp.leaves],
                                   color=(1.0 - sp.color[0], sp.color[1], 1.0 - sp.color[2], sp.color[3]))
        specs += [sp, twin]
    frame = S.serialize_flat(G.flat_from_specs(specs, 48, 40, G.WHITE),
                             L.make_spec(8, 64, 8192, 255, 4, max_strands_per_tile=1 << 24))
    trace = check_warp(frame, 1000, dense_min=0, seed=9)
    assert trace["ties"] > 0


def test_warp_scan_all_substances_and_jitter():
    """Pictures and gradients (colours that depend on the pixel row) and a non-zero
    stochastic factor (one random-field step per section)."""
    frame = S.serialize_flat(G.glyph_page(seed=4, width=160, height=96, n_glyphs=40, n_shapes=10),
                             L.make_spec(32, 32, 4096, 511, 8))
    check_warp(frame, 400, dense_min=0, seed=4)
    frame = S.serialize_flat(G.glyph_page(seed=8, width=100, height=64, n_glyphs=30, n_shapes=8),
                             L.make_spec(32, 32, 4096, 127, 8, stochastic_factor=0.37))
    check_warp(frame, 150, dense_min=0, seed=5)


def test_warp_scan_capacity_and_mixed_columns():
    """Slabs only just large enough (the band step falls back to lane 0 where the
    queue has no room below it), a working capacity below the longest queue (those
    columns go to the full-capacity pass), and a threshold that leaves short queues on
    their lanes."""
    frame = S.serialize_flat(G.random_shapes(seed=301, width=40, height=32, n_shapes=80),
                             L.make_spec(8, 64, 8192, 255, 4, max_strands_per_tile=1 << 24))
    st = {}
    O.render_frame(frame, stats=st)
    trace = check_warp(frame, 1000, dense_min=0, seed=6, capacity=st["max_queue"] + 2)
    assert trace["split_lane0"] > 0
    check_warp(frame, 1000, dense_min=0, seed=7, capacity=st["max_queue"] // 2)
    got, by_warp = host_render_warp(frame, dense_min=st["max_queue"] // 2, seed=8)
    assert 0 < by_warp < 1280
    assert np.array_equal(got, O.render_frame(frame))


def test_warp_scan_generated_scenes():
    """Generated dense scenes (canvas, shape count and sizes, tile shape, stack words,
    the lanes' resume order) through the warp-cooperative scan: bit for bit the
    oracle's image every time."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=12, deadline=None, derandomize=True)
    @hyp.given(seed=st.integers(0, 10 ** 6), w=st.integers(8, 48), h=st.integers(8, 40),
               n=st.integers(4, 90), seg_hi=st.integers(3, 16), tile=st.sampled_from([8, 16, 32]),
               tpt_mul=st.sampled_from([1, 2, 4]), wide=st.booleans(), lanes=st.integers(0, 10 ** 6))
    def run(seed, w, h, n, seg_hi, tile, tpt_mul, wide, lanes):
        flat = G.random_shapes(seed=seed, width=w, height=h, n_shapes=n, seg_lo=2, seg_hi=seg_hi)
        spec = L.make_spec(tile, tile * tpt_mul, 4096, 255 if wide else 127, 4 if wide else 2)
        frame = S.serialize_flat(flat, spec)
        got, _ = host_render_warp(frame, dense_min=0, seed=lanes)
        want = O.render_frame(frame)
        assert np.array_equal(got, want), f"{int((got != want).sum())} of {got.size} pixels differ"

    run()


def _poked(flat, seed, value):
    flat.pairs = flat.pairs.copy()
    k = np.random.default_rng(seed).integers(0, flat.pairs.size)
    flat.pairs.reshape(-1)[k] = value
    return flat


def non_finite_cases():
    """Scenes where a single infinite control-point coordinate once made the product
    differ from the reference kernels: +inf x on a 1x2 canvas (a NaN sort key, so the
    queue order depends on the sort algorithm) and -inf y in a glyph scene (a strand
    wholly above the column whose intercepts are NaN, so skipping them changed the
    enclosure)."""
    cases = []
    for seg_hi in (5, 7, 10):
        flat = G.random_shapes(seed=1558, width=1, height=2, n_shapes=29, seg_lo=2, seg_hi=seg_hi)
        cases.append(S.serialize_flat(_poked(flat, 1558, np.inf), L.make_spec(8, 8, 4096, 127, 2)))
    flat = G.glyph_page(seed=776117, width=40, height=30, n_glyphs=1, n_shapes=1)
    cases.append(S.serialize_flat(_poked(flat, 776117, -np.inf), L.make_spec(8, 8, 4096, 127, 2)))
    return cases


def test_non_finite_coordinates_follow_the_reference():
    for frame in non_finite_cases():
        check(frame)
        if O.ref_available(127, 2):
            assert np.array_equal(O.render_frame(frame), O.ref_render_frame(frame, 4096))


def _extreme(seed, w, h, n, values):
    """A random scene with three coordinates replaced by the given finite values."""
    flat = G.random_shapes(seed=seed, width=w, height=h, n_shapes=n, seg_lo=2, seg_hi=10)
    flat.pairs = flat.pairs.copy()
    where = np.random.default_rng(seed).integers(0, flat.pairs.size, size=len(values))
    for j, v in zip(where, values):
        flat.pairs.reshape(-1)[j] = np.float32(v)
    return flat


def test_huge_finite_coordinates_halve_to_the_end():
    """A curve spanning ~2^124 in x needs 102 halvings before it is flat; a halving cap
    of 96 once stopped it with the iteration-limit status where the reference renders."""
    frame = S.serialize_flat(_extreme(0, 1, 1, 1, [3e37, -3e37, 1e30]), L.make_spec(8, 8, 4096, 127, 2))
    check(frame)
    if O.ref_available(127, 2):
        assert np.array_equal(O.render_frame(frame), O.ref_render_frame(frame, 4096))


def test_coordinates_near_float_max_are_not_culled():
    """Finite coordinates near +-3.4e38: a curve difference overflows and its intercept
    is infinite although every point is finite; y culling of such a strand once changed
    two pixels of this 8x1 scene.  Strands and hulls with coordinates beyond 2^21 are no
    longer culled (per lane and by the warp)."""
    frame = S.serialize_flat(_extreme(16, 8, 1, 6, [3.4e38, -3.4e38, 3.4e38]), L.make_spec(8, 8, 4096, 127, 2))
    check(frame)
    got, _ = host_render_warp(frame, dense_min=0, seed=16)
    assert np.array_equal(got, O.render_frame(frame))
    if O.ref_available(127, 2):
        assert np.array_equal(O.render_frame(frame), O.ref_render_frame(frame, 4096))


def test_generated_extreme_finite_scenes():
    """Huge, tiny and subnormal coordinates: finite inputs never reach the halving cap
    and the column machine, per lane and by the warp, gives the oracle's image."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=20, deadline=None, derandomize=True)
    @hyp.given(seed=st.integers(0, 10 ** 6), w=st.integers(1, 40), h=st.integers(1, 30), n=st.integers(1, 40),
               tile=st.sampled_from([8, 16, 32]),
               values=st.sampled_from([(3e37, -3e37, 1e30), (1e-30, -1e-30, 1e-20), (1e-40, -1e-42, 1e-39),
                                       (3e37, 1e-40, -1e30), (3.4e38, -3.4e38, 3.4e38)]))
    def run(seed, w, h, n, tile, values):
        frame = S.serialize_flat(_extreme(seed, w, h, n, values), L.make_spec(tile, tile, 4096, 127, 2))
        check(frame)
        got, _ = host_render_warp(frame, dense_min=0, seed=seed)  # every column by the warp
        assert np.array_equal(got, O.render_frame(frame))

    run()


def test_generated_non_finite_scenes():
    """Generated scenes with one NaN or infinite coordinate, at several tile shapes,
    stack sizes and jitter sources: the product's column machine gives the oracle's
    image.  (Inputs on which the reference's curve halving never ends are skipped:
    there the kernels stop at their iteration cap and report it.)"""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    from host_column.build import load
    lib = load()

    @hyp.settings(max_examples=25, deadline=None, derandomize=True)
    @hyp.given(seed=st.integers(0, 10 ** 6), w=st.integers(1, 48), h=st.integers(1, 40), n=st.integers(1, 60),
               tile=st.sampled_from([8, 16, 32]), glyph=st.booleans(), counter=st.booleans(),
               value=st.sampled_from([np.nan, np.inf, -np.inf]))
    def run(seed, w, h, n, tile, glyph, counter, value):
        if glyph:
            flat = G.glyph_page(seed=seed, width=max(w, 40), height=max(h, 30), n_glyphs=max(n // 4, 1),
                                n_shapes=max(n // 8, 1))
        else:
            flat = G.random_shapes(seed=seed, width=w, height=h, n_shapes=n, seg_lo=2, seg_hi=12)
        frame = S.serialize_flat(_poked(flat, seed, value),
                                 L.make_spec(tile, tile, 4096, 127, 2, stochastic_factor=0.25 if counter else 0.0))
        lib.host_set_random_source(1 if counter else 0, seed)
        try:
            got = host_render(frame)
        except AssertionError as e:
            if "(2, 0)" in str(e):  # the iteration cap: the reference's halving would not end
                return
            raise
        finally:
            lib.host_set_random_source(0, 0)
        want = O.render_frame(frame, random_source=1 if counter else 0, random_seed=seed)
        assert np.array_equal(got, want), f"{int((got != want).sum())} of {got.size} pixels differ"

    run()
