"""The serializer's device passes (gudni_gb300/csrc/serialize_device.cuh) run on the
CPU (tests/host_serialize: plain loops in a seeded random item order, built with
AddressSanitizer and UBSan) against the host serializer (gudni_serialize): the
geometry pile, the strand table the raster kernels read, the substance, picture-use
and gradient piles, the concatenated shape and tile piles with every tile's job, and
the frame counters, byte for byte."""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import fixture_scenes as F  # noqa: E402
from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402

pytestmark = pytest.mark.skipif(shutil.which("g++") is None or not os.path.isdir("/usr/local/cuda/include"),
                                reason="needs g++ and the CUDA headers")


def _write(path, arrays):
    with open(path, "wb") as f:
        for name, a in arrays.items():
            b = np.ascontiguousarray(a).tobytes() if not isinstance(a, (bytes, bytearray)) else bytes(a)
            f.write(np.uint32(len(name)).tobytes() + name.encode() + np.uint64(len(b)).tobytes() + b)


def _read(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    at = 0
    while at < len(data):
        n = int(np.frombuffer(data, np.uint32, 1, at)[0])
        name = data[at + 4:at + 4 + n].decode()
        size = int(np.frombuffer(data, np.uint64, 1, at + 4 + n)[0])
        out[name] = data[at + 12 + n:at + 12 + n + size]
        at += 12 + n + size
    return out


def device_passes(flat, spec, seed=1, provenance=True):
    """The device serializer's output, computed by its passes on the CPU."""
    from host_serialize.build import build
    arrays = {
        "header": np.array([flat.canvas_w, flat.canvas_h, flat.substance_kind.size, flat.picture_offset.size],
                           np.int32),
        "spec": bytes(spec),
        "substance_kind": flat.substance_kind.astype(np.int32),
        "substance_color": flat.substance_color.astype(np.float32),
        "substance_picture": flat.substance_picture.astype(np.int32),
        "substance_picture_xform": flat.substance_picture_xform.astype(np.float32),
        "substance_radial": flat.substance_radial,
        "substance_shape_start": flat.substance_shape_start.astype(np.int32),
        "shape_compound": flat.shape_compound.astype(np.int32),
        "shape_outline_start": flat.shape_outline_start.astype(np.int32),
        "outline_pair_start": flat.outline_pair_start.astype(np.int32),
        "pairs": flat.pairs.astype(np.float32),
        "picture_size": flat.picture_size.astype(np.int32),
        "picture_offset": flat.picture_offset.astype(np.int32),
    }
    with tempfile.TemporaryDirectory() as d:
        src, dst = os.path.join(d, "scene.bin"), os.path.join(d, "out.bin")
        _write(src, arrays)
        r = subprocess.run([build(), src, dst, str(seed), "1" if provenance else "0"], capture_output=True, text=True,
                           env=dict(os.environ, ASAN_OPTIONS="detect_leaks=0"))
        assert r.returncode == 0, r.stderr[-4000:]
        return _read(dst)


def host_strand_table(geometry):
    from host_column.build import load
    lib = load()
    cap = max(1, geometry.size // 32)
    table = np.zeros((cap, 4), np.uint32)
    ys = np.zeros((cap, 2), np.float32)
    first = np.zeros(geometry.size // 16, np.uint32)
    n = lib.host_strand_table(geometry.ctypes.data, geometry.size, 1, table.ctypes.data, ys.ctypes.data,
                              first.ctypes.data, cap)
    return table[:n], ys[:n], first


def check(flat, spec, seeds=(1,)):
    frame = S.serialize_flat(flat, spec)
    shapes, tiles, jobs = S.concatenated_piles(frame)
    table, ys, first = host_strand_table(frame.geometry)
    for n, seed in enumerate(seeds + (seeds[-1] + 100,)):
        provenance = n < len(seeds)  # the last run without: the piles do not change
        got = device_passes(flat, spec, seed, provenance)
        if provenance:
            assert got["point_offsets"] == frame.point_offsets.astype(np.uint32).tobytes()
            assert got["point_sources"] == frame.point_sources.astype(np.int32).tobytes()
            assert got["point_weights"] == frame.point_weights.astype(np.float32).tobytes()
        else:
            assert "point_offsets" not in got
        assert "error" not in got, got.get("error")
        assert got["geometry"] == frame.geometry.tobytes()
        assert got["strand_table"] == table.tobytes()
        assert got["strand_y"] == ys.tobytes()
        assert got["strand_first"] == first.tobytes()
        assert got["substances"] == np.ascontiguousarray(frame.substances, np.float32).tobytes()
        assert got["picture_uses"] == frame.picture_uses.tobytes()
        assert got["radials"] == frame.radials.tobytes()
        assert got["shapes"] == shapes.tobytes()
        assert got["tiles"] == tiles.tobytes()
        assert got["tile_jobs"] == jobs.tobytes()
        assert int(np.frombuffer(got["n_jobs"], np.uint64)[0]) == len(frame.jobs)
        stats = np.frombuffer(got["stats"], np.int64)
        assert list(stats) == [frame.stats[k] for k in ("shapes", "excluded", "strands", "tiles", "splits",
                                                        "max_tile_shapes", "max_tile_strands", "tile_shape_refs")]
    return frame


@pytest.mark.parametrize("name", list(F.SCENES))
def test_fixture_scenes(name):
    fn, w, h, spec, _ = F.SCENES[name]
    check(S.flatten(fn(), w, h), spec)


@pytest.mark.parametrize("name", list(F.RANDOM))
def test_random_fixture_scenes(name):
    gen, sk = F.RANDOM[name]
    check(G.random_shapes(**gen), L.make_spec(**sk), seeds=(1, 2))


@pytest.mark.parametrize("tile,tpt,max_shape,max_strands,per_call", [
    (32, 32, 127, 4094, 1024),
    (16, 64, 7, 4094, 5),      # tiles split down to the 8-pixel minimum
    (64, 256, 127, 40, 3),     # the strand limit splits; many jobs
    (8, 32, 3, 4094, 1),       # one tile per job
    (128, 128, 1, 4094, 7),    # MAXSHAPE 1: every shape splits a tile
])
def test_random_scene_specs(tile, tpt, max_shape, max_strands, per_call):
    spec = L.make_spec(tile, tpt, 4096, 127, 8)
    spec.max_shape = max_shape
    spec.max_strands_per_tile = max_strands
    spec.max_tiles_per_call = per_call
    frame = check(G.random_shapes(seed=21, width=150, height=97, n_shapes=30), spec, seeds=(3, 4))
    if tile > 8 and (max_shape < 127 or max_strands < 4094):
        assert frame.stats["splits"] > 0


def test_glyph_page_all_substances():
    flat = G.glyph_page(seed=4, width=480, height=270, n_glyphs=150, n_shapes=25)
    frame = check(flat, L.make_spec(32, 32, 4096, 511, 8))
    assert len(frame.radials) > 0 and len(frame.picture_uses) > 0


def test_dense_small_canvas_splits_to_the_minimum():
    flat = G.random_shapes(seed=8, width=87, height=75, n_shapes=300)
    frame = check(flat, L.make_spec(32, 32, 4096, 127, 8))
    assert frame.stats["splits"] > 0 and frame.stats["max_tile_shapes"] > 127


def test_degenerate_shapes():
    """Shapes off the canvas (excluded), one-pair outlines (no strands), knobs in both
    directions, vertical and horizontal runs, NaN and infinite control points, and a
    substance without shapes."""
    flat = G.random_shapes(seed=9, width=64, height=48, n_shapes=12, seg_lo=1, seg_hi=6)
    pairs = flat.pairs.copy()
    pairs[3] = [np.nan, 5.0, np.inf, 7.0]
    pairs[7, 2] = -np.inf
    pairs[10:12] = [[10.0, 10.0, 10.0, 20.0], [10.0, 30.0, 10.0, 40.0]]
    pairs[-4:] += np.float32(500.0)  # the last shape leaves the canvas
    sub_start = flat.substance_shape_start.copy()
    sub_start[2] = sub_start[1]  # substance 1 keeps no shape
    import dataclasses
    flat = dataclasses.replace(flat, pairs=pairs, substance_shape_start=sub_start)
    frame = check(flat, L.make_spec(16, 16, 512, 127, 8))
    assert frame.stats["excluded"] >= 1


def test_one_pixel_canvas_and_empty_scene():
    check(G.random_shapes(seed=10, width=1, height=1, n_shapes=3), L.make_spec(8, 8, 512, 127, 8))
    empty = G.random_shapes(seed=10, width=40, height=30, n_shapes=0)
    check(empty, L.make_spec(16, 16, 512, 127, 8))


def test_page_4k():
    """The 3840x2160 page (12,000 shapes, 16,384 base tiles) at its bench spec."""
    flat = G.glyph_page()
    spec = L.make_spec(32, 32, 4096, 127, 8)
    spec.max_strands_per_tile = 4094
    check(flat, spec)


def test_wide_canvas_three_radix_passes():
    """A 16384-wide canvas at 32-pixel tiles: 512 x 512 base tiles (18-bit tile
    numbers, three radix passes) and many small local shapes."""
    rng = np.random.default_rng(31)
    specs = G.local_shape_specs(rng, 16384, 900, 3000, 4, 12)
    for sp in specs:
        sp.color = (float(rng.random()), float(rng.random()), float(rng.random()), 1.0)
    flat = G.flat_from_specs(specs, 16384, 900, (1, 1, 1, 1))
    frame = check(flat, L.make_spec(32, 32, 4096, 127, 8))
    assert frame.stats["tiles"] >= 512 * 512


def _random_flat(draw, st):
    """A flattened scene with uneven structure: substances without shapes, shapes
    without outlines, outlines of 0-12 pairs, points inside, outside and on the edges of
    the canvas, repeated points, and the odd NaN or infinity."""
    import dataclasses  # noqa: F401
    w = draw(st.integers(1, 300))
    h = draw(st.integers(1, 300))
    n_sub = draw(st.integers(0, 8))
    seed = draw(st.integers(0, 2 ** 32 - 1))
    rng = np.random.default_rng(seed)
    kinds, colors, pics, pxf, sub_start, compounds, outline_start, pair_start, chunks = [], [], [], [], [0], [], [0], [0], []
    n_pairs = 0
    special = np.array([np.nan, np.inf, -np.inf, 0.0, -0.0, w, h, -1e6, 1e6], np.float32)
    for _ in range(n_sub):
        kind = int(rng.integers(0, 3))
        kinds.append(kind)
        colors.append(rng.random(4, dtype=np.float32))
        pics.append(int(rng.integers(0, 2)))
        pxf.append(rng.random(3, dtype=np.float32))
        for _ in range(int(rng.integers(0, 4))):
            compounds.append(int(rng.integers(0, 2)))
            for _ in range(int(rng.integers(0, 4))):
                n = int(rng.integers(0, 13))
                pts = (rng.random((n, 4), dtype=np.float32) * np.float32(1.4) - np.float32(0.2))
                pts *= np.array([w, h, w, h], np.float32)
                if n and rng.random() < 0.3:
                    pts[int(rng.integers(0, n))] = pts[0]  # a repeated point
                if n and rng.random() < 0.1:
                    pts.reshape(-1)[int(rng.integers(0, 4 * n))] = special[int(rng.integers(0, special.size))]
                chunks.append(pts)
                n_pairs += n
                pair_start.append(n_pairs)
            outline_start.append(len(pair_start) - 1)
        sub_start.append(len(compounds))
    pictures = [G.noise_texture(seed=1, size=5), G.noise_texture(seed=2, size=9)]
    offsets, sizes, off = [], [], 0
    for p in pictures:
        offsets.append(off)
        sizes.append((p.shape[1], p.shape[0]))
        off += p.size
    rad = np.zeros(n_sub, dtype=L.RADIAL_DTYPE)
    return S.FlatScene(
        canvas_w=w, canvas_h=h, background=np.ones(4, np.float32),
        substance_kind=np.asarray(kinds, np.int32), substance_color=np.asarray(colors, np.float32).reshape(-1, 4),
        substance_picture=np.asarray(pics, np.int32), substance_picture_xform=np.asarray(pxf, np.float32).reshape(-1, 3),
        substance_radial=rad, substance_shape_start=np.asarray(sub_start, np.int32),
        shape_compound=np.asarray(compounds, np.int32), shape_outline_start=np.asarray(outline_start, np.int32),
        outline_pair_start=np.asarray(pair_start, np.int32),
        pairs=np.concatenate(chunks) if chunks else np.zeros((0, 4), np.float32),
        pictures=np.concatenate([p.reshape(-1) for p in pictures]),
        picture_size=np.asarray(sizes, np.int32), picture_offset=np.asarray(offsets, np.int32))


def test_random_scenes_and_specs():
    """Generated scenes and specs (tile 8-64, MAXSHAPE 1-127, strand limits down to 1,
    one to many tiles per job): the device passes give the host serializer's bytes."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=40, deadline=None, derandomize=True)
    @hyp.given(st.data())
    def run(data):
        flat = _random_flat(data.draw, st)
        tile = data.draw(st.sampled_from([8, 16, 32, 64]))
        spec = L.make_spec(tile, tile * data.draw(st.sampled_from([1, 2, 4])), 512, 127, 8)
        spec.max_shape = data.draw(st.sampled_from([1, 2, 3, 7, 127]))
        spec.max_strands_per_tile = data.draw(st.sampled_from([1, 5, 40, 4094]))
        spec.max_tiles_per_call = data.draw(st.sampled_from([1, 3, 1024]))
        check(flat, spec, seeds=(data.draw(st.integers(0, 1000)),))

    run()


def test_extreme_finite_coordinates():
    """Huge (up to 3.4e38), tiny and subnormal control-point coordinates: the passes'
    piles equal the host serializer's byte for byte (their box, split and tile tests
    compare floats and never convert them to integers)."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    values = {"huge": [3e37, -3e37, 1e30], "tiny": [1e-30, -1e-30, 1e-20], "subnormal": [1e-40, -1e-42, 1e-39],
              "mixed": [3e37, 1e-40, -1e30], "max": [3.4e38, -3.4e38, 3.4e38]}

    @hyp.settings(max_examples=40, deadline=None, derandomize=True)
    @hyp.given(seed=st.integers(0, 10 ** 6), w=st.integers(1, 200), h=st.integers(1, 150), n=st.integers(1, 30),
               tile=st.sampled_from([8, 16, 32]), mode=st.sampled_from(sorted(values)))
    def run(seed, w, h, n, tile, mode):
        flat = G.random_shapes(seed=seed, width=w, height=h, n_shapes=n, seg_lo=2, seg_hi=10)
        flat.pairs = flat.pairs.copy()
        for j, v in zip(np.random.default_rng(seed).integers(0, flat.pairs.size, size=3), values[mode]):
            flat.pairs.reshape(-1)[j] = np.float32(v)
        spec = L.make_spec(tile, tile, 4096, 127, 8)
        spec.max_tiles_per_call = 64
        check(flat, spec)

    run()


@pytest.mark.parametrize("threads", [2, 0])
def test_parallel_host_serializer(threads):
    """gudni_serialize_parallel (the passes on host threads) gives gudni_serialize's
    frame: piles, jobs, counters and point provenance."""
    cases = [(S.flatten(F.SCENES[n][0](), *F.SCENES[n][1:3]), F.SCENES[n][3]) for n in F.SCENES]
    cases.append((G.glyph_page(seed=4, width=480, height=270, n_glyphs=150, n_shapes=25), L.make_spec(32, 32, 4096, 511, 8)))
    spec = L.make_spec(16, 64, 4096, 7, 8)
    spec.max_tiles_per_call = 5
    cases.append((G.random_shapes(seed=21, width=150, height=97, n_shapes=30), spec))
    for flat, spec in cases:
        a = S.serialize_flat(flat, spec, threads=1)
        b = S.serialize_flat(flat, spec, threads=threads)
        assert a.geometry.tobytes() == b.geometry.tobytes()
        assert a.substances.tobytes() == b.substances.tobytes()
        assert a.picture_uses.tobytes() == b.picture_uses.tobytes() and a.radials.tobytes() == b.radials.tobytes()
        assert [(j.shapes.tobytes(), j.tiles.tobytes(), j.columns) for j in a.jobs] == \
               [(j.shapes.tobytes(), j.tiles.tobytes(), j.columns) for j in b.jobs]
        assert a.stats == b.stats
        assert a.point_offsets.tobytes() == b.point_offsets.tobytes()
        assert a.point_sources.tobytes() == b.point_sources.tobytes()
        assert a.point_weights.tobytes() == b.point_weights.tobytes()


def device_strand_table(geometry, seed=1):
    """The strand table of a pile by the device passes (strandTable) on the CPU."""
    from host_serialize.build import build
    with tempfile.TemporaryDirectory() as d:
        src, dst = os.path.join(d, "pile.bin"), os.path.join(d, "out.bin")
        geometry.tofile(src)
        r = subprocess.run([build(), "--strands", src, dst, str(seed)], capture_output=True, text=True,
                           env=dict(os.environ, ASAN_OPTIONS="detect_leaks=0"))
        assert r.returncode == 0, r.stderr[-4000:]
        return _read(dst)


def check_strands(geometry, seed=1):
    got = device_strand_table(geometry, seed)
    assert "error" not in got
    table, ys, first = host_strand_table(geometry)
    assert got["strand_table"] == table.tobytes()
    assert got["strand_y"] == ys.tobytes()
    assert got["strand_first"] == first.tobytes()
    return len(table)


def test_strand_table_of_piles():
    """The pile walk (strand_table.h) and the pointer-doubling passes give the same
    table on serialized piles, and stop at the same place on damaged ones: a
    truncated pile, headers made odd, too small or too large, and a pile cut inside
    its first strand."""
    frame = S.serialize_flat(G.glyph_page(seed=4, width=480, height=270, n_glyphs=150, n_shapes=25),
                             L.make_spec(32, 32, 4096, 511, 8))
    geo = frame.geometry
    n = check_strands(geo)
    assert n == frame.stats["strands"]
    table, _, _ = host_strand_table(geo)
    rng = np.random.default_rng(5)
    for trial in range(8):
        g = geo.copy()
        k = int(rng.integers(1, len(table)))
        off = int(table[k][0]) * 8
        if trial % 4 == 0:
            g = g[:off + 24]  # cut inside strand k (16-byte multiple kept below)
            g = g[:len(g) // 16 * 16]
        elif trial % 4 == 1:
            g[off:off + 2] = np.frombuffer(np.uint16(7).tobytes(), np.uint8)
        elif trial % 4 == 2:
            g[off:off + 2] = np.frombuffer(np.uint16(2).tobytes(), np.uint8)
        else:
            g[off:off + 2] = np.frombuffer(np.uint16(60000).tobytes(), np.uint8)
        assert check_strands(g, seed=trial) == k
    assert check_strands(geo[:16]) == 0
    assert check_strands(np.zeros(0, np.uint8)) == 0


def test_strand_table_of_the_page():
    """The 4K page's pile (a million 16-byte units: the long prefix sums run in
    chunks) through the pointer-doubling passes."""
    frame = S.serialize_flat(G.glyph_page(), L.make_spec(32, 32, 4096, 127, 8))
    assert frame.geometry.size // 16 > (1 << 16)
    assert check_strands(frame.geometry) == frame.stats["strands"]
