"""The serializer on the device (gudni_serialize_device) through the C ABI: its piles,
copied back, equal the host serializer's byte for byte, its counters equal the host's,
and the frame it leaves on the device renders as the oracle renders the host frame."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import fixture_scenes as F  # noqa: E402
from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402
from gudni_gb300.raster import RasterError, Rasterizer  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

STATS = ("shapes", "excluded", "strands", "tiles", "splits", "max_tile_shapes", "max_tile_strands", "tile_shape_refs")


def small_spec(tile, tpt, max_shape=127, per_call=1024):
    spec = L.make_spec(tile, tpt, 4096, max_shape, 8)
    spec.max_tiles_per_call = per_call
    return spec


def scenes():
    fn, w, h, spec, _ = F.SCENES["textured"]
    yield "textured", S.flatten(fn(), w, h), spec
    yield "glyphs", G.glyph_page(seed=4, width=480, height=270, n_glyphs=150, n_shapes=25), small_spec(32, 32, 511)
    yield "random512", G.random_shapes(seed=0, width=512, height=512, n_shapes=64), small_spec(32, 32)
    yield "splits", G.random_shapes(seed=21, width=150, height=97, n_shapes=30), small_spec(16, 64, 7, per_call=5)


@pytest.mark.parametrize("name", ["textured", "glyphs", "random512", "splits"])
def test_device_serializer_matches_host_and_renders(name):
    import torch
    flat, spec = next((f, s) for n, f, s in scenes() if n == name)
    frame = S.serialize_flat(flat, spec)
    shapes, tiles, jobs = S.concatenated_piles(frame)
    dev = torch.device("cuda:0")
    out = torch.zeros(flat.canvas_h * flat.canvas_w, dtype=torch.int32, device=dev)
    with Rasterizer(spec) as r:
        r.upload_pictures(flat.pictures)
        r.upload_random_field(frame.random_field)
        for provenance in (True, False):  # the second serialization reuses the context's buffers
            df = r.serialize_device(flat, provenance=provenance)
            got = r.download_device_frame(df)
            assert got["geometry"].tobytes() == frame.geometry.tobytes()
            assert got["shapes"].tobytes() == shapes.tobytes()
            assert got["tiles"].tobytes() == tiles.tobytes()
            assert np.array_equal(got["tile_jobs"], jobs)
            assert df.n_jobs == len(frame.jobs)
            assert list(df.stats) == [frame.stats[k] for k in STATS]
            if provenance:
                assert np.array_equal(got["point_offsets"], frame.point_offsets)
                assert np.array_equal(got["point_sources"], frame.point_sources)
                assert got["point_weights"].tobytes() == frame.point_weights.tobytes()
            else:
                assert df.n_points == 0
        r.raster_device_frame(df, flat.canvas_w, flat.canvas_h, flat.background, out.data_ptr(),
                              stream=L.current_stream_handle())
        r.sync_status()
        torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint32).reshape(flat.canvas_h, flat.canvas_w)
    assert np.array_equal(got, O.render_frame(frame))


def test_device_serializer_rejects_bad_scenes():
    flat = G.random_shapes(seed=3, width=64, height=48, n_shapes=6)
    spec = small_spec(16, 16)
    with Rasterizer(spec) as r:
        bad = S.FlatScene(**{**flat.__dict__, "shape_outline_start": flat.shape_outline_start[::-1].copy()})
        with pytest.raises(RasterError) as err:
            r.serialize_device(bad)
        assert err.value.code == -1
        pic = G.glyph_page(seed=4, width=200, height=120, n_glyphs=20, n_shapes=5, texture_frac=1.0)
        with pytest.raises(RasterError) as err:  # no picture pile uploaded: usages fall outside
            r.serialize_device(pic)
        assert err.value.code == -1


def test_device_serializer_gives_the_known_piles():
    """The known-answer piles derived from the reference's Haskell host
    (tests/golden/known_piles.py): the device serializer through the C ABI writes the
    same geometry pile and the same jobs, concatenated."""
    import json
    import known_piles as K
    with open(os.path.join(HERE, "golden", "known_piles.json")) as f:
        known = json.load(f)
    for name, (shapes, w, h, tile, tpt, per_job, max_strands) in K.scenes().items():
        spec = L.make_spec(tile, tpt, 4096, 127, 2, max_tiles_per_call=per_job, max_strands_per_tile=max_strands)
        flat = K.flat_scene(shapes, w, h)
        with Rasterizer(spec) as r:
            got = r.download_device_frame(r.serialize_device(flat))
        want = known[name]
        assert got["geometry"].tobytes().hex() == want["geometry"], name
        assert got["shapes"].tobytes() == b"".join(bytes.fromhex(j["shapes"]) for j in want["jobs"]), name
        base, tiles = 0, []
        for j in want["jobs"]:
            t = np.frombuffer(bytes.fromhex(j["tiles"]), dtype=L.TILE_DTYPE).copy()
            t["shape_start"] += base
            tiles.append(t)
            base += len(bytes.fromhex(j["shapes"])) // 16
        assert got["tiles"].tobytes() == np.concatenate(tiles).tobytes(), name


def test_device_serializer_on_the_4k_page():
    """The 3840x2160 page (5000 glyph-like outlines, 2000 shapes, subtract, gradients,
    textures: 12,145 shapes after the combinators) serialized by the device passes is
    the host serializer's frame byte for byte, provenance included, and renders the
    host frame's image."""
    import torch
    flat = G.glyph_page(seed=1)
    spec = L.make_spec(32, 32, 4096, 127, 8)
    frame = S.serialize_flat(flat, spec)
    shapes, tiles, jobs = S.concatenated_piles(frame)
    dev = torch.device("cuda:0")
    out = torch.zeros(flat.canvas_h * flat.canvas_w, dtype=torch.int32, device=dev)
    with Rasterizer(spec) as r:
        r.upload_pictures(flat.pictures)
        r.upload_random_field(frame.random_field)
        df = r.serialize_device(flat, provenance=True)
        got = r.download_device_frame(df)
        assert got["geometry"].tobytes() == frame.geometry.tobytes()
        assert got["shapes"].tobytes() == shapes.tobytes()
        assert got["tiles"].tobytes() == tiles.tobytes()
        assert np.array_equal(got["tile_jobs"], jobs)
        assert list(df.stats) == [frame.stats[k] for k in STATS]
        assert np.array_equal(got["point_offsets"], frame.point_offsets)
        assert got["point_weights"].tobytes() == frame.point_weights.tobytes()
        r.raster_device_frame(df, flat.canvas_w, flat.canvas_h, flat.background, out.data_ptr(),
                              stream=L.current_stream_handle())
        r.sync_status()
        torch.cuda.synchronize()
        host_img = r.raster_frame(frame)
    img = out.cpu().numpy().view(np.uint32).reshape(flat.canvas_h, flat.canvas_w)
    assert np.array_equal(img, host_img)
