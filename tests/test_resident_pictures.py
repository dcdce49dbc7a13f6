"""Pictures packed once into a resident library (scene.PictureLibrary) instead of a
per-frame pile (makePictData, Figure/Picture.hs:159-167): the usages a bound scene
serializes to read the same texels, so the oracle renders the same image; the
geometry, shape and tile piles do not change.  CPU only (the oracle is the checker);
the C-ABI upload path is covered in test_raster_gpu.py."""
import dataclasses
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
from oracle import oracle as O  # noqa: E402


def library_with_others(named: dict) -> S.PictureLibrary:
    """A library that holds the scene's pictures after others, so that every offset
    differs from the per-frame pile's."""
    others = {f"other{i}": G.noise_texture(seed=90 + i, size=8 + 4 * i) for i in range(3)}
    return S.PictureLibrary({**others, **named})


def with_pile(frame, lib):
    return dataclasses.replace(frame, pictures=lib.pile)


def assert_same_piles(a, b):
    assert np.array_equal(a.geometry, b.geometry)
    assert np.array_equal(a.substances, b.substances)
    assert len(a.jobs) == len(b.jobs)
    for ja, jb in zip(a.jobs, b.jobs):
        assert np.array_equal(ja.shapes, jb.shapes) and np.array_equal(ja.tiles, jb.tiles)


def test_named_pictures_render_identically():
    w, h, spec = F.SCENES["textured"][1:4]
    scene = F.textured()
    per_frame = S.serialize(scene, w, h, spec)
    lib = library_with_others(scene.pictures)
    flat = S.flatten(scene, w, h)
    assert flat.picture_names == ["noise"]
    bound = lib.bind(flat)
    assert bound.pictures.size == 0
    frame = S.serialize_flat(bound, spec)
    assert len(frame.picture_uses) == len(per_frame.picture_uses) > 0
    assert np.all(frame.picture_uses["mem_offset"] == lib.offsets["noise"])
    assert np.all(frame.picture_uses["mem_offset"] != per_frame.picture_uses["mem_offset"])
    assert_same_piles(frame, per_frame)
    assert np.array_equal(O.render_frame(with_pile(frame, lib)), O.render_frame(per_frame))


def test_numbered_pictures_and_two_frames_share_one_pile():
    """Generated scenes number their pictures; two frames that use the same texture
    with different usage transforms render from one library pile as from their own
    piles."""
    spec = L.make_spec(32, 32, 4096, 511, 8)
    first = G.glyph_page(seed=4, width=320, height=180, n_glyphs=80, n_shapes=12, texture_frac=0.5)
    xf = first.substance_picture_xform.copy()
    xf[:, 0] += np.float32(13.0)
    xf[:, 1] -= np.float32(7.0)
    xf[:, 2] *= np.float32(1.5)
    second = dataclasses.replace(first, substance_picture_xform=xf)
    texture = first.pictures.reshape(1024, 1024, 4)
    lib = S.PictureLibrary({1: G.noise_texture(seed=10, size=64), 0: texture})
    for flat in (first, second):
        per_frame = S.serialize_flat(flat, spec)
        frame = S.serialize_flat(lib.bind(flat), spec)
        assert len(frame.picture_uses) > 0
        assert lib.offsets[0] != 0 and np.all(frame.picture_uses["mem_offset"] == lib.offsets[0])
        assert_same_piles(frame, per_frame)
        assert np.array_equal(O.render_frame(with_pile(frame, lib)), O.render_frame(per_frame))


def test_bind_rejects_unknown_or_resized_pictures():
    w, h = F.SCENES["textured"][1:3]
    scene = F.textured()
    flat = S.flatten(scene, w, h)
    with pytest.raises(KeyError):
        S.PictureLibrary({"other": G.noise_texture(seed=1, size=48)}).bind(flat)
    with pytest.raises(ValueError):
        S.PictureLibrary({"noise": G.noise_texture(seed=3, size=40)}).bind(flat)
    with pytest.raises(ValueError):
        S.PictureLibrary({"flat": np.zeros((4, 4, 3), np.uint8)})


def test_library_offsets_are_aligned_and_cover_the_pile():
    pics = {k: G.noise_texture(seed=k, size=s) for k, s in enumerate((3, 5, 7, 16))}
    lib = S.PictureLibrary(pics)
    end = 0
    for k, p in pics.items():
        off = lib.offsets[k]
        assert off % 4 == 0 and off == end
        w, h = lib.sizes[k]
        assert np.array_equal(lib.pile[off:off + 4 * w * h].reshape(h, w, 4), p)
        end = off + 4 * w * h
    assert end == lib.pile.size
