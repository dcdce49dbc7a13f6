"""Batch builder: concatenated piles with rebased references render every scene exactly
as the scene's own piles do (checked on the CPU with the oracle); on the GPU, the
batched persistent launch (with and without the captured graph) and the per-scene
launches match the oracle."""
import copy

import numpy as np
import pytest

from gudni_gb300 import batch as B
from gudni_gb300 import lib as L
from gudni_gb300 import scene as S
from gudni_gb300 import scenes as G
from oracle import oracle as O


def small_frames():
    frames = []
    specs = [L.make_spec(16, 16, 1024, 255, 4), L.make_spec(32, 32, 1024, 255, 4), L.make_spec(32, 64, 1024, 255, 4)]
    for i, (w, h, n) in enumerate([(40, 30, 6), (77, 64, 15), (64, 96, 25), (33, 20, 4)]):
        frames.append(S.serialize_flat(G.random_shapes(seed=100 + i, width=w, height=h, n_shapes=n),
                                       specs[i % len(specs)]))
    # one scene with textures, gradients and subtract combinators
    frames.append(S.serialize_flat(G.glyph_page(seed=8, width=120, height=90, n_glyphs=30, n_shapes=6),
                                   L.make_spec(32, 32, 1024, 255, 4)))
    return frames


def scene_view(batch, fi):
    """The frame `fi` re-expressed over the batch's concatenated piles."""
    f = batch.frames[fi]
    first, count = batch.frame_tiles[fi]
    v = copy.copy(f)
    v.geometry, v.substances, v.pictures = batch.geometry, batch.substances, batch.pictures
    v.picture_uses, v.radials = batch.picture_uses, batch.radials
    tiles = batch.tiles[first:first + count].copy()
    # the view's single job indexes the concatenated shape pile directly
    v.jobs = [S.Job(batch.shapes, tiles, len(tiles) * f.spec.threads_per_tile)]
    return v


def test_batch_rebasing_matches_each_frame():
    frames = small_frames()
    batch = B.build_batch(frames)
    assert batch.out_pixels == sum(f.canvas_w * f.canvas_h for f in frames)
    for fi, f in enumerate(frames):
        want = O.render_frame(f)
        got = O.render_frame(scene_view(batch, fi))
        assert np.array_equal(got, want), f"frame {fi}: {(got != want).sum()} pixels differ"


def test_batch_scene_records():
    frames = small_frames()
    batch = B.build_batch(frames)
    assert len(batch.scenes) == sum(len(f.jobs) for f in frames)
    assert np.all(np.diff(batch.frame_offsets) > 0)
    assert batch.tile_cost.shape == (len(batch.tiles),)
    assert set(np.unique(batch.tile_scene)) == set(range(len(batch.scenes)))


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_render_matches_oracle(use_graph):
    frames = small_frames()
    batch = B.build_batch(frames)
    with B.BatchRasterizer(L.make_spec(32, 32, 1024, 255, 4)) as r:
        r.upload(batch)
        for _ in range(2):  # second pass replays the graph
            imgs = r.render_images(use_graph=use_graph)
            for f, img in zip(frames, imgs):
                assert np.array_equal(img, O.render_frame(f))


@pytest.mark.gpu
def test_batch_per_scene_launches_match_oracle(monkeypatch):
    monkeypatch.setenv("GUDNI_WORKING_CAPACITY", "16")  # exercise the full-capacity pass too
    frames = small_frames()
    batch = B.build_batch(frames)
    with B.BatchRasterizer(L.make_spec(32, 32, 1024, 255, 4)) as r:
        r.upload(batch)
        r.render_each_scene()
        imgs = batch.images(r.download())
    for f, img in zip(frames, imgs):
        assert np.array_equal(img, O.render_frame(f))


def test_autotune_buckets_and_tuned_specs():
    """Scenes fall into canvas-size buckets by their longer side; serialize_tuned gives
    every scene its bucket's (tile, threads per tile)."""
    from gudni_gb300 import autotune as A
    assert [A.bucket_of(w, h) for w, h in ((64, 64), (96, 40), (97, 10), (300, 500), (1024, 64))] == [0, 0, 1, 3, 4]
    flats = [G.random_shapes(seed=i, width=w, height=h, n_shapes=4) for i, (w, h) in enumerate(((64, 80), (200, 150)))]
    frames = A.serialize_tuned(flats, {0: (8, 64), 2: (16, 64)}, 127, 4096, 1 << 24)
    assert (frames[0].spec.max_tile_size, frames[0].spec.threads_per_tile) == (8, 64)
    assert (frames[1].spec.max_tile_size, frames[1].spec.threads_per_tile) == (16, 64)
    assert A.scene_cost(flats[1]) == 200 * 150 * 4
