"""The oracle (CPU restatement of the reference kernels) against the golden fixtures
rendered by the reference's own Kernels.cl, and -- where the reference checkout is
present -- against the reference kernels on further seeded scenes."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
sys.path.insert(0, GOLDEN)

import fixture_scenes as F  # noqa: E402
from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402
from oracle import build_ref  # noqa: E402
from oracle import oracle as O  # noqa: E402

with open(os.path.join(GOLDEN, "golden.json")) as f:
    INDEX = json.load(f)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def pile_digest(frame):
    h = hashlib.sha256()
    h.update(frame.geometry.tobytes())
    h.update(frame.substances.tobytes())
    h.update(frame.picture_uses.tobytes())
    h.update(frame.radials.tobytes())
    for j in frame.jobs:
        h.update(j.shapes.tobytes())
        h.update(j.tiles.tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", F.ALL)
def test_serialized_piles_match_golden(name):
    frame = F.build(name)
    assert pile_digest(frame) == INDEX[name]["piles_sha256"]


@pytest.mark.parametrize("name", F.ALL)
def test_oracle_matches_golden(name):
    frame = F.build(name)
    st = {}
    img = O.render_frame(frame, stats=st)
    entry = INDEX[name]
    assert list(img.shape) == entry["shape"]
    if "image_file" in entry:
        want = np.load(os.path.join(GOLDEN, entry["image_file"]))
        assert np.array_equal(img, want), f"{(img != want).sum()} pixels differ"
    assert digest(img) == entry["image_sha256"]
    assert st["thresholds"] == entry["thresholds"]
    assert st["sections"] == entry["sections"]


def test_golden_sources_are_reference_kernels():
    for name, entry in INDEX.items():
        if F.reference_comparable(name):
            assert entry["source"] == "reference-kernels", name


needs_ref = pytest.mark.skipif(not O.ref_available(), reason="reference checkout not present")


@needs_ref
@pytest.mark.parametrize("seed,tpt,tile", [(21, 32, 32), (22, 64, 32), (23, 16, 16), (24, 128, 32)])
def test_oracle_matches_reference_kernels_random(seed, tpt, tile):
    flat = G.random_shapes(seed=seed, width=96 + seed, height=64 + 2 * seed, n_shapes=20, seg_lo=4, seg_hi=20)
    frame = S.serialize_flat(flat, L.make_spec(tile, tpt, 4096, 127, 8))
    st = {}
    a = O.render_frame(frame, stats=st)
    b = O.ref_render_frame(frame, max_thresholds=st["max_queue"] + 8)
    assert np.array_equal(a, b), f"{(a != b).sum()} pixels differ"


@needs_ref
def test_oracle_matches_reference_kernels_glyphs():
    flat = G.glyph_page(seed=9, width=320, height=200, n_glyphs=60, n_shapes=10, radial_frac=0.0)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 255, 4))
    st = {}
    a = O.render_frame(frame, stats=st)
    b = O.ref_render_frame(frame, max_thresholds=st["max_queue"] + 8)
    assert np.array_equal(a, b), f"{(a != b).sum()} pixels differ"


@pytest.mark.parametrize("factor,exact", [(0.25, True), (0.37, False)])
def test_oracle_matches_reference_kernels_stochastic(factor, exact):
    """STOCHASTIC_FACTOR != 0.  The reference pastes the factor as a decimal literal,
    so its jitter term is a double product; the oracle's is float.  A power-of-two
    factor scales exactly in both, so the images agree bit for bit; any other factor
    may round one way or the other now and then, inside the parity bar."""
    if not O.ref_available(127, 8, factor):
        pytest.skip("reference checkout not present")
    spec = L.make_spec(32, 32, 4096, 127, 8, stochastic_factor=factor)
    frame = S.serialize_flat(G.glyph_page(seed=8, width=200, height=150, n_glyphs=50, n_shapes=12, radial_frac=0.0),
                             spec)
    st = {}
    a = O.render_frame(frame, stats=st)
    b = O.ref_render_frame(frame, max_thresholds=st["max_queue"] + 8)
    if exact:
        assert np.array_equal(a, b), f"{(a != b).sum()} pixels differ"
    else:
        from conftest import assert_parity
        assert_parity(a, b, max_lsb=1, min_exact=0.999)


def test_oracle_reports_overflow():
    """A column that needs more thresholds than max_thresholds is reported, not
    silently corrupted (the reference writes past its slab there)."""
    frame = F.build("random_128x96")
    st = {}
    O.render_frame(frame, stats=st, max_thresholds=8)
    assert st["overflow"] == 1


def test_radial_matches_baked_texture():
    """The radial-gradient substance equals, within 1 LSB, the same gradient baked into
    an RGBA8 picture (the reference's PictureFunction route, Figure/Picture.hs:59-73)."""
    w, h = 40, 32
    circle = S.segments_to_outline([S.curved(1, 0, 1, 1), S.curved(0, 1, -1, 1), S.curved(-1, 0, -1, -1),
                                    S.curved(0, -1, 1, -1)])
    body = S.t_translate(20, 16, S.t_scale(14, S.shape([circle])))
    center, radius, inner, outer = (18.0, 15.0), 12.0, (0.9, 0.1, 0.2, 1.0), (0.1, 0.2, 0.8, 1.0)
    direct = S.Scene((1, 1, 1, 1), S.radial_with(center, radius, inner, outer, body))
    ys, xs = np.mgrid[0:h, 0:w].astype(np.float32)
    t = np.minimum(np.sqrt((xs - center[0]) ** 2 + (ys - center[1]) ** 2) / np.float32(radius), 1.0)
    rgba = np.stack([inner[i] + (outer[i] - inner[i]) * t for i in range(4)], -1)
    baked = S.Picture(np.round(rgba * 255).astype(np.uint8))
    tex = S.Scene((1, 1, 1, 1), S.texture_with("g", body), pictures={"g": baked})
    spec = L.make_spec(16, 16, 512, 127, 8)
    a = O.render_frame(S.serialize(direct, w, h, spec))
    b = O.render_frame(S.serialize(tex, w, h, spec))
    from conftest import assert_parity
    # the baked picture quantizes the colour to 8 bits before compositing, so about
    # half the pixels land one LSB apart; none may be further
    assert_parity(a, b, max_lsb=1, min_exact=0.3)


def test_bake_radials_matches_radial_substance():
    """A glyph page with radial gradients renders within one LSB of the same page with
    each gradient baked into a picture (scene.bake_radials, the form the reference
    kernels can take)."""
    flat = G.glyph_page(seed=3, width=256, height=192, n_glyphs=60, n_shapes=30)
    assert np.any(flat.substance_kind == 2)
    baked = S.bake_radials(flat)
    assert not np.any(baked.substance_kind == 2)
    spec = L.make_spec(32, 32, 4096, 127, 8)
    a = O.render_frame(S.serialize_flat(flat, spec))
    b = O.render_frame(S.serialize_flat(baked, spec))
    from conftest import assert_parity
    assert_parity(a, b, max_lsb=1, min_exact=0.5)


@needs_ref
def test_reference_kernels_refuse_radial_tags():
    """The reference kernels read a radial tag as a picture reference with an arbitrary
    usage index; the driver refuses such a job instead of running it."""
    flat = G.glyph_page(seed=3, width=256, height=192, n_glyphs=60, n_shapes=30)
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 127, 8))
    assert len(frame.radials)
    with pytest.raises(RuntimeError):
        O.ref_render_frame(frame, max_thresholds=4096)


@needs_ref
def test_reference_kernels_on_baked_page():
    """The reference kernels on the baked page equal the oracle on the baked page."""
    flat = S.bake_radials(G.glyph_page(seed=3, width=256, height=192, n_glyphs=60, n_shapes=30))
    frame = S.serialize_flat(flat, L.make_spec(32, 32, 4096, 127, 8))
    st = {}
    a = O.render_frame(frame, stats=st)
    b = O.ref_render_frame(frame, max_thresholds=st["max_queue"] + 8)
    assert np.array_equal(a, b)
