"""The FP64 reference adjoint (oracle/adjoint_oracle.cpp) against the raster oracle
and against central differences of the loss."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402
from oracle import oracle as O  # noqa: E402

SPEC = L.make_spec(32, 32, 4096, 127, 8)


def small_scene(seed=5, w=64, h=48, n=6):
    return G.random_shapes(seed=seed, width=w, height=h, n_shapes=n, seg_lo=6, seg_hi=10)


def to_bytes(img):
    """The reference's colour -> BGRA8 conversion (convert_uchar_sat_rtz of 255*c,
    alpha 255) applied to the adjoint's float image."""
    def tb(v):
        v = v.astype(np.float32) * np.float32(255.0)
        return np.where(~(v > 0), 0, np.where(v >= 255, 255, np.floor(v))).astype(np.uint32)
    r, g, b = tb(img[..., 0]), tb(img[..., 1]), tb(img[..., 2])
    return b | (g << 8) | (r << 16) | np.uint32(255 << 24)


def jittered_target(make, sigma, seed=1):
    rng = np.random.default_rng(seed)
    t = make()
    t.pairs = (t.pairs + rng.normal(0, sigma, t.pairs.shape)).astype(np.float32)
    return O.render_float(S.serialize_flat(t, SPEC))


def loss_of(flat, target):
    im = O.render_float(S.serialize_flat(flat, SPEC))
    d = im[..., :3].astype(np.float64) - target[..., :3]
    return float(np.sum(d * d))


@pytest.mark.parametrize("seed", [5, 6, 7])
def test_adjoint_forward_is_the_raster_forward(seed):
    """The adjoint's float image, converted to bytes, is the raster oracle's image."""
    frame = S.serialize_flat(small_scene(seed), SPEC)
    img = O.render_float(frame)
    assert np.array_equal(to_bytes(img), O.render_frame(frame))


def test_adjoint_forward_glyph_page():
    """Same on a page with subtraction, textures and radial gradients."""
    frame = S.serialize_flat(G.glyph_page(seed=3, width=256, height=192, n_glyphs=60, n_shapes=30), SPEC)
    img = O.render_float(frame)
    b = O.render_frame(frame)
    # texture and gradient colours go through the same arithmetic; allow the odd
    # pixel whose colour sits on a byte boundary
    assert np.mean(to_bytes(img) == b) > 0.999


def test_colour_gradient_matches_central_differences():
    make = small_scene
    target = jittered_target(make, 2.0)
    frame = S.serialize_flat(make(), SPEC)
    _, _, g_sub, _ = O.loss_and_gradient(frame, target)
    h = 1e-3
    checked = 0
    for sid in range(len(frame.substances)):
        for ch in range(4):
            if abs(g_sub[sid, ch]) < 1e-2 * np.abs(g_sub).max():
                continue
            fp, fm = make(), make()
            fp.substance_color[sid, ch] += h
            fm.substance_color[sid, ch] -= h
            fd = (loss_of(fp, target) - loss_of(fm, target)) / (2 * h)
            assert abs(fd - g_sub[sid, ch]) <= 1e-3 * abs(fd) + 1e-4, (sid, ch, fd, g_sub[sid, ch])
            checked += 1
    assert checked >= 8


def test_geometry_gradient_matches_central_differences():
    """Point gradients against central differences at h = 1e-2 px and 1e-3 px.

    The loss is piecewise smooth, and not continuous, in the points: a curve is
    rendered as the lines of its column-local bifurcation (Kernels.cl:1233-1258), whose
    depth and branch change with the points, so the lines jump by up to the flatness
    bound when an event is crossed.  A central difference that straddles such an event
    picks up jump / 2h; the adjoint is the derivative of the piece the forward pass
    is on.  So the test bounds the median relative error over the largest entries and
    the share of entries within 10 %, not every entry."""
    make = small_scene
    target = jittered_target(make, 2.0)
    frame = S.serialize_flat(make(), SPEC)
    _, g_geo, _, _ = O.loss_and_gradient(frame, target)
    gp = S.pair_gradient(frame, g_geo)
    idx = np.argsort(-np.abs(gp.ravel()))[:16]
    for h, med_tol in ((1e-2, 0.05), (1e-3, 0.01)):
        a, f = [], []
        for k in idx:
            p, c = divmod(int(k), 4)
            fp, fm = make(), make()
            fp.pairs[p, c] += h
            fm.pairs[p, c] -= h
            f.append((loss_of(fp, target) - loss_of(fm, target)) / (2 * h))
            a.append(gp[p, c])
        a, f = np.asarray(a), np.asarray(f)
        rel = np.abs(a - f) / np.maximum(np.abs(f), 1e-9)
        assert np.median(rel) <= med_tol, (h, rel)
        assert np.mean(rel <= 0.10) >= 0.75, (h, rel)


def test_pair_gradient_sums_knob_splits():
    """pair_gradient is the transpose of the serializer's point provenance: moving a
    scene point by e moves each pile point by weight * e, so <g_pile, d pile> equals
    <pair_gradient(g_pile), e>."""
    flat = small_scene()
    frame = S.serialize_flat(flat, SPEC)
    rng = np.random.default_rng(3)
    g = rng.normal(size=frame.geometry.size // 4)
    gp = S.pair_gradient(frame, g)
    p, c = 3, 1
    e = 1e-2
    flat2 = small_scene()
    flat2.pairs[p, c] += e
    frame2 = S.serialize_flat(flat2, SPEC)
    if frame2.geometry.size != frame.geometry.size:
        pytest.skip("the move changed the pile layout")
    d = frame2.geometry.view(np.float32).astype(np.float64) - frame.geometry.view(np.float32).astype(np.float64)
    # only point floats move (headers and sizes are equal bit patterns)
    lhs = float(np.dot(g, np.nan_to_num(d)))
    assert abs(lhs - gp[p, c] * e) <= 1e-4 * max(1.0, abs(lhs))


def test_adam_step_matches_the_textbook_update():
    """fit.DeviceAdam: bias-corrected first and second moments (Kingma & Ba,
    Algorithm 1), on torch tensors (here on the CPU)."""
    import torch
    from gudni_gb300.fit import DeviceAdam
    opt = DeviceAdam(lr=0.1)
    x = np.array([1.0, -2.0])
    g1, g2 = np.array([0.5, -1.0]), np.array([0.25, 2.0])
    t = lambda a: torch.from_numpy(a.copy())  # noqa: E731
    x1 = opt.step(t(x), t(g1)).numpy()
    np.testing.assert_allclose(x1, x - 0.1 * np.sign(g1), rtol=1e-6)  # first step: lr * g / |g|
    m = 0.9 * 0.1 * g1 + 0.1 * g2
    v = 0.999 * 0.001 * g1 ** 2 + 0.001 * g2 ** 2
    mh, vh = m / (1 - 0.9 ** 2), v / (1 - 0.999 ** 2)
    np.testing.assert_allclose(opt.step(t(x1), t(g2)).numpy(), x1 - 0.1 * mh / (np.sqrt(vh) + 1e-8), rtol=1e-9)


def test_batch_pair_gradients_equal_each_frames_pair_gradient():
    """fit.pair_gradients (every scene of a batch at once, as the fitting step runs it
    on the device) gives scene.pair_gradient of each frame, on the frame's slice of a
    batch pile gradient (here random, on the CPU)."""
    import torch
    from gudni_gb300 import batch as B
    from gudni_gb300.fit import pair_gradients
    flats = [G.random_shapes(seed=s, width=64, height=48, n_shapes=5) for s in range(3)]
    frames = [S.serialize_flat(f, L.make_spec(16, 16, 1024, 127, 2)) for f in flats]
    batch = B.build_batch(frames)
    rng = np.random.default_rng(1)
    gg = rng.standard_normal(batch.geometry.size // 4).astype(np.float32)
    pair_start = np.cumsum([0] + [len(f.pairs) for f in flats])
    got = pair_gradients(frames, batch.frame_geo_offsets, pair_start, torch.from_numpy(gg)).numpy()
    for i, fr in enumerate(frames):
        g0 = int(batch.frame_geo_offsets[i]) // 4
        want = S.pair_gradient(fr, gg[g0:g0 + fr.geometry.size // 4])
        np.testing.assert_allclose(got[pair_start[i]:pair_start[i + 1]], want, rtol=1e-12, atol=1e-12)


def test_fit_checkpoint_round_trip(tmp_path):
    """BatchFit.save / load: a fit continued from a checkpoint has the same curve
    pairs, colours, Adam moments and step counts as the one that wrote it (the state
    here on the CPU, without a rasterizer), and a checkpoint of other scenes is refused."""
    import torch
    from gudni_gb300.fit import BatchFit, DeviceAdam

    def fake_fit(flats):
        f = BatchFit.__new__(BatchFit)
        f.torch, f.dev, f.flats, f.steps = torch, torch.device("cpu"), flats, 0
        f.pair_start = np.cumsum([0] + [len(x.pairs) for x in flats])
        f.sub_start = np.cumsum([0] + [len(x.substance_color) for x in flats])
        f.point_opt, f.color_opt = DeviceAdam(0.5), DeviceAdam(0.01)
        return f

    flats = [G.random_shapes(seed=s, width=64, height=48, n_shapes=4) for s in range(3)]
    a = fake_fit(flats)
    pairs = torch.from_numpy(np.concatenate([x.pairs for x in flats]).astype(np.float64))
    for k in range(3):  # three Adam steps on made-up gradients
        pairs = a.point_opt.step(pairs, torch.full_like(pairs, 0.1 * (k + 1)))
        a.steps += 1
    for i, x in enumerate(a.flats):
        x.pairs = pairs[a.pair_start[i]:a.pair_start[i + 1]].float().numpy()
    path = str(tmp_path / "fit.npz")
    a.save(path)
    b = fake_fit([G.random_shapes(seed=s, width=64, height=48, n_shapes=4) for s in range(3)])
    b.load(path)
    assert b.steps == 3 and b.point_opt.t == 3 and b.color_opt.t == 0 and b.color_opt.m is None
    for x, y in zip(a.flats, b.flats):
        np.testing.assert_array_equal(x.pairs, y.pairs)
        np.testing.assert_array_equal(x.substance_color, y.substance_color)
    assert torch.equal(a.point_opt.m, b.point_opt.m) and torch.equal(a.point_opt.v, b.point_opt.v)
    other = fake_fit([G.random_shapes(seed=9, width=64, height=48, n_shapes=5)])
    with pytest.raises(ValueError):
        other.load(path)
