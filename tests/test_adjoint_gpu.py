"""The CUDA adjoint (gudni_adjoint_tiles_device, gudni_batch_adjoint) against the FP64
reference adjoint in the oracle.  Bar: relative error <= 1e-3 on the gradient
vectors (geometry pile floats and substance colours), and on every entry larger
than 1 % of the largest."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from gudni_gb300 import adjoint as A  # noqa: E402
from gudni_gb300 import batch as B  # noqa: E402
from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402
from gudni_gb300.raster import Rasterizer  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

SPEC = L.make_spec(32, 32, 4096, 127, 8)
REL = 1e-3


def jitter(flat, sigma, seed):
    rng = np.random.default_rng(seed)
    flat.pairs = (flat.pairs + rng.normal(0, sigma, flat.pairs.shape)).astype(np.float32)
    return flat


def case(make, sigma=2.0, spec=SPEC):
    frame = S.serialize_flat(make(), spec)
    target = O.render_float(S.serialize_flat(jitter(make(), sigma, 1), spec))
    return frame, target


def check_vec(got, want, what):
    got = np.asarray(got, np.float64).ravel()
    want = np.asarray(want, np.float64).ravel()
    n = np.linalg.norm(want)
    assert n > 0, what
    rel = np.linalg.norm(got - want) / n
    assert rel <= REL, f"{what}: relative error {rel:.3e}"
    big = np.abs(want) > 0.01 * np.abs(want).max()
    worst = float(np.max(np.abs(got[big] - want[big]) / np.abs(want[big])))
    assert worst <= REL, f"{what}: worst large-entry relative error {worst:.3e}"
    return rel, worst


SCENES = {
    "random_64x48": lambda: G.random_shapes(seed=5, width=64, height=48, n_shapes=6, seg_lo=6, seg_hi=10),
    "random_160x120": lambda: G.random_shapes(seed=9, width=160, height=120, n_shapes=24),
    "glyphs_256x192": lambda: G.glyph_page(seed=3, width=256, height=192, n_glyphs=60, n_shapes=30),
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_adjoint_matches_fp64_reference(name):
    frame, target = case(SCENES[name])
    loss_ref, g_geo, g_sub, img_ref = O.loss_and_gradient(frame, target)
    with Rasterizer(frame.spec) as r:
        loss, img, gg, gs = A.FrameAdjoint(r, frame).loss_and_gradient(target)
        img, gg, gs = img.cpu().numpy(), gg.cpu().numpy(), gs.cpu().numpy()
    # forward: the same float image (I rgb and section area) up to float rounding
    np.testing.assert_allclose(img, img_ref, rtol=1e-5, atol=1e-5)
    assert abs(float(loss) - loss_ref) <= 1e-4 * loss_ref
    check_vec(gg, g_geo, "geometry gradient")
    check_vec(gs, g_sub, "substance gradient")


def test_adjoint_repeatable_and_accumulates_nothing_stale():
    frame, target = case(SCENES["random_160x120"])
    with Rasterizer(frame.spec) as r:
        fa = A.FrameAdjoint(r, frame)
        _, _, g1, s1 = fa.loss_and_gradient(target)
        g1, s1 = g1.cpu().numpy().copy(), s1.cpu().numpy().copy()
        _, _, g2, s2 = fa.loss_and_gradient(target)
        np.testing.assert_allclose(g2.cpu().numpy(), g1, rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(s2.cpu().numpy(), s1, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("name", ["random_160x120", "glyphs_256x192", "dense"])
def test_adjoint_generated_once_equals_regenerated(name):
    """The default adjoint (thresholds generated once per work unit, the forward
    scanning a copy) against gudni_set_adjoint_regenerate(ctx, 1) (the forward's own
    raster generation, the backward's second generation): the same float image bit
    for bit, and the same gradients up to the order of the atomic adds (float sums in
    another order: relative 1e-4 of an entry, or 1e-6 of the largest entry)."""
    if name == "dense":
        spec = L.make_spec(16, 64, 4096, 255, 4, max_strands_per_tile=1 << 24)
        frame, target = case(lambda: G.random_shapes(seed=93, width=128, height=128, n_shapes=120), spec=spec)
    else:
        frame, target = case(SCENES[name])
    with Rasterizer(frame.spec) as r:
        fa = A.FrameAdjoint(r, frame)
        _, i1, g1, s1 = fa.loss_and_gradient(target)
        i1, g1, s1 = i1.cpu().numpy().copy(), g1.cpu().numpy().copy(), s1.cpu().numpy().copy()
        r.set_adjoint_regenerate(True)
        _, i2, g2, s2 = fa.loss_and_gradient(target)
        np.testing.assert_array_equal(i2.cpu().numpy(), i1)
        for got, want in ((g2.cpu().numpy(), g1), (s2.cpu().numpy(), s1)):
            np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-6 * float(np.abs(want).max()))


def test_adjoint_threads_per_tile():
    make = lambda: G.random_shapes(seed=11, width=128, height=96, n_shapes=16)  # noqa: E731
    for tpt, tile in ((16, 16), (64, 32), (128, 32)):
        spec = L.make_spec(tile, tpt, 4096, 127, 8)
        frame, target = case(make, spec=spec)
        _, g_geo, g_sub, _ = O.loss_and_gradient(frame, target)
        with Rasterizer(spec) as r:
            _, _, gg, gs = A.FrameAdjoint(r, frame).loss_and_gradient(target)
            check_vec(gg.cpu().numpy(), g_geo, f"geometry gradient tpt={tpt}")
            check_vec(gs.cpu().numpy(), g_sub, f"substance gradient tpt={tpt}")


def test_batch_adjoint_matches_frames():
    import torch
    makes = [lambda s=s: G.random_shapes(seed=20 + s, width=48 + 16 * s, height=40 + 8 * s, n_shapes=5 + s)
             for s in range(4)]
    frames, targets = zip(*[case(m) for m in makes])
    batch = B.build_batch(list(frames))
    with B.BatchRasterizer(SPEC) as r:
        r.upload(batch)
        dev = torch.device("cuda")
        tgt = np.zeros((batch.out_pixels, 4), np.float32)
        for i, t in enumerate(targets):
            o = int(batch.frame_offsets[i])
            tgt[o:o + t.shape[0] * t.shape[1]] = t.reshape(-1, 4)
        target = torch.from_numpy(tgt).to(dev)
        image = torch.zeros_like(target)
        gg = torch.zeros(batch.geometry.size // 4, dtype=torch.float32, device=dev)
        gs = torch.zeros((len(batch.substances), 4), dtype=torch.float32, device=dev)
        r.adjoint(target, image, gg, gs)
        r.sync_status()
        gg, gs = gg.cpu().numpy(), gs.cpu().numpy()
        for i, f in enumerate(frames):
            _, g_geo, g_sub, _ = O.loss_and_gradient(f, targets[i])
            sg, ss = r.frame_slices(i)
            check_vec(gg[sg], g_geo, f"batch frame {i} geometry")
            check_vec(gs[ss], g_sub, f"batch frame {i} substances")


def test_batch_fit_reduces_loss():
    """A few Adam steps of the batched fitting loop bring every scene closer to its
    target (targets rendered from perturbed copies of the same scenes)."""
    from gudni_gb300 import fit as Fm
    spec = L.make_spec(16, 32, 4096, 127, 8, max_strands_per_tile=1 << 24)
    make = lambda i: G.random_shapes(seed=60 + i, width=64, height=64, n_shapes=12)  # noqa: E731
    targets = []
    for i in range(4):
        t = make(i)
        t = jitter(t, 2.0, 70 + i)
        targets.append(O.render_float(S.serialize_flat(t, spec)))
    fit = Fm.BatchFit([make(i) for i in range(4)], targets, spec, lr_points=0.3, lr_colors=0.01)
    try:
        first = fit.step()
        for _ in range(40):
            last = fit.step()
    finally:
        fit.close()
    assert last < 0.8 * first, (first, last)


def test_batch_fit_resumes_from_a_checkpoint(tmp_path):
    """BatchFit.save / load on the GPU: a fit continued in a new BatchFit from a
    checkpoint sees the same scenes as the fit that wrote it (the same loss, bit for
    bit: the forward image is deterministic) and takes the same step count."""
    from gudni_gb300 import fit as Fm
    spec = L.make_spec(16, 32, 4096, 127, 8, max_strands_per_tile=1 << 24)
    make = lambda i: G.random_shapes(seed=80 + i, width=48, height=40, n_shapes=8)  # noqa: E731
    targets = [O.render_float(S.serialize_flat(jitter(make(i), 2.0, 90 + i), spec)) for i in range(3)]
    path = str(tmp_path / "fit.npz")
    a = Fm.BatchFit([make(i) for i in range(3)], targets, spec, lr_points=0.3, lr_colors=0.01)
    try:
        for _ in range(3):
            a.step()
        a.save(path)
        want = a.evaluate()
    finally:
        a.close()
    b = Fm.BatchFit([make(i) for i in range(3)], targets, spec, lr_points=0.3, lr_colors=0.01)
    try:
        b.load(path)
        assert b.steps == 3
        assert b.evaluate() == want
        b.step()
        assert b.steps == 4
    finally:
        b.close()
