"""Seeded synthetic scenes for the raster path's workloads.

The reference ships no scene data or golden images; these generators produce the
shapes, sizes and value distributions of its headline configurations from a fixed
seed (numpy PCG64, identical on x86 and Arm):

  random_shapes      closed shapes of U{8..32} quadratic segments, anchors and controls
                     uniform over the canvas, RGB U[0,1], alpha U[0.3,1], all unioned
                     in z-order (first shape front-most) -- the 512x512 64-shape plain
                     workload, the batched mix and the differentiation scenes
  glyph_page         the 3840x2160 page: glyph-like outlines laid out in lines plus
                     random shapes, subtract combinators, radial gradients, textures
  batch_mix          256 scenes with log-uniform sides and shape counts

Scenes are built directly as FlatScene records (the traversal order the shape-tree
walker produces), so large batches serialize without building Python trees; the
tree form of the same scene is available for cross-checking.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Tuple

import numpy as np

from . import lib as L
from . import scene as S


def _rng(seed) -> np.random.Generator:
    return np.random.default_rng(seed)


@dataclass
class ShapeSpec:
    """One substance of a generated scene: its outlines (list of (n,4) float32 arrays
    per compound leaf), compound types, and substance."""
    leaves: List[List[np.ndarray]]
    compounds: List[int]
    kind: int = 0
    color: Tuple[float, float, float, float] = (0, 0, 0, 1)
    picture: int = 0
    picture_xform: Tuple[float, float, float] = (0.0, 0.0, 1.0)
    radial: Optional[tuple] = None


def flat_from_specs(specs: List[ShapeSpec], width: int, height: int, background,
                    pictures: Optional[List[np.ndarray]] = None) -> S.FlatScene:
    kinds, colors, pics, pxf, sub_start = [], [], [], [], [0]
    rad = np.zeros(len(specs), dtype=L.RADIAL_DTYPE)
    compounds, outline_start, pair_start, chunks = [], [0], [0], []
    n_pairs = 0
    for i, sp in enumerate(specs):
        kinds.append(sp.kind)
        colors.append(sp.color)
        pics.append(sp.picture)
        pxf.append(sp.picture_xform)
        if sp.radial is not None:
            cx, cy, r, inner, outer = sp.radial
            rad[i]["center_x"], rad[i]["center_y"], rad[i]["radius"] = cx, cy, r
            rad[i]["inner"], rad[i]["outer"] = inner, outer
        for leaf, comp in zip(sp.leaves, sp.compounds):
            compounds.append(comp)
            for o in leaf:
                chunks.append(o)
                n_pairs += o.shape[0]
                pair_start.append(n_pairs)
            outline_start.append(len(pair_start) - 1)
        sub_start.append(len(compounds))
    sizes, offsets, pdata, off = [], [], [], 0
    for p in pictures or []:
        sizes.append((p.shape[1], p.shape[0]))
        offsets.append(off)
        pdata.append(p.reshape(-1))
        off += p.size
    return S.FlatScene(
        canvas_w=width, canvas_h=height,
        background=np.asarray(background, np.float32),
        substance_kind=np.asarray(kinds, np.int32),
        substance_color=np.ascontiguousarray(np.asarray(colors, np.float32).reshape(-1, 4)),
        substance_picture=np.asarray(pics, np.int32),
        substance_picture_xform=np.ascontiguousarray(np.asarray(pxf, np.float32).reshape(-1, 3)),
        substance_radial=rad,
        substance_shape_start=np.asarray(sub_start, np.int32),
        shape_compound=np.asarray(compounds, np.int32),
        shape_outline_start=np.asarray(outline_start, np.int32),
        outline_pair_start=np.asarray(pair_start, np.int32),
        pairs=np.ascontiguousarray(np.concatenate(chunks) if chunks else np.zeros((0, 4), np.float32),
                                   dtype=np.float32),
        pictures=np.concatenate(pdata) if pdata else np.zeros(0, np.uint8),
        picture_size=np.asarray(sizes, np.int32).reshape(-1, 2),
        picture_offset=np.asarray(offsets, np.int32),
    )


def random_shape_specs(rng, width, height, n_shapes, seg_lo=8, seg_hi=32,
                       alpha_lo=0.3) -> List[ShapeSpec]:
    """Closed shapes of U{seg_lo..seg_hi} curved segments with anchors and controls
    uniform in [0,width)x[0,height), RGB U[0,1], alpha U[alpha_lo,1]."""
    specs = []
    scale = np.asarray([width, height, width, height], np.float32)
    for _ in range(n_shapes):
        n = int(rng.integers(seg_lo, seg_hi + 1))
        pts = (rng.random((n, 4), dtype=np.float32) * scale).astype(np.float32)
        rgb = rng.random(3, dtype=np.float32)
        a = np.float32(alpha_lo + (1.0 - alpha_lo) * rng.random(dtype=np.float32))
        specs.append(ShapeSpec([[pts]], [S.ADD], 0, (float(rgb[0]), float(rgb[1]), float(rgb[2]), float(a))))
    return specs


def local_shape_specs(rng, width, height, n_shapes, seg_lo=8, seg_hi=32, size_lo=16.0,
                      size_hi=1024.0) -> List[ShapeSpec]:
    """Random closed shapes like random_shape_specs, but each confined to a box of
    side log-uniform in [size_lo, size_hi] placed uniformly on the canvas, so the
    shapes per tile vary strongly across the canvas."""
    specs = []
    for _ in range(n_shapes):
        n = int(rng.integers(seg_lo, seg_hi + 1))
        side = np.float32(np.exp(rng.uniform(np.log(size_lo), np.log(size_hi))))
        ox = np.float32(rng.random() * width) - side / 2
        oy = np.float32(rng.random() * height) - side / 2
        pts = rng.random((n, 4), dtype=np.float32) * side
        pts[:, 0::2] += ox
        pts[:, 1::2] += oy
        rgb = rng.random(3, dtype=np.float32)
        a = np.float32(0.3 + 0.7 * rng.random(dtype=np.float32))
        specs.append(ShapeSpec([[pts.astype(np.float32)]], [S.ADD], 0,
                               (float(rgb[0]), float(rgb[1]), float(rgb[2]), float(a))))
    return specs


WHITE = (1.0, 1.0, 1.0, 1.0)


def random_shapes(seed=0, width=512, height=512, n_shapes=64, seg_lo=8, seg_hi=32) -> S.FlatScene:
    """The plain small workload: 512x512 canvas, 64 random closed shapes of 8-32
    quadratic segments, all unioned in z-order onto a white background."""
    rng = _rng(seed)
    return flat_from_specs(random_shape_specs(rng, width, height, n_shapes, seg_lo, seg_hi),
                           width, height, WHITE)


def random_shapes_tree(seed=0, width=512, height=512, n_shapes=64, seg_lo=8, seg_hi=32) -> S.Scene:
    """The same scene as random_shapes, built through the ShapeTree API."""
    rng = _rng(seed)
    specs = random_shape_specs(rng, width, height, n_shapes, seg_lo, seg_hi)
    items = [S.solid(sp.color, S.shape([S.Outline(sp.leaves[0][0])])) for sp in specs]
    return S.Scene(WHITE, S.overlap(items))


def noise_texture(seed=7, size=1024) -> np.ndarray:
    """Seeded size x size RGBA8 uniform-noise picture."""
    return _rng(seed).integers(0, 256, size=(size, size, 4), dtype=np.uint8)


def _glyph_contour(rng, n_seg, cx, cy, em, inner=False) -> np.ndarray:
    """A glyph-like closed contour: a wobbly loop of quadratic segments around (cx,cy)
    with radius ~em/2 (em/4 for the inner counter)."""
    ang = np.sort(rng.random(n_seg, dtype=np.float32)) * np.float32(2 * np.pi)
    base = np.float32(em * (0.22 if inner else 0.45))
    r = base * (np.float32(0.75) + np.float32(0.5) * rng.random(n_seg, dtype=np.float32))
    on_x = cx + r * np.cos(ang)
    on_y = cy + r * np.sin(ang)
    nxt = np.roll(np.arange(n_seg), -1)
    mid_ang = ang + np.float32(0.5) * ((np.roll(ang, -1) - ang) % np.float32(2 * np.pi))
    rc = base * (np.float32(0.6) + np.float32(0.8) * rng.random(n_seg, dtype=np.float32))
    off_x = cx + rc * np.cos(mid_ang)
    off_y = cy + rc * np.sin(mid_ang)
    del nxt
    pts = np.stack([on_x, on_y, off_x, off_y], axis=1).astype(np.float32)
    if inner:  # counter runs the other way
        pts = pts[::-1].copy()
    return pts


def glyph_page(seed=1, width=3840, height=2160, n_glyphs=5000, n_shapes=2000,
               subtract_frac=0.3, radial_frac=0.2, texture_frac=0.1) -> S.FlatScene:
    """The 4K page: n_glyphs glyph-like outlines (2 contours of 10-40 quadratic
    segments, em size log-uniform 12-48 px) laid out in lines, plus n_shapes random
    shapes of 8-32 segments each confined to a box of side log-uniform 16-1024 px;
    subtract_frac of the substances subtract a smaller second shape, radial_frac use
    a radial gradient, texture_frac a seeded 1024^2 noise texture.  Substances are
    shuffled into one z-order."""
    rng = _rng(seed)
    specs: List[ShapeSpec] = []
    x, y, line_h = 8.0, 8.0, 0.0
    for _ in range(n_glyphs):
        em = float(np.exp(rng.uniform(np.log(12.0), np.log(48.0))))
        if x + em > width - 8:
            x = 8.0
            y += line_h * 1.2
            line_h = 0.0
        if y + em > height - 8:
            y = 8.0
        cx, cy = np.float32(x + em / 2), np.float32(y + em / 2)
        outer = _glyph_contour(rng, int(rng.integers(10, 41)), cx, cy, em)
        inner = _glyph_contour(rng, int(rng.integers(10, 41)), cx, cy, em, inner=True)
        specs.append(_decorate(rng, ShapeSpec([[outer, inner]], [S.ADD]), width, height,
                               subtract_frac, radial_frac, texture_frac, em))
        x += em * 0.8
        line_h = max(line_h, em)
    for sp in local_shape_specs(rng, width, height, n_shapes, 8, 32):
        specs.append(_decorate(rng, sp, width, height, subtract_frac, radial_frac, texture_frac,
                               float(min(width, height)) / 8))
    order = rng.permutation(len(specs))
    specs = [specs[i] for i in order]
    return flat_from_specs(specs, width, height, WHITE, [noise_texture(seed + 6)])


def _decorate(rng, sp: ShapeSpec, width, height, subtract_frac, radial_frac, texture_frac, size):
    rgb = rng.random(3, dtype=np.float32)
    a = float(0.3 + 0.7 * rng.random())
    sp.color = (float(rgb[0]), float(rgb[1]), float(rgb[2]), a)
    u = rng.random()
    if u < radial_frac:
        sp.kind = 2
        c2 = rng.random(3, dtype=np.float32)
        sp.radial = (float(rng.random() * width), float(rng.random() * height),
                     float(4.0 + rng.random() * size * 2), sp.color,
                     (float(c2[0]), float(c2[1]), float(c2[2]), float(0.3 + 0.7 * rng.random())))
    elif u < radial_frac + texture_frac:
        sp.kind = 1
        sp.picture = 0
        sp.picture_xform = (float(-rng.random() * 256), float(-rng.random() * 256),
                            float(0.5 + 2.0 * rng.random()))
    if rng.random() < subtract_frac:
        # subtract a smaller copy of the first outline, shrunk toward its centroid
        o = sp.leaves[0][0]
        cx, cy = o[:, 0].mean(), o[:, 1].mean()
        k = np.float32(0.5)
        small = o.copy()
        small[:, 0::2] = (cx + (o[:, 0::2] - cx) * k).astype(np.float32)
        small[:, 1::2] = (cy + (o[:, 1::2] - cy) * k).astype(np.float32)
        # cSubtract a b: b sits above a with the subtract tag (traversal visits b first)
        sp.leaves = [[small]] + sp.leaves
        sp.compounds = [S.SUBTRACT] + sp.compounds
    return sp


def log_uniform_int(rng, lo, hi) -> int:
    return int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))


def batch_mix(seed=2, n_scenes=256, side_lo=64, side_hi=1024, shapes_lo=10, shapes_hi=2000):
    """The batched workload: scenes with canvas sides and shape counts log-uniform,
    same shape generator as random_shapes.  Returns a list of FlatScenes."""
    rng = _rng(seed)
    scenes = []
    for _ in range(n_scenes):
        w = log_uniform_int(rng, side_lo, side_hi)
        h = log_uniform_int(rng, side_lo, side_hi)
        n = log_uniform_int(rng, shapes_lo, shapes_hi)
        sub_seed = int(rng.integers(0, 2**31))
        scenes.append(random_shapes(sub_seed, w, h, n))
    return scenes
