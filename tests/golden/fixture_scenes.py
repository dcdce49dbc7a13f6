"""Known-answer scenes for the raster path.

The reference ships no expected outputs; its interactive test scenes
(benchmarks/GudniTests.hs:65-98, 100-125, 245-414) name the edge cases that matter:
a sub-pixel square, a knob (a curve bulging past its end points), a self-intersecting
hourglass, collinear points, sub-pixel brackets, shape subtraction, many shapes per
tile (the MAXSHAPE cap), textures.  The scenes below exercise the same cases with
their own geometry, plus seeded random scenes.  make_golden.py renders them with the
reference's own kernels (oracle/_ref) and stores the results in this folder.
"""
from __future__ import annotations

import numpy as np

from gudni_gb300 import lib as L
from gudni_gb300 import scene as S
from gudni_gb300 import scenes as G


def rect(w, h):
    return S.segments_to_outline([S.straight(0, 0), S.straight(w, 0), S.straight(w, h), S.straight(0, h)])


def _solid(color, outlines):
    return S.solid(color, S.shape(outlines))


def tiny_square():
    return S.Scene((0, 0, 0, 1), S.t_translate(0.1, 0.1, _solid((1, 0, 0, 1), [rect(2, 2)])))


def knob():
    o = S.segments_to_outline([S.curved(0, 0, 1, 1), S.straight(0, 2)])
    return S.Scene((1, 1, 1, 1), S.t_translate(5, 3, S.t_scale(10, _solid((0.2, 0.2, 0.25, 1), [o]))))


def hourglass():
    o = S.segments_to_outline([S.straight(0, 0), S.straight(1, 1), S.straight(1, 0), S.straight(0, 1)])
    return S.Scene((1, 1, 1, 1), S.t_translate(2.5, 1.25, S.t_scale(12, _solid((0.1, 0.3, 0.6, 1), [o]))))


def six_point_rectangle():
    o = S.segments_to_outline([S.straight(0, 0), S.straight(1, 0), S.straight(2, 0), S.straight(2, 1),
                               S.straight(1, 1), S.straight(0, 1)])
    return S.Scene((1, 1, 1, 1), S.t_translate(3, 4, S.t_scale(9, _solid((0.4, 0.4, 0.4, 1), [o]))))


def two_brackets():
    a = S.segments_to_outline([S.straight(-0.2, 0.0), S.straight(1.2, 1.4), S.straight(1.2, 1.6),
                               S.straight(-0.2, 0.2)])
    b = S.segments_to_outline([S.straight(-0.2, 0.4), S.straight(1.2, 1.8), S.straight(1.2, 2.0),
                               S.straight(-0.2, 0.6)])
    tree = S.t_translate(4, 4, S.t_scale(3, S.overlap([_solid((1, 1, 1, 1), [a]), _solid((1, 1, 1, 1), [b])])))
    return S.Scene((0, 0, 0, 1), tree)


def open_squares():
    open_sq = S.cSubtract(S.shape([rect(5, 5)]), S.t_translate(1, 1, S.shape([rect(3, 3)])))
    items = [S.t_translate(2 + 6 * i, 2 + 3 * i, S.t_scale(1 + 0.5 * i, S.solid((1, 0.6, 0, 0.5), open_sq)))
             for i in range(4)]
    return S.Scene((1, 1, 1, 1), S.overlap(items))


def thin_rectangles(n=160):
    """More thin full-width rectangles than MAXSHAPE=127 allows per column."""
    cols = [(1, 0, 0, 1), (0, 1, 0, 1), (0, 0, 1, 1)]
    items = [S.t_translate(0, 0.35 * i, S.solid(cols[i % 3], S.shape([rect(61.5, 0.3)]))) for i in range(n)]
    return S.Scene((1, 1, 1, 1), S.overlap(items))


def textured():
    pict = S.Picture(G.noise_texture(seed=3, size=48))
    circle = S.segments_to_outline([S.curved(1, 0, 1, 1), S.curved(0, 1, -1, 1), S.curved(-1, 0, -1, -1),
                                    S.curved(0, -1, 1, -1)])
    ring = S.cSubtract(S.t_scale(20, S.shape([circle])), S.t_scale(9, S.shape([circle])))
    items = [
        S.t_translate(30, 26, S.texture_with("noise", ring)),
        S.t_translate(20, 30, S.t_scale(0.75, S.texture_with("noise", S.shape([rect(40, 20)])))),
        S.t_translate(5, 5, S.solid((0, 0, 1, 0.2), S.shape([rect(8, 200)]))),
    ]
    return S.Scene((1, 1, 1, 1), S.overlap(items), pictures={"noise": pict})


def radial():
    """Radial-gradient substance (new; not in the reference kernels)."""
    circle = S.segments_to_outline([S.curved(1, 0, 1, 1), S.curved(0, 1, -1, 1), S.curved(-1, 0, -1, -1),
                                    S.curved(0, -1, 1, -1)])
    items = [S.t_translate(32, 24, S.radial_with((0, 0), 18, (1, 0, 0, 1), (0, 0, 1, 0.5),
                                                 S.t_scale(20, S.shape([circle])))),
             S.t_translate(10, 10, S.radial_with((5, 5), 7, (0, 1, 0, 0.8), (1, 1, 0, 1), S.shape([rect(20, 12)])))]
    return S.Scene((1, 1, 1, 1), S.overlap(items))


def spec_small(**kw):
    d = dict(max_tile_size=16, threads_per_tile=16, max_thresholds=512, max_shape=127, stack_sections=8)
    d.update(kw)
    return L.make_spec(**d)


# name -> (builder, width, height, spec, reference-comparable)
SCENES = {
    "tiny_square": (tiny_square, 8, 8, spec_small(max_tile_size=8, threads_per_tile=8), True),
    "knob": (knob, 24, 28, spec_small(), True),
    "hourglass": (hourglass, 20, 18, spec_small(), True),
    "six_point_rectangle": (six_point_rectangle, 24, 16, spec_small(threads_per_tile=64), True),
    "two_brackets": (two_brackets, 16, 16, spec_small(), True),
    "open_squares": (open_squares, 48, 40, spec_small(max_tile_size=32, threads_per_tile=32), True),
    "thin_rectangles": (thin_rectangles, 64, 60, spec_small(max_tile_size=32, threads_per_tile=32), True),
    "textured": (textured, 64, 56, spec_small(max_tile_size=32, threads_per_tile=64), True),
    "radial": (radial, 64, 48, spec_small(max_tile_size=32, threads_per_tile=32), False),
}

# seeded random scenes: (generator kwargs, spec kwargs)
RANDOM = {
    "random_128x96": (dict(seed=11, width=128, height=96, n_shapes=24),
                      dict(max_tile_size=32, threads_per_tile=32, max_thresholds=4096, max_shape=127,
                           stack_sections=8)),
    "random_odd_tiles": (dict(seed=12, width=100, height=70, n_shapes=40, seg_lo=3, seg_hi=12),
                         dict(max_tile_size=16, threads_per_tile=32, max_thresholds=256, max_shape=127,
                              stack_sections=8)),
    "random_512_cfg": (dict(seed=0, width=512, height=512, n_shapes=64),
                       dict(max_tile_size=32, threads_per_tile=32, max_thresholds=4096, max_shape=127,
                            stack_sections=8)),
}


def build(name):
    """Serialized frame of a named fixture scene."""
    if name in SCENES:
        fn, w, h, spec, _ = SCENES[name]
        return S.serialize(fn(), w, h, spec)
    gen, sk = RANDOM[name]
    return S.serialize_flat(G.random_shapes(**gen), L.make_spec(**sk))


def reference_comparable(name) -> bool:
    return RANDOM.get(name) is not None or SCENES[name][4]


ALL = list(SCENES) + list(RANDOM)
