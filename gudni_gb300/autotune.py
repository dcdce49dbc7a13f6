"""Autotuner for the batched raster form: picks tile size and threads per tile per
canvas-size bucket by timing candidate specs on sample scenes of the bucket.

The spec changes the arithmetic (each column computes in coordinates relative to its
own slab), so parity is always checked against the oracle run with the same spec the
autotuner chose.  There is no counterpart in the reference, whose tile size and
threads per tile both equal the device's maximum work-group size (OpenCL/Setup.hs:
81-83).
"""
from __future__ import annotations

import time
from typing import Dict, List, Sequence, Tuple

from . import batch as B
from . import lib as L
from . import scene as S

# (tile size, threads per tile); threads per tile must be >= tile size.  More threads
# per tile make shorter columns (more parallel work, more threshold generation; an
# 8-pixel tile with 64 threads has one-pixel columns); smaller tiles give each column
# fewer shapes.
CANDIDATES: Tuple[Tuple[int, int], ...] = ((8, 32), (8, 64), (16, 64), (32, 256))
BUCKETS: Tuple[int, ...] = (96, 192, 384, 768, 1 << 30)  # upper bound of max(canvas side)


def bucket_of(w: int, h: int) -> int:
    side = max(w, h)
    for i, b in enumerate(BUCKETS):
        if side <= b:
            return i
    return len(BUCKETS) - 1


def spec_for(tile: int, tpt: int, max_shape: int, max_thresholds: int, strands_per_tile: int) -> L.Spec:
    return L.make_spec(max_tile_size=tile, threads_per_tile=tpt, max_thresholds=max_thresholds,
                       max_shape=max_shape, max_strands_per_tile=strands_per_tile)


def scene_cost(f: S.FlatScene) -> float:
    """A rough work estimate: pixels x shapes."""
    return float(f.canvas_w) * float(f.canvas_h) * float(len(f.substance_kind))


def autotune(flats: Sequence[S.FlatScene], max_shape: int, max_thresholds: int, strands_per_tile: int,
             samples: int = 2, reps: int = 3, candidates=CANDIDATES, device: int = 0,
             log=None, dense_columns: int = 0) -> Dict[int, Tuple[int, int]]:
    """Return {bucket: (tile, threads_per_tile)}.  Each candidate renders the bucket's
    sample scenes (its median and, with samples > 1, its most expensive scene by
    scene_cost) as one batch; the fastest mean over `reps` replays wins.  A candidate
    whose first render is over three times the best so far is not replayed.  The
    candidates are timed with the warp-cooperative dense-column threshold the batch
    will render with (`dense_columns`, gudni_set_dense_columns)."""
    by_bucket: Dict[int, List[S.FlatScene]] = {}
    for f in flats:
        by_bucket.setdefault(bucket_of(f.canvas_w, f.canvas_h), []).append(f)
    choice: Dict[int, Tuple[int, int]] = {}
    base = spec_for(32, 32, max_shape, max_thresholds, strands_per_tile)
    with B.BatchRasterizer(base, device) as r:
        if dense_columns:
            r.set_dense_columns(dense_columns)
        for b, members in sorted(by_bucket.items()):
            ranked = sorted(members, key=scene_cost)
            picks = [ranked[len(ranked) // 2]] + ([ranked[-1]] if samples > 1 and len(ranked) > 1 else [])
            best = None
            for tile, tpt in candidates:
                spec = spec_for(tile, tpt, max_shape, max_thresholds, strands_per_tile)
                batch = B.build_batch([S.serialize_flat(f, spec) for f in picks])
                r.upload(batch)
                t0 = time.perf_counter()
                r.render(use_graph=False)
                r.sync_status()
                dt = time.perf_counter() - t0
                if best is None or dt < 3.0 * best[0]:
                    t0 = time.perf_counter()
                    for _ in range(reps):
                        r.render(use_graph=False)
                    r.sync_status()
                    dt = (time.perf_counter() - t0) / reps
                if log:
                    log(f"bucket {b} tile {tile} tpt {tpt}: {dt * 1e3:.3f} ms")
                if best is None or dt < best[0]:
                    best = (dt, (tile, tpt))
            choice[b] = best[1]
    return choice


def serialize_tuned(flats: Sequence[S.FlatScene], choice: Dict[int, Tuple[int, int]], max_shape: int,
                    max_thresholds: int, strands_per_tile: int) -> List[S.Frame]:
    frames = []
    for f in flats:
        tile, tpt = choice.get(bucket_of(f.canvas_w, f.canvas_h), (32, 32))
        frames.append(S.serialize_flat(f, spec_for(tile, tpt, max_shape, max_thresholds, strands_per_tile)))
    return frames
