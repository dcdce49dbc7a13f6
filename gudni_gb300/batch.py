"""Batched rendering: many scenes of uneven size in one persistent launch.

A Batch concatenates serialized frames (each with its own raster spec) into one set
of piles, rebasing every cross-reference:
  * shape geo_start by the frame's offset in the geometry pile (16-byte units),
  * the substance id in every shape tag by the frame's offset in the substance pile,
  * picture / gradient ids held in texture and gradient substances by the frame's
    offset in the picture-use / gradient piles, picture-use byte offsets by the
    frame's offset in the picture pile,
  * tile shape slices by the job's offset in the concatenated shape pile.
Every (frame, job) pair becomes one scene record (canvas, output offset, background,
threads per tile, job index); tiles carry their scene index and an estimated cost
used to schedule the most expensive tiles first.

BatchRasterizer uploads a batch once and renders it through gudni_batch_render,
optionally replaying a captured CUDA graph.  There is no counterpart in the
reference, which renders one scene per frame.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List

import numpy as np

from . import lib as L
from .raster import Rasterizer

BATCH_SCENE_DTYPE = np.dtype([("bitmap_w", "<i4"), ("bitmap_h", "<i4"), ("compute_depth", "<i4"),
                              ("job_index", "<i4"), ("out_offset", "<u8"), ("background", "<f4", (4,))])
assert BATCH_SCENE_DTYPE.itemsize == 40


@dataclass
class Batch:
    geometry: np.ndarray
    substances: np.ndarray
    pictures: np.ndarray
    picture_uses: np.ndarray
    radials: np.ndarray
    shapes: np.ndarray
    tiles: np.ndarray
    tile_scene: np.ndarray
    tile_cost: np.ndarray
    scenes: np.ndarray
    out_pixels: int
    frames: list              # the source frames
    frame_offsets: np.ndarray  # first output pixel of each frame
    frame_tiles: list          # (first tile, tile count) of each frame
    frame_geo_offsets: np.ndarray = None  # first byte of each frame in the geometry pile
    frame_sub_offsets: np.ndarray = None  # first substance of each frame

    def images(self, out: np.ndarray) -> List[np.ndarray]:
        """Split the batch output into per-frame (H, W) images."""
        res = []
        for f, off in zip(self.frames, self.frame_offsets):
            n = f.canvas_w * f.canvas_h
            res.append(out[off:off + n].reshape(f.canvas_h, f.canvas_w))
        return res


def _tile_costs(frame, job) -> np.ndarray:
    """Estimated work per tile: (strands + shapes of the tile) x its pixels."""
    strands = job.shapes["num_strands"].astype(np.int64)
    cum = np.concatenate([[0], np.cumsum(strands)])
    start = job.tiles["shape_start"].astype(np.int64)
    length = job.tiles["shape_length"].astype(np.int64)
    tile_strands = cum[start + length] - cum[start]
    w = np.minimum(job.tiles["right"], frame.canvas_w) - np.minimum(job.tiles["left"], frame.canvas_w)
    h = np.minimum(job.tiles["bottom"], frame.canvas_h) - np.minimum(job.tiles["top"], frame.canvas_h)
    pixels = np.maximum(w, 0).astype(np.int64) * np.maximum(h, 0).astype(np.int64)
    return ((tile_strands + length) * pixels).astype(np.float32)


def build_batch(frames) -> Batch:
    geo, subs, pics, uses, rads = [], [], [], [], []
    shapes, tiles, tile_scene, costs, scenes = [], [], [], [], []
    geo_off = sub_off = pic_off = use_off = rad_off = shape_off = out_off = 0
    frame_offsets, frame_tiles, frame_geo, frame_sub = [], [], [], []
    tile_count = 0
    for fi, f in enumerate(frames):
        if f.geometry.size % 16:
            raise ValueError("geometry pile must be a multiple of 16 bytes")
        geo.append(f.geometry)
        # substance kinds from the tags that reference them
        s = f.substances.copy()
        su = s.view(np.uint32).reshape(-1, 4)
        kinds = np.zeros(len(s), np.uint64)
        for job in f.jobs:
            t = job.shapes["tag"]
            kinds[(t & np.uint64(L.TAG_ID_MASK)).astype(np.int64)] = t & np.uint64(L.TAG_SUBSTANCE_MASK)
        pic_sub = kinds == np.uint64(L.TAG_PICTURE)
        rad_sub = kinds == np.uint64(L.TAG_RADIAL)
        su[pic_sub, 0] += np.uint32(use_off)
        su[rad_sub, 0] += np.uint32(rad_off)
        subs.append(s)
        u = f.picture_uses.copy()
        u["mem_offset"] += np.int32(pic_off)
        uses.append(u)
        rads.append(f.radials)
        pics.append(f.pictures)
        frame_offsets.append(out_off)
        frame_geo.append(geo_off)
        frame_sub.append(sub_off)
        first_tile = tile_count
        for ji, job in enumerate(f.jobs):
            sh = job.shapes.copy()
            sh["geo_start"] += np.uint32(geo_off // 16)
            tag = sh["tag"]
            sh["tag"] = (tag & ~np.uint64(L.TAG_ID_MASK)) | ((tag & np.uint64(L.TAG_ID_MASK)) + np.uint64(sub_off))
            shapes.append(sh)
            tl = job.tiles.copy()
            tl["shape_start"] += np.uint32(shape_off)
            tiles.append(tl)
            scene_index = len(scenes)
            tile_scene.append(np.full(len(tl), scene_index, np.int32))
            costs.append(_tile_costs(f, job))
            rec = np.zeros(1, BATCH_SCENE_DTYPE)
            rec["bitmap_w"], rec["bitmap_h"] = f.canvas_w, f.canvas_h
            rec["compute_depth"] = f.compute_depth
            rec["job_index"] = ji
            rec["out_offset"] = out_off
            rec["background"] = f.background
            scenes.append(rec)
            shape_off += len(sh)
            tile_count += len(tl)
        frame_tiles.append((first_tile, tile_count - first_tile))
        geo_off += f.geometry.size
        sub_off += len(f.substances)
        pic_off += f.pictures.size
        use_off += len(f.picture_uses)
        rad_off += len(f.radials)
        out_off += f.canvas_w * f.canvas_h
    cat = lambda xs, dt: np.concatenate(xs) if xs else np.zeros(0, dt)  # noqa: E731
    return Batch(
        geometry=cat(geo, np.uint8), substances=np.concatenate(subs).reshape(-1, 4).astype(np.float32),
        pictures=cat(pics, np.uint8), picture_uses=cat(uses, L.PICTURE_USE_DTYPE),
        radials=cat(rads, L.RADIAL_DTYPE), shapes=cat(shapes, L.SHAPE_DTYPE), tiles=cat(tiles, L.TILE_DTYPE),
        tile_scene=cat(tile_scene, np.int32), tile_cost=cat(costs, np.float32),
        scenes=np.concatenate(scenes) if scenes else np.zeros(0, BATCH_SCENE_DTYPE), out_pixels=int(out_off),
        frames=list(frames), frame_offsets=np.asarray(frame_offsets, np.int64), frame_tiles=frame_tiles,
        frame_geo_offsets=np.asarray(frame_geo, np.int64), frame_sub_offsets=np.asarray(frame_sub, np.int64))


def bind(lib) -> None:
    """Declare the batch entry points' signatures on the CUDA library."""
    vp, sz = C.c_void_p, C.c_size_t
    lib.gudni_batch_upload.restype = C.c_int
    lib.gudni_batch_upload.argtypes = [vp, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, vp, vp, sz, vp,
                                       sz, sz]
    lib.gudni_batch_render.restype = C.c_int
    lib.gudni_batch_render.argtypes = [vp, C.c_int, vp]
    lib.gudni_batch_render_tiles.restype = C.c_int
    lib.gudni_batch_render_tiles.argtypes = [vp, sz, sz, vp]
    lib.gudni_batch_output.restype = vp
    lib.gudni_batch_output.argtypes = [vp]
    lib.gudni_batch_download.restype = C.c_int
    lib.gudni_batch_download.argtypes = [vp, vp]


class BatchRasterizer(Rasterizer):
    """A Rasterizer that holds one uploaded batch."""

    def __init__(self, spec: L.Spec, device: int = 0):
        super().__init__(spec, device)
        bind(self.lib)
        self.batch = None

    def upload(self, batch: Batch, schedule: bool = True) -> None:
        self._keep = [batch.geometry, batch.substances, batch.pictures, batch.picture_uses, batch.radials,
                      batch.shapes, batch.tiles, batch.tile_scene, batch.tile_cost, batch.scenes]
        self._check(self.lib.gudni_batch_upload(
            self.ctx, L.ptr(batch.geometry), batch.geometry.size, L.ptr(batch.substances), len(batch.substances),
            L.ptr(batch.pictures), batch.pictures.size, L.ptr(batch.picture_uses), len(batch.picture_uses),
            L.ptr(batch.radials), len(batch.radials), L.ptr(batch.shapes), len(batch.shapes), L.ptr(batch.tiles),
            L.ptr(batch.tile_scene), L.ptr(batch.tile_cost) if schedule else None, len(batch.tiles),
            L.ptr(batch.scenes), len(batch.scenes), batch.out_pixels))
        self.batch = batch

    def render(self, use_graph: bool = True, stream: int = 0) -> None:
        self._check(self.lib.gudni_batch_render(self.ctx, 1 if use_graph else 0, stream or None))

    def render_tiles(self, first: int, count: int, stream: int = 0) -> None:
        self._check(self.lib.gudni_batch_render_tiles(self.ctx, first, count, stream or None))

    def render_each_scene(self, stream: int = 0) -> None:
        """The plain path: one launch pair per frame of the batch, in order."""
        for first, count in self.batch.frame_tiles:
            self.render_tiles(first, count, stream)

    def output_ptr(self) -> int:
        return int(self.lib.gudni_batch_output(self.ctx))

    def download(self) -> np.ndarray:
        out = np.zeros(self.batch.out_pixels, np.uint32)
        self._check(self.lib.gudni_batch_download(self.ctx, out.ctypes.data))
        return out

    def render_images(self, use_graph: bool = True) -> List[np.ndarray]:
        self.render(use_graph)
        return self.batch.images(self.download())

    def adjoint(self, target, image, grad_geometry, grad_substances, stream: int = 0) -> None:
        """Enqueue the adjoint of every scene of the batch in one launch
        (gudni_batch_adjoint) on `stream` (0: torch's current stream).  All four are
        device tensors: target and image
        (out_pixels, 4) float32 at the scenes' output offsets, grad_geometry
        (geometry bytes / 4,) and grad_substances (n_substances, 4) float32, ADDED to."""
        import torch
        b = self.batch
        for t, shape in ((target, (b.out_pixels, 4)), (image, (b.out_pixels, 4)),
                         (grad_geometry, (b.geometry.size // 4,)), (grad_substances, (len(b.substances), 4))):
            assert t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and tuple(t.shape) == shape
        if not stream:
            stream = L.current_stream_handle()
        self._check(self.lib.gudni_batch_adjoint(self.ctx, target.data_ptr(), image.data_ptr(),
                                                 grad_geometry.data_ptr(), grad_substances.data_ptr(),
                                                 stream or None))

    def frame_slices(self, i: int):
        """(geometry float slice, substance slice) of frame i in the batch gradients."""
        b = self.batch
        f = b.frames[i]
        g0 = int(b.frame_geo_offsets[i]) // 4
        s0 = int(b.frame_sub_offsets[i])
        return slice(g0, g0 + f.geometry.size // 4), slice(s0, s0 + len(f.substances))
