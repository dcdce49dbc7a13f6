"""Host-side mirror of the reference's OpenCL dispatch, over the CUDA C ABI.

  Rasterizer(spec)           setupOpenCL        (OpenCL/Setup.hs:102-147)
  Rasterizer.upload_common   BuffersInCommon    (OpenCL/CallKernels.hs:208-240)
  Rasterizer.upload_pictures / upload_random_field / upload_frame
                             the same buffers split into a resident part (pictures,
                             random field) and a per-frame part
  Rasterizer.serialize_device the host serializer's piles built by kernels
  Rasterizer.raster_job      raster/generateCall (OpenCL/CallKernels.hs:88-206)
  Rasterizer.queue_jobs      queueRasterJobs    (OpenCL/CallKernels.hs:218-242)

Every call goes through libgudni_cuda.so; there is no CPU path.  If the library is
missing or no CUDA device is present, construction raises.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import lib as L


class RasterError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{L.STATUS.get(code, code)}: {message}")
        self.code = code


class Rasterizer:
    def __init__(self, spec: L.Spec, device: int = 0):
        self.lib = L.load_cuda()
        self.spec = spec
        self._spec_ref = L.Spec(*[getattr(spec, f) for f, _ in L.Spec._fields_])
        h = self.lib.gudni_create(C.byref(self._spec_ref), device)
        if not h:
            raise RuntimeError("gudni_create failed: " + self.lib.gudni_last_error(None).decode())
        self.ctx = h

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.gudni_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc != 0:
            raise RasterError(rc, self.lib.gudni_last_error(self.ctx).decode())

    def upload_common(self, frame) -> None:
        rf = frame.random_field if frame.random_field is not None else None
        self._check(self.lib.gudni_upload_common(
            self.ctx, L.ptr(frame.geometry), frame.geometry.size, L.ptr(frame.substances),
            len(frame.substances), L.ptr(frame.pictures), frame.pictures.size, L.ptr(frame.picture_uses),
            len(frame.picture_uses), L.ptr(frame.radials), len(frame.radials), L.ptr(rf)))

    def upload_pictures(self, pictures) -> None:
        """Upload a picture pile that stays on the device across frames
        (gudni_upload_pictures): a scene.PictureLibrary or a uint8 array."""
        pile = np.ascontiguousarray(getattr(pictures, "pile", pictures), dtype=np.uint8)
        self._check(self.lib.gudni_upload_pictures(self.ctx, L.ptr(pile), pile.size))

    def upload_random_field(self, random_field: Optional[np.ndarray]) -> None:
        """Upload the random field kept across frames (None removes it)."""
        rf = None if random_field is None else np.ascontiguousarray(random_field, dtype=np.float32)
        if rf is not None and rf.size != L.RANDOM_FIELD_SIZE:
            raise ValueError(f"the random field holds {L.RANDOM_FIELD_SIZE} floats")
        self._check(self.lib.gudni_upload_random_field(self.ctx, L.ptr(rf)))

    def upload_frame(self, frame) -> None:
        """Upload a frame's own piles (gudni_upload_frame); its picture usages point
        into the resident picture pile (a frame serialized from
        PictureLibrary.bind)."""
        self._check(self.lib.gudni_upload_frame(
            self.ctx, L.ptr(frame.geometry), frame.geometry.size, L.ptr(frame.substances), len(frame.substances),
            L.ptr(frame.picture_uses), len(frame.picture_uses), L.ptr(frame.radials), len(frame.radials)))

    def raster_job(self, frame, job_index: int, out: np.ndarray, frame_number: int = 0) -> None:
        """Rasterize one job into the host bitmap `out` ((H, W) uint32)."""
        job = frame.jobs[job_index]
        assert out.dtype == np.uint32 and out.flags.c_contiguous and out.size == frame.canvas_w * frame.canvas_h
        bg = np.ascontiguousarray(frame.background, np.float32)
        self._check(self.lib.gudni_raster_job(
            self.ctx, L.ptr(job.shapes), len(job.shapes), L.ptr(job.tiles), len(job.tiles), job.columns,
            frame.canvas_w, frame.canvas_h, frame.compute_depth, frame_number, job_index, bg.ctypes.data,
            out.ctypes.data))

    def queue_jobs(self, frame, out: Optional[np.ndarray] = None, frame_number: int = 0,
                   upload: str = "common") -> np.ndarray:
        """Upload the common buffers and rasterize every job (host buffers).
        upload="frame" uploads only the frame's own piles and keeps the resident
        pictures and random field (upload_pictures / upload_random_field)."""
        if out is None:
            out = np.zeros((frame.canvas_h, frame.canvas_w), dtype=np.uint32)
        if upload == "frame":
            self.upload_frame(frame)
        elif upload == "common":
            self.upload_common(frame)
        else:
            raise ValueError(f"upload must be 'common' or 'frame', not {upload!r}")
        for j in range(len(frame.jobs)):
            self.raster_job(frame, j, out, frame_number)
        return out

    def raster_frame(self, frame, out: Optional[np.ndarray] = None, frame_number: int = 0,
                     upload_common: bool = True) -> np.ndarray:
        """All jobs of a frame in one launch (host buffers)."""
        if out is None:
            out = np.zeros((frame.canvas_h, frame.canvas_w), dtype=np.uint32)
        assert out.dtype == np.uint32 and out.flags.c_contiguous and out.size == frame.canvas_w * frame.canvas_h
        if upload_common:
            self.upload_common(frame)
        descs = (L.JobDesc * max(1, len(frame.jobs)))()
        for i, j in enumerate(frame.jobs):
            descs[i] = L.JobDesc(L.ptr(j.shapes), len(j.shapes), L.ptr(j.tiles), len(j.tiles), j.columns)
        bg = np.ascontiguousarray(frame.background, np.float32)
        self._check(self.lib.gudni_raster_frame(self.ctx, descs, len(frame.jobs), frame.canvas_w, frame.canvas_h,
                                                frame.compute_depth, frame_number, bg.ctypes.data, out.ctypes.data))
        return out

    def raster_tiles_device(self, frame, shapes_ptr: int, n_shapes: int, tiles_ptr: int, tile_jobs_ptr: int,
                            n_tiles: int, out_ptr: int, stream: int = 0, frame_number: int = 0) -> None:
        """Enqueue a whole frame whose concatenated piles are device-resident
        (scene.concatenated_piles layout).  `stream`: a CUDA stream handle; 0 means the
        context's own non-blocking stream (lib.current_stream_handle() gives torch's
        current stream, the legacy default stream included)."""
        bg = np.ascontiguousarray(frame.background, np.float32)
        self._check(self.lib.gudni_raster_tiles_device(
            self.ctx, shapes_ptr, n_shapes, tiles_ptr, tile_jobs_ptr or None, n_tiles, frame.canvas_w,
            frame.canvas_h, frame.compute_depth, frame_number, bg.ctypes.data, out_ptr, stream or None))

    def serialize_device(self, flat, provenance: bool = False) -> L.DeviceFrame:
        """Serialize a flattened scene (scene.FlatScene) on the device
        (gudni_serialize_device): the same piles as scene.serialize_flat, computed by
        kernels and kept on the device as this context's current frame, with the
        points' provenance when asked.  Its picture offsets point into the resident
        picture pile (upload_pictures)."""
        from . import scene as S
        desc, keep = S.scene_desc(flat)
        frame = L.DeviceFrame()
        flags = L.SERIALIZE_PROVENANCE if provenance else 0
        self._check(self.lib.gudni_serialize_device(self.ctx, C.byref(desc), flags, C.byref(frame)))
        del keep
        return frame

    def download_device_frame(self, frame: L.DeviceFrame) -> dict:
        """The piles of a device-serialized frame on the host: geometry, and shapes,
        tiles and tile_jobs in the concatenated layout (scene.concatenated_piles); with
        provenance also point_offsets, point_sources and point_weights."""
        out = {"geometry": np.empty(frame.geometry_bytes, np.uint8),
               "shapes": np.empty(frame.n_shapes, L.SHAPE_DTYPE),
               "tiles": np.empty(frame.n_tiles, L.TILE_DTYPE),
               "tile_jobs": np.empty(frame.n_tiles, np.int32),
               "point_offsets": np.empty(frame.n_points, np.uint32),
               "point_sources": np.empty((frame.n_points, 3), np.int32),
               "point_weights": np.empty((frame.n_points, 3), np.float32)}
        self._check(self.lib.gudni_device_frame_download(
            self.ctx, C.byref(frame), *[L.ptr(out[k]) for k in ("geometry", "shapes", "tiles", "tile_jobs",
                                                                 "point_offsets", "point_sources", "point_weights")]))
        return out

    def raster_device_frame(self, frame: L.DeviceFrame, canvas_w: int, canvas_h: int, background, out_ptr: int,
                            stream: int = 0, frame_number: int = 0) -> None:
        """Enqueue the render of a device-serialized frame into the device bitmap at
        `out_ptr` (canvas_h * canvas_w BGRA words)."""
        bg = np.ascontiguousarray(background, np.float32)
        self._check(self.lib.gudni_raster_tiles_device(
            self.ctx, frame.shapes, frame.n_shapes, frame.tiles, frame.tile_jobs, frame.n_tiles, canvas_w, canvas_h,
            L.compute_depth(self.spec.threads_per_tile), frame_number, bg.ctypes.data, out_ptr, stream or None))

    def enable_counters(self, on: bool = True) -> None:
        self._check(self.lib.gudni_enable_counters(self.ctx, 1 if on else 0))

    def set_device_strand_table(self, on: bool = True) -> None:
        """Build the strand table of later uploads on the device from the uploaded pile
        (gudni_set_device_strand_table) instead of on the host; the table is the same."""
        self._check(self.lib.gudni_set_device_strand_table(self.ctx, 1 if on else 0))

    def set_random_source(self, source: int, seed: int = 0) -> None:
        """Where the stochastic jitter comes from when the spec's stochastic_factor
        is not 0 (gudni_set_random_source): lib.RANDOM_FIELD (the reference's random
        field) or lib.RANDOM_COUNTER (a counter-based hash of seed, pixel and
        section)."""
        self._check(self.lib.gudni_set_random_source(self.ctx, int(source), int(seed)))

    def set_dense_columns(self, min_thresholds: int) -> None:
        """Scan columns whose queues hold at least `min_thresholds` thresholds with the
        whole warp (gudni_set_dense_columns); 0 keeps every column on its own lane.
        The image does not change."""
        self._check(self.lib.gudni_set_dense_columns(self.ctx, int(min_thresholds)))

    def set_cooperative_units(self, on: Optional[bool] = True) -> None:
        """Warp-cooperative work units (gudni_set_cooperative_units): True for every
        launch, False for none, None to let each launch choose.  A context starts with
        False."""
        self._check(self.lib.gudni_set_cooperative_units(self.ctx, -1 if on is None else (1 if on else 0)))

    def set_adjoint_regenerate(self, on: bool = True) -> None:
        """The adjoint's backward pass regenerates each column's thresholds
        (gudni_set_adjoint_regenerate) instead of scanning the forward pass's queue."""
        self._check(self.lib.gudni_set_adjoint_regenerate(self.ctx, 1 if on else 0))

    def read_counters(self) -> dict:
        c = (C.c_int64 * 4)()
        self._check(self.lib.gudni_read_counters(self.ctx, c))
        return {"sections": c[0], "texels": c[1], "thresholds": c[2], "max_shape_bits": c[3]}

    def launch_count(self) -> int:
        return int(self.lib.gudni_launch_count(self.ctx))

    def raster_job_device(self, frame, job_index: int, shapes_ptr: int, tiles_ptr: int, out_ptr: int,
                          stream: int = 0, frame_number: int = 0) -> None:
        """Enqueue one job with device-resident shapes/tiles/out (torch data_ptr()s) on
        `stream` (0: the context's own stream; see raster_tiles_device)."""
        job = frame.jobs[job_index]
        bg = np.ascontiguousarray(frame.background, np.float32)
        self._check(self.lib.gudni_raster_job_device(
            self.ctx, shapes_ptr, len(job.shapes), tiles_ptr, len(job.tiles), job.columns, frame.canvas_w,
            frame.canvas_h, frame.compute_depth, frame_number, job_index, bg.ctypes.data, out_ptr,
            stream or None))

    def sync_status(self) -> None:
        self._check(self.lib.gudni_sync_status(self.ctx))

    def scratch_bytes(self) -> int:
        return int(self.lib.gudni_scratch_bytes(self.ctx))


def bgra_to_rgb(words: np.ndarray) -> np.ndarray:
    """(H, W) BGRA words -> (H, W, 3) uint8 RGB."""
    b = (words & 0xFF).astype(np.uint8)
    g = ((words >> 8) & 0xFF).astype(np.uint8)
    r = ((words >> 16) & 0xFF).astype(np.uint8)
    return np.stack([r, g, b], axis=-1)
