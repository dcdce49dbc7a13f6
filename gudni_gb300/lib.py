"""ctypes bindings of the package's C ABI (include/gudni_cuda.h, include/gudni_serialize.h)
and numpy dtypes of the reference-compatible records."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

# ------------------------------------------------------------------ records
SHAPE_DTYPE = np.dtype([("tag", "<u8"), ("geo_start", "<u4"), ("num_strands", "<u4")])
TILE_DTYPE = np.dtype([("left", "<i4"), ("top", "<i4"), ("right", "<i4"), ("bottom", "<i4"),
                       ("hdepth", "<i2"), ("vdepth", "<i2"), ("column_allocation", "<i4"),
                       ("shape_start", "<u4"), ("shape_length", "<u4")])
PICTURE_USE_DTYPE = np.dtype([("translate_x", "<f4"), ("translate_y", "<f4"), ("size_x", "<i4"),
                              ("size_y", "<i4"), ("mem_offset", "<i4"), ("scale", "<f4")])
RADIAL_DTYPE = np.dtype([("center_x", "<f4"), ("center_y", "<f4"), ("radius", "<f4"),
                         ("pad", "<f4"), ("inner", "<f4", (4,)), ("outer", "<f4", (4,))])
assert SHAPE_DTYPE.itemsize == 16 and TILE_DTYPE.itemsize == 32
assert PICTURE_USE_DTYPE.itemsize == 24 and RADIAL_DTYPE.itemsize == 48

RANDOM_FIELD_SIZE = 4096

TAG_SUBSTANCE_MASK = 0xC000000000000000
TAG_SOLID = 0x8000000000000000
TAG_PICTURE = 0x4000000000000000
TAG_RADIAL = 0xC000000000000000
TAG_COMPOUND_MASK = 0x3000000000000000
TAG_ADD = 0x2000000000000000
TAG_SUBTRACT = 0x3000000000000000
TAG_ID_MASK = 0x0FFFFFFFFFFFFFFF

STATUS = {
    0: "ok", -1: "bad input", -2: "threshold overflow", -3: "iteration limit",
    -4: "CUDA error", -5: "no device", -6: "not ready", -7: "out of memory",
}


class Spec(C.Structure):
    """gudni_spec: the reference's RasterSpec plus its compile-time knobs."""
    _fields_ = [("max_tile_size", C.c_int32), ("threads_per_tile", C.c_int32),
                ("max_strands_per_tile", C.c_int32), ("max_tiles_per_call", C.c_int32),
                ("max_thresholds", C.c_int32), ("max_shape", C.c_int32),
                ("stack_sections", C.c_int32), ("stochastic_factor", C.c_float)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def make_spec(max_tile_size=32, threads_per_tile=None, max_thresholds=1024, max_shape=127,
              stack_sections=None, max_tiles_per_call=1024, max_strands_per_tile=None,
              stochastic_factor=0.0) -> Spec:
    """Build a spec; defaults follow the reference (threads per tile = tile size,
    max strands per tile = max thresholds - 2, OpenCL/Setup.hs:71-87)."""
    if threads_per_tile is None:
        threads_per_tile = max_tile_size
    if stack_sections is None:
        stack_sections = max(1, -(-(max_shape + 1) // 64))
    if max_strands_per_tile is None:
        max_strands_per_tile = max_thresholds - 2
    return Spec(max_tile_size, threads_per_tile, max_strands_per_tile, max_tiles_per_call,
                max_thresholds, max_shape, stack_sections, stochastic_factor)


def compute_depth(threads_per_tile: int) -> int:
    """adjustedLog (Raster/TileTree.hs:74-75) of threads per tile."""
    d = 0
    while (1 << d) < threads_per_tile:
        d += 1
    return d


# ------------------------------------------------------------------ host library
class SceneDesc(C.Structure):
    _fields_ = [("canvas_w", C.c_int32), ("canvas_h", C.c_int32), ("background", C.c_float * 4),
                ("n_substances", C.c_int32),
                ("substance_kind", C.c_void_p), ("substance_color", C.c_void_p),
                ("substance_picture", C.c_void_p), ("substance_picture_xform", C.c_void_p),
                ("substance_radial", C.c_void_p), ("substance_shape_start", C.c_void_p),
                ("shape_compound", C.c_void_p), ("shape_outline_start", C.c_void_p),
                ("outline_pair_start", C.c_void_p), ("pairs", C.c_void_p),
                ("n_pictures", C.c_int32), ("picture_size", C.c_void_p),
                ("picture_offset", C.c_void_p)]


_host = None
_cuda = None


def load_host():
    """The host serializer library (built on first use)."""
    global _host
    if _host is None:
        path = _build.build_host()
        lib = C.CDLL(path)
        lib.gudni_serialize.restype = C.c_void_p
        lib.gudni_serialize.argtypes = [C.POINTER(SceneDesc), C.POINTER(Spec)]
        lib.gudni_serialize_parallel.restype = C.c_void_p
        lib.gudni_serialize_parallel.argtypes = [C.POINTER(SceneDesc), C.POINTER(Spec), C.c_int]
        lib.gudni_serialize_error.restype = C.c_char_p
        lib.gudni_frame_free.argtypes = [C.c_void_p]
        for name in ("geometry_bytes", "n_substances", "n_picture_uses", "n_radials", "n_jobs"):
            fn = getattr(lib, "gudni_frame_" + name)
            fn.restype = C.c_size_t
            fn.argtypes = [C.c_void_p]
        for name in ("geometry", "substances", "picture_uses", "radials"):
            fn = getattr(lib, "gudni_frame_" + name)
            fn.restype = C.c_void_p
            fn.argtypes = [C.c_void_p]
        for name in ("job_n_shapes", "job_n_tiles"):
            fn = getattr(lib, "gudni_frame_" + name)
            fn.restype = C.c_size_t
            fn.argtypes = [C.c_void_p, C.c_size_t]
        for name in ("job_shapes", "job_tiles"):
            fn = getattr(lib, "gudni_frame_" + name)
            fn.restype = C.c_void_p
            fn.argtypes = [C.c_void_p, C.c_size_t]
        lib.gudni_frame_job_columns.restype = C.c_int32
        lib.gudni_frame_job_columns.argtypes = [C.c_void_p, C.c_size_t]
        lib.gudni_frame_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        lib.gudni_frame_n_points.restype = C.c_size_t
        lib.gudni_frame_n_points.argtypes = [C.c_void_p]
        for name in ("point_offsets", "point_sources", "point_weights"):
            fn = getattr(lib, "gudni_frame_" + name)
            fn.restype = C.c_void_p
            fn.argtypes = [C.c_void_p]
        _host = lib
    return _host


def _copy(ptr, count, dtype) -> np.ndarray:
    dtype = np.dtype(dtype)
    if count == 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    buf = (C.c_uint8 * (count * dtype.itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype).copy()  # one copy, out of the library's memory


# ------------------------------------------------------------------ CUDA library
class DeviceFrame(C.Structure):
    """gudni_device_frame: a frame serialized on the device (its piles stay there)."""
    _fields_ = [("geometry_bytes", C.c_size_t), ("n_strands", C.c_size_t), ("n_shapes", C.c_size_t),
                ("n_tiles", C.c_size_t), ("n_jobs", C.c_size_t), ("stats", C.c_int64 * 8),
                ("geometry", C.c_void_p), ("shapes", C.c_void_p), ("tiles", C.c_void_p),
                ("tile_jobs", C.c_void_p), ("n_points", C.c_size_t), ("point_offsets", C.c_void_p),
                ("point_sources", C.c_void_p), ("point_weights", C.c_void_p)]


SERIALIZE_PROVENANCE = 1
RANDOM_FIELD, RANDOM_COUNTER = 0, 1  # gudni_set_random_source


class JobDesc(C.Structure):
    """gudni_job_desc."""
    _fields_ = [("shapes", C.c_void_p), ("n_shapes", C.c_size_t), ("tiles", C.c_void_p),
                ("n_tiles", C.c_size_t), ("columns_to_alloc", C.c_int32)]


def cuda_library_path() -> str:
    return _build.CUDA_LIB


def load_cuda(build_if_missing: bool = True):
    """The CUDA raster library.  Raises if it is not built or cannot load: there is
    no CPU fallback for the raster path."""
    global _cuda
    if _cuda is not None:
        return _cuda
    path = _build.CUDA_LIB
    if build_if_missing:
        path = _build.build_cuda()
    if not os.path.isfile(path):
        raise RuntimeError(f"CUDA raster library missing: {path} (run __graft_entry__.build())")
    lib = C.CDLL(path)
    vp, sz, i32 = C.c_void_p, C.c_size_t, C.c_int32
    lib.gudni_create.restype = vp
    lib.gudni_create.argtypes = [C.POINTER(Spec), C.c_int]
    lib.gudni_destroy.argtypes = [vp]
    lib.gudni_last_error.restype = C.c_char_p
    lib.gudni_last_error.argtypes = [vp]
    lib.gudni_upload_common.restype = C.c_int
    lib.gudni_upload_common.argtypes = [vp, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp]
    lib.gudni_upload_pictures.restype = C.c_int
    lib.gudni_upload_pictures.argtypes = [vp, vp, sz]
    lib.gudni_upload_random_field.restype = C.c_int
    lib.gudni_upload_random_field.argtypes = [vp, vp]
    lib.gudni_upload_frame.restype = C.c_int
    lib.gudni_upload_frame.argtypes = [vp, vp, sz, vp, sz, vp, sz, vp, sz]
    lib.gudni_set_device_strand_table.restype = C.c_int
    lib.gudni_set_device_strand_table.argtypes = [vp, C.c_int]
    lib.gudni_set_random_source.restype = C.c_int
    lib.gudni_set_random_source.argtypes = [vp, C.c_int, C.c_uint64]
    lib.gudni_serialize_device.restype = C.c_int
    lib.gudni_serialize_device.argtypes = [vp, C.POINTER(SceneDesc), C.c_int, C.POINTER(DeviceFrame)]
    lib.gudni_device_frame_download.restype = C.c_int
    lib.gudni_device_frame_download.argtypes = [vp, C.POINTER(DeviceFrame), vp, vp, vp, vp, vp, vp, vp]
    job_args = [vp, vp, sz, vp, sz, i32, i32, i32, i32, i32, i32, vp, vp]
    lib.gudni_raster_job.restype = C.c_int
    lib.gudni_raster_job.argtypes = job_args
    lib.gudni_raster_job_device.restype = C.c_int
    lib.gudni_raster_job_device.argtypes = job_args + [vp]
    lib.gudni_sync_status.restype = C.c_int
    lib.gudni_sync_status.argtypes = [vp]
    lib.gudni_scratch_bytes.restype = sz
    lib.gudni_scratch_bytes.argtypes = [vp]
    lib.gudni_raster_frame.restype = C.c_int
    lib.gudni_raster_frame.argtypes = [vp, C.POINTER(JobDesc), sz, i32, i32, i32, i32, vp, vp]
    lib.gudni_raster_tiles_device.restype = C.c_int
    lib.gudni_raster_tiles_device.argtypes = [vp, vp, sz, vp, vp, sz, i32, i32, i32, i32, vp, vp, vp]
    lib.gudni_enable_counters.restype = C.c_int
    lib.gudni_enable_counters.argtypes = [vp, C.c_int]
    lib.gudni_read_counters.restype = C.c_int
    lib.gudni_read_counters.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.gudni_set_dense_columns.restype = C.c_int
    lib.gudni_set_dense_columns.argtypes = [vp, i32]
    lib.gudni_set_cooperative_units.restype = C.c_int
    lib.gudni_set_cooperative_units.argtypes = [vp, C.c_int]
    lib.gudni_set_adjoint_regenerate.restype = C.c_int
    lib.gudni_set_adjoint_regenerate.argtypes = [vp, C.c_int]
    lib.gudni_launch_count.restype = C.c_uint64
    lib.gudni_launch_count.argtypes = [vp]
    lib.gudni_adjoint_tiles_device.restype = C.c_int
    lib.gudni_adjoint_tiles_device.argtypes = [vp, vp, sz, vp, vp, sz, i32, i32, i32, vp, vp, vp, vp, vp, vp]
    lib.gudni_batch_adjoint.restype = C.c_int
    lib.gudni_batch_adjoint.argtypes = [vp, vp, vp, vp, vp, vp]
    _cuda = lib
    return lib


CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the runtime's handle for the legacy default stream


def current_stream_handle() -> int:
    """torch's current CUDA stream as a handle the C ABI can take.  A null stream
    argument means the context's own (non-blocking) stream there, so torch's legacy
    default stream, whose handle is 0, is passed as cudaStreamLegacy instead."""
    import torch
    return torch.cuda.current_stream().cuda_stream or CUDA_STREAM_LEGACY


def ptr(a) -> int | None:
    """Address of a numpy array's data (None for an empty array)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data if a.size else None
    return a
