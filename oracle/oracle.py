"""ORACLE -- test infrastructure only.

Python driver of the CPU restatement of gudni's raster kernels
(oracle/raster_oracle.cpp) and of the reference's own Kernels.cl compiled for the CPU
(oracle/_ref/, made by oracle/build_ref.py when the reference checkout is present).

Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module,
and only as the checker / baseline: the product path never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgudni_oracle.so")
SRC = os.path.join(HERE, "raster_oracle.cpp")
HDR = os.path.join(ROOT, "include", "gudni_cuda.h")


ADJ_SRC = os.path.join(HERE, "adjoint_oracle.cpp")


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [SRC, ADJ_SRC]
    if force or not os.path.isfile(LIB) or max(os.path.getmtime(p) for p in srcs + [HDR]) > os.path.getmtime(LIB):
        cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-strict-aliasing", "-fopenmp",
               "-fPIC", "-shared"] + srcs + ["-o", LIB]
        subprocess.run(cmd, check=True)
    return LIB


class OracleStats(C.Structure):
    _fields_ = [("max_queue", C.c_int64), ("thresholds", C.c_int64), ("sections", C.c_int64),
                ("max_shape_bits", C.c_int64), ("overflow", C.c_int64)]


_lib = None
_ref_libs: dict = {}


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        vp = C.c_void_p
        lib.oracle_raster_job.restype = C.c_int
        lib.oracle_raster_job.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_float,
                                          vp, C.c_int, C.POINTER(OracleStats)]
        sz = C.c_size_t
        lib.oracle_adjoint_job.restype = C.c_int
        lib.oracle_adjoint_job.argtypes = [vp, sz, vp, sz, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_int, vp, C.c_int, C.c_int, vp, vp, vp, vp, C.c_int]
        lib.oracle_set_random_source.restype = None
        lib.oracle_set_random_source.argtypes = [C.c_int, C.c_uint64]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data if (a is not None and a.size) else None


def render_frame(frame, n_threads: int = 0, max_thresholds: Optional[int] = None,
                 stats: Optional[dict] = None, random_source: int = 0, random_seed: int = 0) -> np.ndarray:
    """Rasterize a serialized frame on the CPU; returns (H, W) uint32 BGRA words.
    Pixels no job writes stay 0.  random_source 1 takes the stochastic jitter from the
    counter-based hash with `random_seed` instead of the random field."""
    lib = _load()
    lib.oracle_set_random_source(int(random_source), int(random_seed))
    spec = frame.spec
    out = np.zeros((frame.canvas_h, frame.canvas_w), dtype=np.uint32)
    maxt = max_thresholds or spec.max_thresholds
    agg = {"max_queue": 0, "thresholds": 0, "sections": 0, "max_shape_bits": 0, "overflow": 0}
    bg = np.ascontiguousarray(frame.background, dtype=np.float32)
    for ji, job in enumerate(frame.jobs):
        st = OracleStats()
        lib.oracle_raster_job(_p(frame.geometry), _p(frame.substances), _p(frame.pictures), _p(frame.picture_uses),
                              _p(frame.radials), _p(frame.random_field), _p(job.shapes), _p(job.tiles),
                              len(job.tiles), spec.threads_per_tile, frame.compute_depth, frame.canvas_w,
                              frame.canvas_h, 0, ji, _p(bg), maxt, spec.max_shape, spec.stack_sections,
                              spec.stochastic_factor, _p(out), n_threads, C.byref(st))
        agg["max_queue"] = max(agg["max_queue"], st.max_queue)
        agg["thresholds"] += st.thresholds
        agg["sections"] += st.sections
        agg["max_shape_bits"] = max(agg["max_shape_bits"], st.max_shape_bits)
        agg["overflow"] |= st.overflow
    if stats is not None:
        stats.update(agg)
    return out


def ref_available(max_shape: int = 127, sections: int = 8, stochastic: float = 0.0) -> bool:
    from . import build_ref
    return (os.path.isfile(build_ref.library_name(max_shape, sections, stochastic))
            or os.path.isfile(build_ref.source_name(max_shape, sections, stochastic))
            or os.path.isfile(os.path.join(build_ref.DEFAULT_REFERENCE, build_ref.KERNELS_REL)))


def _load_ref(max_shape: int, sections: int, stochastic: float = 0.0):
    key = (max_shape, sections, stochastic)
    if key not in _ref_libs:
        from . import build_ref
        path = build_ref.build(max_shape=max_shape, sections=sections, stochastic=stochastic)
        if path is None or not os.path.isfile(path):
            raise FileNotFoundError("reference kernels not built (no reference checkout)")
        lib = C.CDLL(path)
        vp, sz = C.c_void_p, C.c_size_t
        lib.gudni_ref_raster_job.restype = C.c_int
        lib.gudni_ref_raster_job.argtypes = [vp, sz, vp, sz, vp, sz, vp, sz, vp, vp, sz, vp, C.c_int, C.c_int,
                                             C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_int, vp,
                                             C.c_int]
        _ref_libs[key] = lib
    return _ref_libs[key]


def ref_render_frame(frame, max_thresholds: int, n_threads: int = 0) -> np.ndarray:
    """Rasterize with the reference's own Kernels.cl (compiled for the CPU)."""
    spec = frame.spec
    lib = _load_ref(spec.max_shape, spec.stack_sections, float(np.float32(spec.stochastic_factor)))
    out = np.zeros((frame.canvas_h, frame.canvas_w), dtype=np.uint32)
    bg = np.ascontiguousarray(frame.background, dtype=np.float32)
    for ji, job in enumerate(frame.jobs):
        rc = lib.gudni_ref_raster_job(_p(frame.geometry), frame.geometry.size, _p(frame.substances),
                                      len(frame.substances), _p(frame.pictures), frame.pictures.size,
                                      _p(frame.picture_uses), len(frame.picture_uses), _p(frame.random_field),
                                      _p(job.shapes), len(job.shapes), _p(job.tiles), len(job.tiles),
                                      spec.threads_per_tile, frame.compute_depth, frame.canvas_w,
                                      frame.canvas_h, 0, ji, _p(bg), max_thresholds, _p(out), n_threads)
        if rc != 0:
            raise RuntimeError(f"reference kernels failed: {rc}")
    return out


def _adjoint(frame, target, max_thresholds, n_threads):
    lib = _load()
    spec = frame.spec
    img = np.zeros((frame.canvas_h, frame.canvas_w, 4), np.float32)
    g_geo = np.zeros(frame.geometry.size // 4, np.float64)
    g_sub = np.zeros(4 * len(frame.substances), np.float64)
    bg = np.ascontiguousarray(frame.background, dtype=np.float32)
    tgt = None if target is None else np.ascontiguousarray(target, dtype=np.float32)
    maxt = max_thresholds or spec.max_thresholds
    for job in frame.jobs:
        rc = lib.oracle_adjoint_job(_p(frame.geometry), frame.geometry.size, _p(frame.substances), len(frame.substances),
                                    _p(frame.pictures), _p(frame.picture_uses), _p(frame.radials), _p(job.shapes),
                                    _p(job.tiles), len(job.tiles), spec.threads_per_tile, frame.compute_depth,
                                    frame.canvas_w, frame.canvas_h, _p(bg), maxt, spec.max_shape, _p(img),
                                    _p(tgt), _p(g_geo) if tgt is not None else None,
                                    _p(g_sub) if tgt is not None else None, n_threads)
        if rc != 0:
            raise RuntimeError(f"oracle adjoint failed: {rc}")
    return img, g_geo, g_sub


def render_float(frame, n_threads: int = 0, max_thresholds: Optional[int] = None) -> np.ndarray:
    """(H, W, 4) float image: RGB before the byte conversion and the pixel's total
    section area."""
    img, _, _ = _adjoint(frame, None, max_thresholds, n_threads)
    return img


def loss_and_gradient(frame, target: np.ndarray, n_threads: int = 0, max_thresholds: Optional[int] = None):
    """FP64 reference of L = sum (I_rgb - T_rgb)^2 and its gradient with respect to
    every float of the geometry pile and every substance colour."""
    img, g_geo, g_sub = _adjoint(frame, target, max_thresholds, n_threads)
    d = img[..., :3].astype(np.float64) - np.asarray(target, np.float64)[..., :3]
    return float(np.sum(d * d)), g_geo, g_sub.reshape(-1, 4), img
