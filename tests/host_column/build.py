"""Build recipe of the host-compiled column machine (test infrastructure)."""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(HERE, "host_column.cpp")
OUT = os.path.join(HERE, "_build", "libhost_column.so")
DEPS = [SRC, os.path.join(HERE, "warp_emu.h")] + [
    os.path.join(ROOT, "gudni_gb300", "csrc", f)
    for f in ("raster_device.cuh", "adjoint_device.cuh", "strand_table.h", "warp_column.cuh", "tile_coop.cuh")] + [
    os.path.join(ROOT, "include", "gudni_cuda.h")]
CUDA_INCLUDE = "/usr/local/cuda/include"


def build() -> str:
    if not os.path.isfile(OUT) or max(os.path.getmtime(d) for d in DEPS) > os.path.getmtime(OUT):
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        # -O1: the same IEEE results as -O2 (no contraction, no fast math) from a
        # compile that takes a third of the time
        subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fno-strict-aliasing", "-fPIC", "-shared",
                        "-w", "-pthread", "-I", CUDA_INCLUDE, "-I", os.path.join(ROOT, "include"), SRC, "-o", OUT], check=True)
    return OUT


def load():
    lib = C.CDLL(build())
    vp, sz, i = C.c_void_p, C.c_size_t, C.c_int
    lib.host_column_raster_job.restype = C.c_int
    lib.host_column_raster_job.argtypes = [vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, i, i, i, i, i, vp, vp,
                                           C.c_float, i, i, vp, C.POINTER(C.c_int)]
    lib.host_column_set_adjoint_regenerate.restype = None
    lib.host_column_set_adjoint_regenerate.argtypes = [i]
    lib.host_column_adjoint_job.restype = C.c_int
    lib.host_column_adjoint_job.argtypes = [vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, i, i, i, i, i, vp, i,
                                            i, vp, vp, vp, vp, C.POINTER(C.c_int)]
    lib.host_column_raster_job_warp.restype = C.c_int
    lib.host_column_raster_job_warp.argtypes = [vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, i, i, i, i, i,
                                                vp, vp, C.c_float, i, i, i, i, C.c_uint64, vp,
                                                C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.host_column_raster_job_coop.restype = C.c_int
    lib.host_column_raster_job_coop.argtypes = [vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, i, i, i, i, i,
                                                vp, vp, C.c_float, i, i, i, C.c_uint64, vp, C.POINTER(C.c_int),
                                                C.POINTER(C.c_int)]
    lib.host_warp_trace.restype = None
    lib.host_warp_trace.argtypes = [C.POINTER(C.c_longlong)]
    lib.host_set_random_source.restype = None
    lib.host_set_random_source.argtypes = [C.c_int, C.c_uint64]
    lib.host_strand_table.restype = sz
    lib.host_strand_table.argtypes = [vp, sz, C.c_uint, vp, vp, vp, sz]
    return lib
