"""Build the package's native libraries in-tree.

  gudni_gb300/_build/libgudni_host.so   host serializer (g++)
  gudni_gb300/_build/libgudni_cuda.so   sm_103a raster kernels + C ABI (nvcc)
  gudni_gb300/_build/gudni_render       native host program over both (render_main.cpp)

The two libraries are plain shared libraries with C entry points (include/*.h),
loaded through ctypes; nothing is installed into site-packages.  Compilation runs in parallel and
only when a source is newer than its library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")

HOST_LIB = os.path.join(BUILD, "libgudni_host.so")
CUDA_LIB = os.path.join(BUILD, "libgudni_cuda.so")

HOST_SOURCES = [os.path.join(CSRC, "serialize.cpp")]
HOST_DEPS = [os.path.join(CSRC, "serialize_device.cuh")]
CUDA_SOURCES = [os.path.join(CSRC, f) for f in ("raster.cu", "raster_counter.cu", "adjoint.cu", "capi.cu",
                                                  "noalloc.cu")]
HEADERS = [os.path.join(INCLUDE, h) for h in ("gudni_cuda.h", "gudni_serialize.h")] + [
    os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
# Exact IEEE single precision: no FMA contraction, IEEE division and square root,
# no flush-to-zero -- the raster arithmetic must match the reference bit for bit.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off"]
GXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-strict-aliasing", "-fopenmp"]


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.isfile(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources + HEADERS if os.path.exists(s))


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA extension cannot be built")
    return path


def cuda_include() -> str:
    """The CUDA headers (vector types for the serializer's shared pass code)."""
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "include")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_host(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force or _stale(HOST_LIB, HOST_SOURCES + HOST_DEPS):
        cmd = ["g++"] + GXX_FLAGS + ["-shared", "-I", INCLUDE, "-I", CSRC, "-I", cuda_include()] + HOST_SOURCES + [
            "-o", HOST_LIB]
        try:
            _run(cmd)
        except RuntimeError:  # a toolchain without OpenMP: the parallel serializer runs on one thread
            _run([a for a in cmd if a != "-fopenmp"])
    return HOST_LIB


def build_cuda(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not (force or _stale(CUDA_LIB, CUDA_SOURCES)):
        return CUDA_LIB
    objs = []
    cmds = []
    for src in CUDA_SOURCES:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        cmds.append([nvcc(), ARCH] + NVCC_FLAGS + ["-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(_run, cmds))
    _run([nvcc(), ARCH, "-shared", "-o", CUDA_LIB] + objs + ["-lcudart"])
    return CUDA_LIB


RENDER_SOURCES = [os.path.join(CSRC, "render_main.cpp")]
RENDER = os.path.join(BUILD, "gudni_render")


def build_render(force: bool = False) -> str:
    """gudni_render, the native host program (links both libraries and the CUDA runtime)."""
    if force or _stale(RENDER, RENDER_SOURCES + [HOST_LIB, CUDA_LIB]):
        _run([nvcc(), "-O2", "-std=c++17", "-I", INCLUDE] + RENDER_SOURCES +
             ["-o", RENDER, "-L", BUILD, "-lgudni_cuda", "-lgudni_host", "-Xlinker", "-rpath," + BUILD])
    return RENDER


def build_all(force: bool = False) -> dict:
    with ThreadPoolExecutor(max_workers=2) as ex:
        h = ex.submit(build_host, force)
        c = ex.submit(build_cuda, force)
        out = {"host": h.result(), "cuda": c.result()}
    out["render"] = build_render(force)
    return out


if __name__ == "__main__":
    print(build_all(force=True))
