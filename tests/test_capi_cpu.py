"""The C-ABI libraries load on a machine without a GPU and export every entry point
their headers declare; no compute call is made here."""
import ctypes as C
import os
import re

import pytest

from gudni_gb300 import build as B
from gudni_gb300 import lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gudni_[a-z0-9_]+)\s*\(", text)))


def test_cuda_library_exports_header():
    path = B.build_cuda()
    lib = C.CDLL(path)
    names = declared("gudni_cuda.h")
    assert "gudni_raster_job" in names and "gudni_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_host_library_exports_header():
    lib = C.CDLL(B.build_host())
    missing = [n for n in declared("gudni_serialize.h") if not hasattr(lib, n)]
    assert not missing, missing


def test_create_without_device_fails_cleanly(cuda_available):
    if cuda_available:
        pytest.skip("a GPU is present")
    lib = L.load_cuda()
    spec = L.make_spec()
    assert not lib.gudni_create(C.byref(spec), 0)
    assert lib.gudni_last_error(None).decode()


def test_invalid_spec_rejected():
    lib = L.load_cuda()
    spec = L.make_spec()
    spec.threads_per_tile = 48  # not a power of two
    assert not lib.gudni_create(C.byref(spec), 0)
    assert "threads_per_tile" in lib.gudni_last_error(None).decode() or "device" in lib.gudni_last_error(None).decode()


def test_headers_compile_as_c_and_link(tmp_path):
    """The ABI is plain C: a C99 translation unit that includes both headers and takes
    the address of every declared entry point compiles with gcc and links against the
    two libraries (nothing is run)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    cuda_lib, host_lib = B.build_cuda(), B.build_host()
    names = declared("gudni_cuda.h") + declared("gudni_serialize.h")
    src = tmp_path / "abi.c"
    src.write_text("#include <stdio.h>\n#include \"gudni_cuda.h\"\n#include \"gudni_serialize.h\"\n"
                   "int main(void) {\n  const void* fns[] = {\n" +
                   "".join(f"    (const void*)&{n},\n" for n in names) +
                   "  };\n  printf(\"%d\\n\", (int)(sizeof fns / sizeof fns[0]));\n  return 0;\n}\n")
    exe = tmp_path / "abi"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe), cuda_lib, host_lib, "-Wl,-rpath," + os.path.dirname(cuda_lib)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_no_alloc_refuses_a_stochastic_spec():
    """The no-allocation entry point takes no random field: a spec with a non-zero
    STOCHASTIC_FACTOR is refused before anything reaches a device (the pointers below
    are never dereferenced)."""
    lib = L.load_cuda()
    fn = lib.gudni_raster_job_noalloc
    fn.restype = C.c_int
    vp, sz, i32 = C.c_void_p, C.c_size_t, C.c_int32
    fn.argtypes = [C.POINTER(L.Spec), vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz,
                   i32, i32, i32, i32, vp, vp, vp]
    spec = L.make_spec(32, 32, 4096, 127, 2, stochastic_factor=0.25)
    bg = (C.c_float * 4)(1, 1, 1, 1)
    fake = 1 << 20  # 16-byte aligned, never read
    rc = fn(C.byref(spec), fake, 16, fake, 1, None, 0, None, 0, None, 0, fake, 1, fake, 1, 32, 32, 5, 0, bg, fake,
            None)
    assert rc == -1
    assert "stochastic" in lib.gudni_last_error(None).decode()
