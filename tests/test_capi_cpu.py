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
