"""Build recipe of the host-run device serializer (test infrastructure): a standalone
program built with AddressSanitizer and UBSan."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(HERE, "host_serialize.cpp")
OUT = os.path.join(HERE, "_build", "host_serialize")
DEPS = [SRC, os.path.join(ROOT, "gudni_gb300", "csrc", "serialize_device.cuh"),
        os.path.join(ROOT, "include", "gudni_cuda.h"), os.path.join(ROOT, "include", "gudni_serialize.h")]
CUDA_INCLUDE = "/usr/local/cuda/include"


def build() -> str:
    if not os.path.isfile(OUT) or max(os.path.getmtime(d) for d in DEPS) > os.path.getmtime(OUT):
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-ffp-contract=off", "-fno-strict-aliasing",
                        "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer",
                        "-I", CUDA_INCLUDE, "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(ROOT, "gudni_gb300", "csrc"), SRC, "-o", OUT], check=True)
    return OUT
