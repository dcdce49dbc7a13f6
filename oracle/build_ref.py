"""ORACLE -- test infrastructure only.

Build recipe for oracle/_ref/: the reference's own OpenCL kernels
(src/Graphics/Gudni/OpenCL/Kernels.cl, read where it lies under the reference
checkout) compiled for the CPU as C++, to pin the restatement in
oracle/raster_oracle.cpp.

Steps, all mechanical:
  1. Replace the file's first 40 lines with the #define block the reference host
     injects at JIT time (OpenCL/Setup.hs:45-64, CppDefines.hs:66-70), preceded by
     the OpenCL-C shim (oracle/ref_shim.h).  MAXSHAPE and SHAPESTACKSECTIONS are
     compile-time constants as in the reference; MAXTHRESHOLDS becomes a runtime
     capacity (it only sizes the per-column slabs).
  2. Rewrite OpenCL vector literals `(float4)(a, b, ...)` into calls of the shim's
     constructor `ocl_make<float4>(a, b, ...)` (C++ would read them as casts of a
     comma expression).
  3. Append the host driver oracle/ref_driver.inc and compile with g++.

Outputs go to oracle/_ref/ only (git-ignored).  Nothing in the package imports this.
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
# Where the reference checkout lies: the GUDNI_REFERENCE environment variable, else the
# build container's checkout (this recipe is the one file that reads it there).
DEFAULT_REFERENCE = os.environ.get("GUDNI_REFERENCE") or "/root/reference"
KERNELS_REL = os.path.join("src", "Graphics", "Gudni", "OpenCL", "Kernels.cl")
SOURCE_PADDING = 40  # sOURCEfILEpADDING, Raster/Constants.hs:70
# Optimisation level of the CPU build (GUDNI_REF_OPT, default -O2: one recipe that
# builds the same on the x86 build machine and the Arm GPU host; -O3 is there to
# compare the two once).
OPT = os.environ.get("GUDNI_REF_OPT") or "-O2"

VECTOR_LITERAL = re.compile(
    r"\(\s*(float2|float4|float8|int2|int4|uchar4|COLOR|SPACE2|SPACE4|THRESHOLD)\s*\)\s*\(")


def defines(max_shape: int, sections: int, stochastic: float) -> list[str]:
    """The #define list of cppDefines (OpenCL/Setup.hs:45-64)."""
    return [
        f"#define STOCHASTIC_FACTOR {stochastic!r}",
        "#define RANDOMFIELDSIZE 4096",
        "#define MAXTHRESHOLDS (gudni_ref_max_thresholds)",
        f"#define MAXSHAPE {max_shape}",
        f"#define SHAPESTACKSECTIONS {sections}",
        "#define SHAPETAG_SUBSTANCETYPE_BITMASK 0xC000000000000000",
        "#define SHAPETAG_SUBSTANCETYPE_SOLIDCOLOR 0x8000000000000000",
        "#define SHAPETAG_SUBSTANCETYPE_PICTURE 0x4000000000000000",
        "#define SHAPETAG_SUBSTANCETYPE_SHIFT 30",
        "#define SHAPETAG_COMPOUNDTYPE_BITMASK 0x3000000000000000",
        "#define SHAPETAG_COMPOUNDTYPE_CONTINUE 0x1000000000000000",
        "#define SHAPETAG_COMPOUNDTYPE_ADD 0x2000000000000000",
        "#define SHAPETAG_COMPOUNDTYPE_SUBTRACT 0x3000000000000000",
        "#define SHAPETAG_COMPOUNDTYPE_SHIFT 28",
        "#define SHAPETAG_SUBSTANCEID_BITMASK 0x0FFFFFFFFFFFFFFF",
    ]


def variant(max_shape: int, sections: int, stochastic: float = 0.0) -> str:
    """File-name tag of one compile-time configuration (MAXSHAPE, SHAPESTACKSECTIONS,
    STOCHASTIC_FACTOR)."""
    tag = f"m{max_shape}_s{sections}"
    return tag if stochastic == 0.0 else f"{tag}_st{stochastic!r}"


def library_name(max_shape: int, sections: int, stochastic: float = 0.0) -> str:
    opt = "" if OPT == "-O2" else "_" + OPT.lstrip("-")
    return os.path.join(OUT_DIR, f"libgudni_ref_{variant(max_shape, sections, stochastic)}{opt}.so")


def compile_flags() -> list[str]:
    """The g++ flags of the CPU build (no -march=native: the same recipe on both hosts)."""
    return ["-std=c++17", OPT, "-ffp-contract=off", "-fno-strict-aliasing", "-fopenmp"]


def source_name(max_shape: int, sections: int, stochastic: float = 0.0) -> str:
    return os.path.join(OUT_DIR, f"ref_kernels_{variant(max_shape, sections, stochastic)}.cpp")


def generate(reference: str, max_shape: int, sections: int, stochastic: float = 0.0) -> str:
    src_path = os.path.join(reference, KERNELS_REL)
    with open(src_path, "r") as f:
        lines = f.read().split("\n")
    head = ['#include "ref_shim.h"'] + defines(max_shape, sections, stochastic)
    head += ["// padding"] * max(0, SOURCE_PADDING - len(head))
    body = "\n".join(lines[SOURCE_PADDING:])
    body = VECTOR_LITERAL.sub(lambda m: f"ocl_make<{m.group(1)}>(", body)
    text = "\n".join(head) + "\n" + body + '\n#include "ref_driver.inc"\n'
    os.makedirs(OUT_DIR, exist_ok=True)
    out = source_name(max_shape, sections, stochastic)
    with open(out, "w") as f:
        f.write(text)
    return out


def build(reference: str = DEFAULT_REFERENCE, max_shape: int = 127, sections: int = 8,
          force: bool = False, stochastic: float = 0.0) -> str | None:
    """Build the reference kernels for one (MAXSHAPE, SHAPESTACKSECTIONS,
    STOCHASTIC_FACTOR) configuration.  Returns the library path, or None when neither
    the reference checkout nor a translation unit generated from it is present."""
    lib = library_name(max_shape, sections, stochastic)
    cpp = source_name(max_shape, sections, stochastic)
    deps = [os.path.join(HERE, "ref_driver.inc"), os.path.join(HERE, "ref_shim.h")]
    if os.path.isfile(lib) and not force and os.path.getmtime(lib) >= max(os.path.getmtime(d) for d in deps):
        return lib
    if os.path.isfile(os.path.join(reference, KERNELS_REL)):
        cpp = generate(reference, max_shape, sections, stochastic)
    elif not os.path.isfile(cpp):
        # neither the reference checkout nor a translation unit generated from it
        return None
    cmd = ["g++"] + compile_flags() + ["-fPIC", "-shared", "-w", "-Wno-psabi", "-I", HERE, cpp, "-o", lib]
    subprocess.run(cmd, check=True)
    return lib


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    ap.add_argument("--max-shape", type=int, default=127)
    ap.add_argument("--sections", type=int, default=8)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    lib = build(a.reference, a.max_shape, a.sections, a.force)
    print(lib if lib else "reference checkout not found; nothing built")
    return 0


if __name__ == "__main__":
    sys.exit(main())
