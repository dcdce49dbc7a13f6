"""The records the Python mirror hands to the C ABI (ctypes structures and numpy
dtypes) have the headers' layout: a C program compiled with gcc prints the size of
every struct of include/gudni_cuda.h and include/gudni_serialize.h and the offset
and size of each member, and each mirror must agree field by field.  Nothing is
run on a GPU."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from gudni_gb300 import batch as B
from gudni_gb300 import lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# C struct -> (Python mirror, [(mirror field, C member)])
MIRRORS = {
    "gudni_shape": (L.SHAPE_DTYPE, [("tag", "tag"), ("geo_start", "geo_start"), ("num_strands", "num_strands")]),
    "gudni_tile_info": (L.TILE_DTYPE, [("left", "left"), ("top", "top"), ("right", "right"), ("bottom", "bottom"),
                                       ("hdepth", "hdepth"), ("vdepth", "vdepth"),
                                       ("column_allocation", "column_allocation"),
                                       ("shape_start", "shapes.start"), ("shape_length", "shapes.length")]),
    "gudni_picture_use": (L.PICTURE_USE_DTYPE, [(n, n) for n in ("translate_x", "translate_y", "size_x", "size_y",
                                                                  "mem_offset", "scale")]),
    "gudni_radial": (L.RADIAL_DTYPE, [(n, n) for n in ("center_x", "center_y", "radius", "pad", "inner", "outer")]),
    "gudni_batch_scene": (B.BATCH_SCENE_DTYPE, [(n, n) for n in ("bitmap_w", "bitmap_h", "compute_depth",
                                                                  "job_index", "out_offset", "background")]),
    "gudni_spec": (L.Spec, [(n, n) for n, _ in L.Spec._fields_]),
    "gudni_scene_desc": (L.SceneDesc, [(n, n) for n, _ in L.SceneDesc._fields_]),
    "gudni_device_frame": (L.DeviceFrame, [(n, n) for n, _ in L.DeviceFrame._fields_]),
    "gudni_job_desc": (L.JobDesc, [(n, n) for n, _ in L.JobDesc._fields_]),
}


def c_layout(tmp_path):
    """{struct: (size, {member: (offset, size)})} as gcc lays the headers out."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "gudni_cuda.h"', '#include "gudni_serialize.h"',
             "int main(void) {"]
    for struct, (_, fields) in MIRRORS.items():
        lines.append(f'  printf("{struct} - %zu %zu\\n", (size_t)0, sizeof({struct}));')
        for _, member in fields:
            lines.append(f'  printf("{struct} {member} %zu %zu\\n", offsetof({struct}, {member}), '
                         f'sizeof((({struct}*)0)->{member}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    layout = {}
    for line in out.splitlines():
        struct, member, off, size = line.split()
        entry = layout.setdefault(struct, [0, {}])
        if member == "-":
            entry[0] = int(size)
        else:
            entry[1][member] = (int(off), int(size))
    return layout


def mirror_layout(mirror):
    """(size, {field: (offset, size)}) of a ctypes structure or a numpy dtype."""
    if isinstance(mirror, np.dtype):
        return mirror.itemsize, {n: (mirror.fields[n][1], mirror.fields[n][0].itemsize) for n in mirror.names}
    return C.sizeof(mirror), {n: (getattr(mirror, n).offset, getattr(mirror, n).size) for n, _ in mirror._fields_}


def test_mirrors_have_the_header_layout(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    layout = c_layout(tmp_path)
    for struct, (mirror, fields) in MIRRORS.items():
        size, members = layout[struct]
        msize, mfields = mirror_layout(mirror)
        assert msize == size, (struct, msize, size)
        assert sorted(mfields) == sorted(f for f, _ in fields), (struct, "fields not all compared")
        for field, member in fields:
            assert mfields[field] == members[member], (struct, field, mfields[field], members[member])


# ------------------------------------------------------------------ signatures
def header_prototypes():
    """{function: (return type, [parameter types])} of both headers, types as written."""
    import re
    protos = {}
    for header in ("gudni_cuda.h", "gudni_serialize.h"):
        text = open(os.path.join(ROOT, "include", header)).read()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
        text = "\n".join(line for line in text.splitlines() if not line.lstrip().startswith("#"))
        for stmt in re.split(r"[;{}]", text):
            m = re.fullmatch(r"\s*(.*?)\b(gudni_[a-z0-9_]+)\s*\((.*)\)\s*", stmt, flags=re.S)
            if not m:
                continue
            ret, name, params = m.group(1).strip(), m.group(2), m.group(3).strip()
            types = []
            if params not in ("", "void"):
                for p in params.split(","):
                    p = " ".join(p.split())
                    types.append(p if "*" in p or "[" in p else p.rsplit(" ", 1)[0])  # drop the name
            protos[name] = (ret, types)
    return protos


def c_kind(ctype):
    """(kind, bytes) of a C type as the ABI passes it."""
    if "*" in ctype or "[" in ctype:  # an array parameter is a pointer
        return ("ptr", 8)
    base = ctype.replace("const", "").replace("struct", "").split()
    base = base[-1] if base else ctype
    if base == "void":
        return None
    sizes = {"int": 4, "int32_t": 4, "uint32_t": 4, "int64_t": 8, "uint64_t": 8, "size_t": 8, "int16_t": 2,
             "uint16_t": 2, "uint8_t": 1}
    if base in ("float", "double"):
        return ("float", 4 if base == "float" else 8)
    assert base in sizes, f"unmapped C type {ctype!r}"
    return ("int", sizes[base])


def ctypes_kind(t):
    if t is None:
        return None
    if t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
        return ("ptr", 8)
    if t in (C.c_float, C.c_double):
        return ("float", C.sizeof(t))
    return ("int", C.sizeof(t))


def bound_libraries():
    """The two libraries with every binding the package makes (the batch entry points
    are declared by batch.bind, which BatchRasterizer calls)."""
    cuda = L.load_cuda()
    B.bind(cuda)
    return [L.load_host(), cuda]


def used_entry_points():
    """Every gudni_* entry point the package names."""
    import re
    pkg = os.path.join(ROOT, "gudni_gb300")
    names = set()
    for fn in os.listdir(pkg):
        if fn.endswith(".py"):
            names |= set(re.findall(r"\b(gudni_[a-z0-9_]+)\b", open(os.path.join(pkg, fn)).read()))
    return names


def test_bindings_match_the_header_prototypes():
    """Every declared entry point the package calls has argtypes (when it takes
    arguments) and a restype (when it returns other than int) that agree with the
    header prototype in kind and size: ctypes passes undeclared arguments as C ints."""
    protos = header_prototypes()
    libs = bound_libraries()
    used = sorted(used_entry_points() & set(protos))
    assert len(used) > 40
    for name in used:
        ret, params = protos[name]
        fn = next(getattr(lib, name) for lib in libs if hasattr(lib, name))
        if params:
            assert fn.argtypes is not None, (name, "no argtypes")
            assert len(fn.argtypes) == len(params), (name, len(fn.argtypes), params)
            for i, (v, p) in enumerate(zip(fn.argtypes, params)):
                assert ctypes_kind(v) == c_kind(p), (name, i, v, p)
        want = c_kind(ret)
        if want not in (None, ("int", 4)):
            assert ctypes_kind(fn.restype) == want, (name, fn.restype, ret)


HASKELL_KINDS = {"CInt": ("int", 4), "Int32": ("int", 4), "CUInt": ("int", 4), "Word32": ("int", 4),
                 "CSize": ("int", 8), "Word64": ("int", 8), "Int64": ("int", 8), "CULong": ("int", 8),
                 "CLong": ("int", 8), "CFloat": ("float", 4), "Float": ("float", 4), "CDouble": ("float", 8),
                 "Double": ("float", 8), "CString": ("ptr", 8), "()": None}


def haskell_kind(t):
    t = " ".join(t.split())
    while t.startswith("(") and t.endswith(")") and t != "()":
        t = t[1:-1].strip()
    if t.startswith("Ptr ") or t.startswith("FunPtr "):
        return ("ptr", 8)
    assert t in HASKELL_KINDS, f"unmapped Haskell type {t!r}"
    return HASKELL_KINDS[t]


def test_haskell_imports_match_the_header_prototypes():
    """The foreign imports of the Haskell drop-in modules (haskell/Graphics/Gudni/CUDA/)
    take the arguments and return the result the header declares (number, and pointer,
    integer or float of each, with its size)."""
    import glob
    import re
    protos = header_prototypes()
    sources = sorted(glob.glob(os.path.join(ROOT, "haskell", "**", "*.hs"), recursive=True))
    assert any(s.endswith(os.path.join("CUDA", "CallKernels.hs")) for s in sources)
    text = "".join(open(s).read() for s in sources)
    imports = re.findall(r'foreign import ccall (?:safe|unsafe) "(gudni_[a-z0-9_]+)"\s+\w+\s*::\s*(.*?)'
                         r'\bIO\s+(\(\s*\)|\([^)]*\)|\w+)', text, flags=re.S)
    assert len(imports) >= 10
    for name, args, result in imports:
        assert name in protos, f"{name} is not declared in include/"
        ret, params = protos[name]
        types = [a for a in args.split("->") if a.strip()]
        assert len(types) == len(params), (name, len(types), params)
        for i, (t, p) in enumerate(zip(types, params)):
            assert haskell_kind(t) == c_kind(p), (name, i, t, p)
        assert haskell_kind(result) == c_kind(ret), (name, result, ret)
