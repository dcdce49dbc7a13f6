"""Known-answer piles for the serializer: tests/golden/known_piles.json holds the
geometry pile and every job's shape and tile records of five edge scenes, derived by
tests/golden/known_piles.py, a second restatement written step by step from the
reference's Haskell host (Raster/Strand.hs, Deknob.hs, ReorderTable.hs, Enclosure.hs,
Serialize.hs, TileTree.hs, Job.hs).  The scenes: a knob bulging right
(benchmarks/GudniTests.hs:247-255) and one bulging left with an off-axis control (both
split by findSplit), a shape of two outlines, a 21-curve run split into strands of 16
and 5 curves with a vertical segment and a reversed return, 130 shapes crowding one
leaf past mAXsHAPE - 1 (a split, jobs of two tiles, the last job first), and a strand
limit splitting leaves down to 8 pixels.  The sequential serializer, its parallel
passes, and the device passes (run on the CPU here, on the GPU in
test_serialize_device_gpu.py) must give these bytes."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
sys.path.insert(0, HERE)

import known_piles as K  # noqa: E402
from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402

with open(os.path.join(HERE, "golden", "known_piles.json")) as f:
    KNOWN = json.load(f)


def case(name):
    shapes, w, h, tile, tpt, per_job, max_strands = K.scenes()[name]
    spec = L.make_spec(tile, tpt, 4096, 127, 2, max_tiles_per_call=per_job, max_strands_per_tile=max_strands)
    return K.flat_scene(shapes, w, h), spec


def test_derivation_gives_the_fixture():
    """The committed fixture is what the derivation computes."""
    assert K.derive_all() == KNOWN


@pytest.mark.parametrize("threads", [1, 0])
@pytest.mark.parametrize("name", sorted(KNOWN))
def test_host_serializers_give_the_known_piles(name, threads):
    flat, spec = case(name)
    frame = S.serialize_flat(flat, spec, threads=threads)
    want = KNOWN[name]
    assert frame.geometry.tobytes().hex() == want["geometry"]
    assert len(frame.jobs) == len(want["jobs"])
    for job, wj in zip(frame.jobs, want["jobs"]):
        assert job.shapes.tobytes().hex() == wj["shapes"]
        assert job.tiles.tobytes().hex() == wj["tiles"]


@pytest.mark.parametrize("name", sorted(KNOWN))
def test_device_passes_give_the_known_piles(name):
    """The device serializer's passes, run on the CPU, write the known geometry pile
    and the known jobs concatenated (each tile's shape slice offset into the
    concatenated shape pile)."""
    import shutil
    if shutil.which("g++") is None or not os.path.isdir("/usr/local/cuda/include"):
        pytest.skip("needs g++ and the CUDA headers")
    from test_serialize_device import device_passes
    flat, spec = case(name)
    got = device_passes(flat, spec, seed=3, provenance=False)
    assert "error" not in got, got.get("error")
    want = KNOWN[name]
    assert got["geometry"].hex() == want["geometry"]
    shapes = b"".join(bytes.fromhex(j["shapes"]) for j in want["jobs"])
    assert got["shapes"].hex() == shapes.hex()
    tiles = []
    base = 0
    for j in want["jobs"]:
        t = np.frombuffer(bytes.fromhex(j["tiles"]), dtype=L.TILE_DTYPE).copy()
        t["shape_start"] += base
        tiles.append(t)
        base += len(bytes.fromhex(j["shapes"])) // 16
    assert got["tiles"] == np.concatenate(tiles).tobytes()
