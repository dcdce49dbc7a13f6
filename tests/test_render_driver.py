"""gudni_render, the native host program over the C ABI: its scene-file reader (CPU,
no device touched), its clean failure without a GPU, and (on a GPU) its images through
the host and the device serializer against the oracle."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import fixture_scenes as F  # noqa: E402
from gudni_gb300 import build as B  # noqa: E402
from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402


def render_exe():
    B.build_all()
    return B.RENDER


def read_ppm(path):
    with open(path, "rb") as f:
        data = f.read()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"P6" and parts[2] == b"255"
    w, h = map(int, parts[1].split())
    return np.frombuffer(parts[3], np.uint8).reshape(h, w, 3)


def bgra_to_rgb(img):
    b = img.view(np.uint8).reshape(img.shape + (4,))
    return b[..., [2, 1, 0]]


def test_scene_file_is_read_back(tmp_path):
    flat = G.glyph_page(seed=4, width=300, height=200, n_glyphs=40, n_shapes=8)
    spec = L.make_spec(16, 64, 4096, 255, 8)
    path = str(tmp_path / "scene.bin")
    S.write_scene_file(path, flat, spec)
    r = subprocess.run([render_exe(), path, "--describe"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    assert d == {"canvas": [300, 200], "substances": int(flat.substance_kind.size),
                 "shapes": int(flat.shape_compound.size), "pairs": int(flat.pairs.shape[0]),
                 "pictures": int(flat.picture_offset.size), "picture_bytes": int(flat.pictures.size),
                 "random_field": True, "tile": 16, "threads_per_tile": 64}


def test_truncated_or_inconsistent_file_is_refused(tmp_path):
    flat = G.random_shapes(seed=2, width=64, height=48, n_shapes=5)
    path = str(tmp_path / "scene.bin")
    S.write_scene_file(path, flat, L.make_spec(16, 16, 512, 127, 8))
    data = open(path, "rb").read()
    cut = str(tmp_path / "cut.bin")
    open(cut, "wb").write(data[:len(data) // 2])
    assert subprocess.run([render_exe(), cut, "--describe"], capture_output=True).returncode == 1
    import dataclasses
    bad = dataclasses.replace(flat, outline_pair_start=flat.outline_pair_start[::-1].copy())
    S.write_scene_file(path, bad, L.make_spec(16, 16, 512, 127, 8))
    r = subprocess.run([render_exe(), path, "--describe"], capture_output=True, text=True)
    assert r.returncode == 1 and "out of order" in r.stderr


def test_no_device_is_a_clean_error(tmp_path, cuda_available):
    if cuda_available:
        pytest.skip("a GPU is present")
    flat = G.random_shapes(seed=2, width=64, height=48, n_shapes=5)
    path = str(tmp_path / "scene.bin")
    S.write_scene_file(path, flat, L.make_spec(16, 16, 512, 127, 8))
    r = subprocess.run([render_exe(), path, str(tmp_path / "out.ppm")], capture_output=True, text=True)
    assert r.returncode == 3 and "gudni_create" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("device_serializer", [False, True])
def test_render_matches_oracle(tmp_path, device_serializer):
    from oracle import oracle as O
    fn, w, h, spec, _ = F.SCENES["textured"]
    flat = S.flatten(fn(), w, h)
    path = str(tmp_path / "scene.bin")
    S.write_scene_file(path, flat, spec)
    out = str(tmp_path / "out.ppm")
    cmd = [render_exe(), path, out, "--frames", "2"] + (["--device-serializer"] if device_serializer else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout)
    assert line["serializer"] == ("device" if device_serializer else "host") and line["frames"] == 2
    want = bgra_to_rgb(O.render_frame(S.serialize_flat(flat, spec)))
    assert np.array_equal(read_ppm(out), want)
