"""Generate the golden raster fixtures in tests/golden/.

For every fixture scene (fixture_scenes.py) this renders the serialized frame with
the reference's own kernels -- src/Graphics/Gudni/OpenCL/Kernels.cl compiled for the
CPU by oracle/build_ref.py -- and stores the BGRA image (small scenes) or its SHA-256
(large scenes), together with the SHA-256 of the serialized piles the image was
rendered from.  Scenes that use the radial-gradient substance, which the reference
does not have, are rendered with the oracle and marked as such.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import fixture_scenes as F  # noqa: E402
from oracle import oracle as O  # noqa: E402

FULL_IMAGE_LIMIT = 128 * 128


def pile_digest(frame) -> str:
    h = hashlib.sha256()
    h.update(frame.geometry.tobytes())
    h.update(frame.substances.tobytes())
    h.update(frame.picture_uses.tobytes())
    h.update(frame.radials.tobytes())
    for j in frame.jobs:
        h.update(j.shapes.tobytes())
        h.update(j.tiles.tobytes())
    return h.hexdigest()


def image_digest(img: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(img).tobytes()).hexdigest()


def main() -> int:
    index = {}
    for name in F.ALL:
        frame = F.build(name)
        st = {}
        oracle_img = O.render_frame(frame, stats=st)
        if F.reference_comparable(name):
            img = O.ref_render_frame(frame, max_thresholds=max(64, st["max_queue"] + 8))
            source = "reference-kernels"
            assert np.array_equal(img, oracle_img), f"oracle disagrees with reference kernels on {name}"
        else:
            img = oracle_img
            source = "oracle"
        entry = {"source": source, "shape": list(img.shape), "image_sha256": image_digest(img),
                 "piles_sha256": pile_digest(frame), "max_queue": int(st["max_queue"]),
                 "thresholds": int(st["thresholds"]), "sections": int(st["sections"])}
        if img.size <= FULL_IMAGE_LIMIT:
            np.save(os.path.join(HERE, f"{name}.npy"), img)
            entry["image_file"] = f"{name}.npy"
        index[name] = entry
        print(f"{name:24s} {source:18s} {img.shape} thresholds={st['thresholds']}")
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
