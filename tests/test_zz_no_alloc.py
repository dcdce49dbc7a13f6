"""gudni_raster_job_noalloc: the entry point for callers that cannot allocate device
memory (a plugin inside another framework's allocator, a sandbox without allocation
rights, a real-time loop that must not hit cudaMalloc's implicit synchronisation).

The test owns every device buffer (allocated here with torch) and calls the entry
point through the C ABI twice in a row; each time its output must match the frame
entry point (gudni_raster_frame, which allocates its own buffers) within the raster
parity bar -- <=1 LSB per channel, >=99.9% of pixels exact -- and in fact bit for bit.
The file sorts last so that a run stopping at the first failure has run every other
test; it also passes alone in a fresh process."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from conftest import assert_parity  # noqa: E402
from gudni_gb300 import lib as L  # noqa: E402
from gudni_gb300 import scene as S  # noqa: E402
from gudni_gb300 import scenes as G  # noqa: E402
from gudni_gb300.raster import Rasterizer  # noqa: E402

pytestmark = pytest.mark.gpu


def _bind(lib):
    vp, sz, i32 = C.c_void_p, C.c_size_t, C.c_int32
    fn = lib.gudni_raster_job_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(L.Spec), vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz, vp, sz,
                   i32, i32, i32, i32, vp, vp, vp]
    return fn


def _device(a, torch):
    """A device copy of a numpy record array, as raw bytes (owned by the test)."""
    raw = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
    if raw.size == 0:
        return None, torch.zeros(16, dtype=torch.uint8, device="cuda")
    t = torch.from_numpy(raw.copy()).to("cuda")
    return t.data_ptr(), t


def test_no_alloc_matches_frame_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    # a scene with every substance type, subtract combinators and two jobs
    flat = G.glyph_page(seed=13, width=200, height=150, n_glyphs=60, n_shapes=12)
    spec = L.make_spec(max_tile_size=32, threads_per_tile=32, max_thresholds=4096, max_shape=255,
                       stack_sections=4, max_tiles_per_call=20)
    frame = S.serialize_flat(flat, spec)
    assert len(frame.jobs) >= 2 and len(frame.radials) and len(frame.picture_uses)

    with Rasterizer(frame.spec) as r:
        want = r.raster_frame(frame)

    lib = L.load_cuda()
    fn = _bind(lib)
    keep = []
    common = {}
    for name in ("geometry", "substances", "pictures", "picture_uses", "radials"):
        p, t = _device(getattr(frame, name), torch)
        keep.append(t)
        common[name] = p
    jobs = []
    for job in frame.jobs:
        ps, ts = _device(job.shapes, torch)
        pt, tt = _device(job.tiles, torch)
        keep += [ts, tt]
        jobs.append((ps, len(job.shapes), pt, len(job.tiles)))
    out = torch.zeros(frame.canvas_w * frame.canvas_h, dtype=torch.int32, device="cuda")
    bg = np.ascontiguousarray(frame.background, np.float32)
    spec_c = L.Spec(*[getattr(frame.spec, f) for f, _ in L.Spec._fields_])
    torch.cuda.synchronize()

    for call in range(2):  # the scratch keeps the previous call's contents
        out.fill_(0x5A5A5A5A)
        for j, (ps, ns, pt, nt) in enumerate(jobs):
            rc = fn(C.byref(spec_c), common["geometry"], frame.geometry.size, common["substances"],
                    len(frame.substances), common["pictures"], frame.pictures.size, common["picture_uses"],
                    len(frame.picture_uses), common["radials"], len(frame.radials), ps, ns, pt, nt,
                    frame.canvas_w, frame.canvas_h, frame.compute_depth, j, bg.ctypes.data, out.data_ptr(), None)
            assert rc == 0, lib.gudni_last_error(None).decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint32).reshape(frame.canvas_h, frame.canvas_w)
        assert_parity(got, want)
        assert np.array_equal(got, want), f"call {call}: {(got != want).sum()} pixels differ"


def test_no_alloc_rejects_columns_beyond_its_capacity():
    """A column needing more than GUDNI_NOALLOC_CAPACITY (512) thresholds is refused
    with a clear error; the allocating entry point renders the same scene."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    # 300 tall slivers inside one pixel column: two thresholds each in that column
    items = [S.t_translate(5.2 + 0.002 * i, 1, S.solid((0.1, 0.2, 0.3, 0.5), S.shape([
        S.segments_to_outline([S.straight(0, 0), S.straight(0.001, 0), S.straight(0.001, 20),
                               S.straight(0, 20)])]))) for i in range(300)]
    spec = L.make_spec(max_tile_size=16, threads_per_tile=16, max_thresholds=4096, max_shape=1023,
                       stack_sections=16)
    frame = S.serialize(S.Scene((1, 1, 1, 1), S.overlap(items)), 16, 24, spec)
    with Rasterizer(frame.spec) as r:
        r.raster_frame(frame)  # fine with the allocating entry point
    lib = L.load_cuda()
    fn = _bind(lib)
    keep = []
    ptrs = {}
    for name in ("geometry", "substances"):
        p, t = _device(getattr(frame, name), torch)
        keep.append(t)
        ptrs[name] = p
    job = frame.jobs[0]
    ps, ts = _device(job.shapes, torch)
    pt, tt = _device(job.tiles, torch)
    out = torch.zeros(frame.canvas_w * frame.canvas_h, dtype=torch.int32, device="cuda")
    bg = np.ascontiguousarray(frame.background, np.float32)
    spec_c = L.Spec(*[getattr(frame.spec, f) for f, _ in L.Spec._fields_])
    torch.cuda.synchronize()
    rc = fn(C.byref(spec_c), ptrs["geometry"], frame.geometry.size, ptrs["substances"], len(frame.substances),
            None, 0, None, 0, None, 0, ps, len(job.shapes), pt, len(job.tiles), frame.canvas_w, frame.canvas_h,
            frame.compute_depth, 0, bg.ctypes.data, out.data_ptr(), None)
    assert rc == -2
    assert "512" in lib.gudni_last_error(None).decode()


def test_no_alloc_orders_after_async_copies_on_its_stream():
    """A caller that writes the records with asynchronous copies on its own
    non-blocking stream and calls the entry point on that stream gets the image of
    those records: the call reads nothing from the host before its launch, so the
    kernel runs after the copies.  A sleep kernel ahead of the copies keeps them in
    flight when the call is made.  A malformed tile and a misaligned picture use
    written the same way are found by the kernel and returned as bad input."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    flat = G.glyph_page(seed=21, width=160, height=96, n_glyphs=40, n_shapes=8)
    spec = L.make_spec(max_tile_size=32, threads_per_tile=32, max_thresholds=4096, max_shape=127,
                       stack_sections=2)
    frame = S.serialize_flat(flat, spec)
    assert len(frame.jobs) == 1 and len(frame.picture_uses)
    with Rasterizer(frame.spec) as r:
        want = r.raster_frame(frame)
    lib = L.load_cuda()
    fn = _bind(lib)
    stream = torch.cuda.Stream()  # torch's pool streams are non-blocking
    job = frame.jobs[0]

    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).pin_memory()

    host = {n: pinned(getattr(frame, n)) for n in ("geometry", "substances", "pictures", "picture_uses", "radials")}
    host["shapes"], host["tiles"] = pinned(job.shapes), pinned(job.tiles)
    dev = {n: torch.zeros(max(t.numel(), 16), dtype=torch.uint8, device="cuda") for n, t in host.items()}
    out = torch.zeros(frame.canvas_w * frame.canvas_h, dtype=torch.int32, device="cuda")
    bg = np.ascontiguousarray(frame.background, np.float32)
    spec_c = L.Spec(*[getattr(frame.spec, f) for f, _ in L.Spec._fields_])
    torch.cuda.synchronize()

    def call(tiles_src, uses_src):
        with torch.cuda.stream(stream):
            torch.cuda._sleep(50_000_000)  # tens of milliseconds ahead of the copies
            for n, t in host.items():
                src = {"tiles": tiles_src, "picture_uses": uses_src}.get(n, t)
                dev[n][:src.numel()].copy_(src, non_blocking=True)
            out.fill_(0)
        return fn(C.byref(spec_c), dev["geometry"].data_ptr(), frame.geometry.size, dev["substances"].data_ptr(),
                  len(frame.substances), dev["pictures"].data_ptr(), frame.pictures.size,
                  dev["picture_uses"].data_ptr(), len(frame.picture_uses), dev["radials"].data_ptr(),
                  len(frame.radials), dev["shapes"].data_ptr(), len(job.shapes), dev["tiles"].data_ptr(),
                  len(job.tiles), frame.canvas_w, frame.canvas_h, frame.compute_depth, 0, bg.ctypes.data,
                  out.data_ptr(), C.c_void_p(stream.cuda_stream))

    for _ in range(2):
        assert call(host["tiles"], host["picture_uses"]) == 0, lib.gudni_last_error(None).decode()
        stream.synchronize()
        got = out.cpu().numpy().view(np.uint32).reshape(frame.canvas_h, frame.canvas_w)
        assert_parity(got, want)
        assert np.array_equal(got, want)

    bad_tiles = job.tiles.copy()
    bad_tiles["shape_length"][0] = len(job.shapes) + 5  # past the shape pile
    assert call(pinned(bad_tiles), host["picture_uses"]) == -1
    assert "outside" in lib.gudni_last_error(None).decode()
    bad_uses = frame.picture_uses.copy()
    bad_uses["mem_offset"] += 2  # not a multiple of 4
    assert call(host["tiles"], pinned(bad_uses)) == -1
    stream.synchronize()
    # and the next good call renders the frame again
    assert call(host["tiles"], host["picture_uses"]) == 0
    stream.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint32).reshape(frame.canvas_h, frame.canvas_w), want)
