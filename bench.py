#!/usr/bin/env python
"""Benchmark of the GB300 raster path (gudni's generate -> sort -> render kernels).

Workload (default): the 3840x2160 page -- 5000 glyph-like outlines plus 2000 random
shapes, 30% with subtract combinators, 20% radial gradients, 10% textured from a
seeded 1024x1024 RGBA8 noise picture (seeded synthetic data; the reference ships no
scene data).  Raster spec: 32x32 tiles, 32 threads per tile, MAXTHRESHOLDS 4096,
MAXSHAPE 127, 8 stack words.

A step renders the whole frame (all of its jobs).
  value  Mpixels/s with the frame's piles resident in HBM, one fused launch per frame
         (gudni_raster_tiles_device), timed with CUDA events on the launching stream
  e2e    the same metric through the frame-level C ABI call with HOST buffers
         (gudni_upload_common + gudni_raster_frame from pinned memory, output read
         back), timed on the host clock
The L2 (126 MB) is flushed between timed steps by writing a 256 MB buffer.

`--impl reference` times the reference's own kernels (Kernels.cl compiled for the
CPU, oracle/_ref) -- or, where that translation unit is not present, the oracle's
restatement -- on all host cores, one frame per step.  The reference has no radial
gradient substance, so its arm renders the page with every gradient baked into an
RGBA8 picture (scene.bake_radials, the reference's PictureFunction route); the line
reports that image's parity with the oracle's rendering of the page itself.

Other workloads (--workload): scene4k (the page from its flattened scene to pixels:
the serializer's passes on the device, gudni_serialize_device, then the raster
launch, against the host serializer), page1080 (a quarter page, the profiled size),
random512 (512x512, 64 random shapes), batch256 (the batched form: 256 scenes in one
persistent launch, CUDA graph, autotuned tile shapes, against one launch pair per
scene), adjoint1024 (forward vs fwd+adjoint on 1024x1024 with 500 shapes, gradients
checked against the FP64 reference and central differences), fit64 (batched
fitting of 64 scenes by Adam, steps/s).

Multi-GPU: frames are independent, so N ranks render N replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

UNIT = "Mpixels/s"
PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "raster_tiles_{}.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-sample-frames", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="page4k", choices=sorted(WORKLOADS))
    ap.add_argument("--dense-columns", type=int, default=0,
                    help="scan columns with at least this many thresholds by the whole warp (0: off)")
    ap.add_argument("--device-strand-table", action="store_true",
                    help="uploads build the strand table on the device (gudni_set_device_strand_table)")
    ap.add_argument("--cooperative-units", default="off", choices=["off", "on", "auto"],
                    help="warp-cooperative work units (gudni_set_cooperative_units) in every rasterizer")
    ap.add_argument("--scenes", type=int, default=256)
    ap.add_argument("--adjoint-side", type=int, default=1024, help="adjoint1024: canvas side (1024)")
    ap.add_argument("--adjoint-shapes", type=int, default=500, help="adjoint1024: random shapes (500)")
    ap.add_argument("--plain-untimed-pass", type=int, default=1,
                    help="batch256: one untimed pass of the per-scene path before timing it")
    ap.add_argument("--no-forms", action="store_true",
                    help="page4k: leave out the batched, fwd+adjoint and fitting sub-records")
    ap.add_argument("--form-dense-columns", type=int, default=32,
                    help="page4k sub-records: the batched form's warp-cooperative dense columns threshold")
    ap.add_argument("--fit-steps", type=int, default=5, help="page4k sub-records: timed fitting steps")
    ap.add_argument("--fit-resume", default=None,
                    help="fit64: continue from a state written by --fit-checkpoint (BatchFit.load)")
    ap.add_argument("--fit-checkpoint", default=None,
                    help="fit64: write the fit's state here at the end (BatchFit.save)")
    ap.add_argument("--fit-total-steps", type=int, default=None,
                    help="fit64: stop the timed steps once the fit has taken this many Adam steps in all")
    ap.add_argument("--fit-time-limit", type=float, default=None,
                    help="fit64: stop the timed steps after this many seconds (then --fit-checkpoint)")
    ap.add_argument("--tile", type=int, default=None, help="tile size (default: the workload's)")
    ap.add_argument("--threads-per-tile", type=int, default=None, help="threads per tile (default: the workload's)")
    return ap.parse_args()


# default (tile size, threads per tile) of the plain workloads: the page keeps the
# reference's default (threads per tile = tile size); the 512x512 scene of 64
# canvas-wide shapes has few, long columns at that setting and runs 256 threads per
# 32x32 tile (8 rows per column), the reference's other knob
PLAIN_TILES = {"page4k": (32, 32), "page1080": (32, 32), "random512": (32, 256)}


def tile_override(args, tile, tpt):
    """The workload's (tile size, threads per tile) unless given on the command line."""
    return (args.tile or tile), (args.threads_per_tile or tpt)


WORKLOADS = {
    # the headline plain workload
    "page4k": ("page_3840x2160_glyphs5000_shapes2000",
               "Mpixels/s (plain single-frame raster, 3840x2160 page, <=1 LSB RGBA8)"),
    # a quarter of the page (1920x1080, 1250 glyphs, 500 shapes): the size profiled in full
    "page1080": ("page_1920x1080_glyphs1250_shapes500",
                 "Mpixels/s (plain single-frame raster, 1920x1080 page, <=1 LSB RGBA8)"),
    # the small CPU-runnable plain workload: 512x512, 64 random shapes of 8-32 segments
    "random512": ("random_512x512_shapes64",
                  "Mpixels/s (plain single-frame raster, 512x512 64 shapes, <=1 LSB RGBA8)"),
    # the batched form (run_batch)
    "batch256": ("batch_mix_256_scenes", "frames/s (batched raster, 256-scene mix, <=1 LSB RGBA8)"),
    # the differentiable form (run_adjoint): 1024x1024, 500 random shapes of 16 segments
    "adjoint1024": ("random_1024x1024_shapes500_seg16",
                    "Mpixels/s (fwd+adjoint, 1024x1024 500 shapes, grads vs FP64 reference)"),
    # batched fitting (run_fit): 64 scenes of 256x256, 128 shapes each, Adam on points and colours
    "fit64": ("fit_64x256x256_shapes128", "steps/s (batched fwd+adjoint fitting, 64 scenes 256x256)"),
    # the 256-scene mix's densest scene alone (run_dense): 87x75, 1817 canvas-wide shapes
    "densest": ("batch_mix_scene25_87x75_shapes1817",
                "Mpixels/s (the batched mix's densest scene, 87x75 with 1817 shapes, <=1 LSB RGBA8)"),
    # scene to pixels on the device (run_scene): the page serialized by kernels, then rendered
    "scene4k": ("scene_page_3840x2160_glyphs5000_shapes2000",
                "Mpixels/s (scene to pixels: device serializer + raster, 3840x2160 page, <=1 LSB RGBA8)"),
}


def make_frame(workload: str = "page4k", baked: bool = False, tile: int = 32, tpt: int = 32):
    """The workload's serialized frame.  baked=True expresses each radial gradient as
    a picture (scene.bake_radials), the form the reference kernels can render."""
    from gudni_gb300 import lib as L
    from gudni_gb300 import scene as S
    from gudni_gb300 import scenes as G

    spec = L.make_spec(max_tile_size=tile, threads_per_tile=tpt, max_thresholds=4096, max_shape=127,
                       stack_sections=8)
    if workload == "page4k":
        flat = G.glyph_page(seed=1)
    elif workload == "page1080":
        flat = G.glyph_page(seed=1, width=1920, height=1080, n_glyphs=1250, n_shapes=500)
    else:
        flat = G.random_shapes(seed=0)
    if baked:
        flat = S.bake_radials(flat)
    return S.serialize_flat(flat, spec)


def reference_runner(workload: str, frame):
    """A callable rendering the workload once on the host cores, and what it is: the
    reference's own kernels (oracle/_ref) on the workload with radial gradients baked
    into pictures, else the oracle restatement on the workload itself.  Also returns
    the reference image and the oracle image, for the parity note."""
    from oracle import oracle as O
    want = O.render_frame(frame)
    fn, kind, img = (lambda: O.render_frame(frame)), "port", want  # noqa: E731
    if O.ref_available(frame.spec.max_shape, frame.spec.stack_sections):
        try:
            ref_frame = (make_frame(workload, baked=True, tile=frame.spec.max_tile_size,
                                    tpt=frame.spec.threads_per_tile) if len(frame.radials) else frame)
            st = {}
            O.render_frame(ref_frame, stats=st)
            cap = int(st["max_queue"]) + 16  # the reference writes past a full slab
            img = O.ref_render_frame(ref_frame, max_thresholds=cap)  # build + warm
            fn = lambda: O.ref_render_frame(ref_frame, max_thresholds=cap)  # noqa: E731
            kind = "reference"
        except Exception as e:  # noqa: BLE001
            print(f"reference kernels unavailable ({e}); timing the oracle", file=sys.stderr)
            fn, kind, img = (lambda: O.render_frame(frame)), "port", want  # noqa: E731
    return fn, kind, img, want


def apply_coop(r, args):
    """The --cooperative-units choice on a rasterizer (gudni_set_cooperative_units)."""
    mode = getattr(args, "cooperative_units", "off")
    r.set_cooperative_units({"on": True, "off": False, "auto": None}[mode])


def ref_build_flags():
    from oracle import build_ref
    return build_ref.compile_flags()


def lsb_parity(a, b):
    d = np.abs(a.view(np.uint8).astype(np.int16) - b.view(np.uint8).astype(np.int16))
    return {"max_lsb": int(d.max()), "exact_pixel_frac": float(np.mean(np.all(d.reshape(-1, 4) == 0, axis=1)))}


def config_dict(frame, workload="page4k"):
    sp = frame.spec
    return {"workload": WORKLOADS[workload][0], "canvas": [frame.canvas_w, frame.canvas_h],
            "shapes": int(frame.stats["shapes"]), "strands": int(frame.stats["strands"]),
            "tiles": int(frame.n_tiles), "jobs": len(frame.jobs),
            "tile_size": sp.max_tile_size, "threads_per_tile": sp.threads_per_tile,
            "max_thresholds": sp.max_thresholds, "max_shape": sp.max_shape,
            "stack_sections": sp.stack_sections, "l2": "flushed between steps (256 MB write)",
            "data": "synthetic, seeded"}


def algorithmic_bytes(frame, texels: int) -> int:
    """B_alg per frame: every tile reads its shape records and strand trees once, the
    tile records, substance and picture-use records, the texels it samples, and
    writes every pixel once."""
    geo = frame.geometry
    # bytes of each shape's strands, by walking the strand headers
    shape_bytes = {}
    total = 0
    for job in frame.jobs:
        for s in job.shapes:
            key = (int(s["geo_start"]), int(s["num_strands"]))
            if key not in shape_bytes:
                off = key[0] * 16
                nb = 0
                for _ in range(key[1]):
                    size = int(geo[off]) | (int(geo[off + 1]) << 8)
                    nb += 8 * size
                    off += 8 * size
                shape_bytes[key] = nb
            total += 16 + shape_bytes[key]
        total += 32 * len(job.tiles)
    total += 16 * len(frame.substances) + 24 * len(frame.picture_uses) + 48 * len(frame.radials)
    total += 4 * texels + 4 * frame.canvas_w * frame.canvas_h
    return int(total)


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(workload):
    path = PROFILE_SUMMARY.format(WORKLOADS[workload][0])
    if os.path.isfile(path):
        with open(path) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch"), d
    return None, None


def cpu_baseline(workload, frame, frames: int):
    """The reference kernels (or the oracle restatement) on all host cores, one frame
    per sample; returns (Mpixels/s, kind, cores, oracle image, seconds per frame,
    reference-vs-oracle parity)."""
    cores = os.cpu_count() or 1
    fn, kind, img, want = reference_runner(workload, frame)
    t0 = time.perf_counter()
    for _ in range(frames):
        fn()
    dt = (time.perf_counter() - t0) / frames
    return frame.canvas_w * frame.canvas_h / dt / 1e6, kind, cores, want, dt, lsb_parity(img, want)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    if args.workload not in ("page4k", "page1080", "random512"):  # batch256, adjoint1024, fit64, scene4k
        print(json.dumps({"impl": "reference", "unavailable": f"workload {args.workload} has no reference "
                          "counterpart (the reference renders one scene per call and has no adjoint)"}))
        return 0
    frame = make_frame(args.workload, False, *tile_override(args, *PLAIN_TILES[args.workload]))
    fn, kind, img, want = reference_runner(args.workload, frame)
    for _ in range(args.warmup):
        fn()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        fn()
        times.append(time.perf_counter() - t0)
    ms = 1000 * sum(times) / len(times)
    v = frame.canvas_w * frame.canvas_h / (ms / 1000) / 1e6
    cores = os.cpu_count() or 1
    sample = "one full frame per step (all jobs), OpenMP over all host cores"
    if kind == "reference" and len(frame.radials):
        sample += "; radial gradients baked into pictures (the reference has no radial substance)"
    line = {"impl": "reference", "metric": WORKLOADS[args.workload][1], "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(frame, args.workload),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample,
                             "build": " ".join(ref_build_flags()) if kind == "reference" else None},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "parity_reference_vs_oracle": lsb_parity(img, want)}
    print(json.dumps(line))
    return 0


BATCH_MAX_SHAPE = 2047        # up to 2000 canvas-wide shapes per scene touch every column
BATCH_MAX_THRESHOLDS = 32768
BATCH_STRANDS_PER_TILE = 1 << 24  # no strand-count tile splitting


def run_batch(args, emit=True):
    """The batched form: 256 scenes (sides log-uniform 64-1024 px, 10-2000 random shapes
    of 8-32 segments) in one persistent launch replayed from a CUDA graph, tile size and
    threads per tile per canvas-size bucket from the autotuner; against one launch pair
    per scene over the same resident piles.  Returns the result line (printed when
    `emit`)."""
    import torch
    from gudni_gb300 import autotune as A
    from gudni_gb300 import batch as B
    from gudni_gb300 import lib as L

    torch.cuda.set_device(0)
    t0 = time.perf_counter()
    flats = __import__("gudni_gb300.scenes", fromlist=["batch_mix"]).batch_mix(seed=2, n_scenes=args.scenes)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    choice = A.autotune(flats, BATCH_MAX_SHAPE, BATCH_MAX_THRESHOLDS, BATCH_STRANDS_PER_TILE, samples=1, reps=2,
                        log=lambda m: print(m, file=sys.stderr, flush=True), dense_columns=args.dense_columns)
    t_tune = time.perf_counter() - t0
    t0 = time.perf_counter()
    frames = A.serialize_tuned(flats, choice, BATCH_MAX_SHAPE, BATCH_MAX_THRESHOLDS, BATCH_STRANDS_PER_TILE)
    batch = B.build_batch(frames)
    t_ser = time.perf_counter() - t0
    spec = A.spec_for(32, 32, BATCH_MAX_SHAPE, BATCH_MAX_THRESHOLDS, BATCH_STRANDS_PER_TILE)
    r = B.BatchRasterizer(spec)
    apply_coop(r, args)
    if args.dense_columns:
        r.set_dense_columns(args.dense_columns)
    r.upload(batch)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    torch.cuda.set_stream(stream)

    def timed(fn, steps):
        ts = []
        for _ in range(steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            flush.zero_()
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return ts

    h = stream.cuda_stream
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    for i in range(args.warmup):
        t0 = time.perf_counter()
        r.render(use_graph=True, stream=h)
        r.sync_status()
        log(f"warm-up batch {i}: {time.perf_counter() - t0:.2f} s")
    launches0 = r.launch_count()
    with ClockSampler(0) as clocks:
        bt = timed(lambda: r.render(use_graph=True, stream=h), args.steps)
    r.sync_status()
    launches = r.launch_count() - launches0
    log(f"batched: {bt} ms")
    # the plain path: one launch pair per scene, each timed on its own, summed (after
    # one untimed pass over every scene, unless the batched warm-up already ran the
    # kernels: --plain-untimed-pass 0)
    if args.plain_untimed_pass:
        r.render_each_scene(stream=h)
    r.sync_status()
    per_scene = []
    for i, (first, count) in enumerate(batch.frame_tiles):
        per_scene.append(timed(lambda: r.render_tiles(first, count, stream=h), 1)[0])
    r.sync_status()
    log(f"plain per scene (ms): max {max(per_scene):.1f}, sum {sum(per_scene):.1f}")
    batched_ms = sum(bt) / len(bt)
    plain_ms = sum(per_scene)
    pixels = batch.out_pixels
    n = len(frames)
    out = r.download()
    parity = None
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        imgs = batch.images(out)
        order = np.argsort([f.canvas_w * f.canvas_h * f.stats["shapes"] for f in frames])[:16]
        worst, exact = 0, 1.0
        for i in order:
            want = O.render_frame(frames[i])
            d = np.abs(imgs[i].view(np.uint8).astype(np.int16) - want.view(np.uint8).astype(np.int16))
            worst = max(worst, int(d.max()))
            exact = min(exact, float(np.mean(np.all(d.reshape(-1, 4) == 0, axis=1))))
        parity = {"scenes_checked": len(order), "max_lsb": worst, "min_exact_pixel_frac": exact}
    line = {"metric": "frames/s (batched raster, 256-scene mix, <=1 LSB RGBA8)", "value": n / (batched_ms / 1000),
            "unit": "frames/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": batched_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"batch_mix_{n}_scenes", "scenes": n, "pixels": int(pixels),
                       "tiles": int(len(batch.tiles)), "shapes": int(sum(f.stats["shapes"] for f in frames)),
                       "max_shape": BATCH_MAX_SHAPE, "max_thresholds": BATCH_MAX_THRESHOLDS,
                       "autotune": {str(k): list(v) for k, v in choice.items()},
                       "l2": "flushed between steps (256 MB write)", "data": "synthetic, seeded",
                       "dense_columns": args.dense_columns},
            "mpixels_per_s": pixels / (batched_ms / 1000) / 1e6,
            "plain_per_scene": {"ms_per_batch": plain_ms, "frames_per_s": n / (plain_ms / 1000),
                                "launches_per_scene": "3 ordering kernels + fast pass (+ full-capacity pass)",
                                "slowest_scene_ms": max(per_scene),
                                "timing": "each scene's launch pair timed alone, summed"},
            "batched_over_plain": plain_ms / batched_ms,
            "gpu_launches": int(launches), "clocks": clocks.summary(), "parity_vs_oracle": parity,
            "host_s": {"generate": t_gen, "autotune": t_tune, "serialize": t_ser}}
    if emit:
        print(json.dumps(line))
    r.close()
    return line


ADJ_SPEC = dict(max_tile_size=32, threads_per_tile=32, max_thresholds=4096, max_shape=511, stack_sections=8,
                max_strands_per_tile=1 << 24)  # 500 canvas-wide shapes: no strand-count tile splitting


def adjoint_scene(jitter_px: float = 0.0, side: int = 1024, shapes: int = 500):
    """side x side canvas (1024), `shapes` random shapes (500) of 16 quadratic segments
    (seeded); the target copy has every control point jittered by N(0, jitter_px)."""
    from gudni_gb300 import scenes as G
    flat = G.random_shapes(seed=3, width=side, height=side, n_shapes=shapes, seg_lo=16, seg_hi=16)
    if jitter_px:
        rng = np.random.default_rng(4)
        flat.pairs = (flat.pairs + rng.normal(0, jitter_px, flat.pairs.shape)).astype(np.float32)
    return flat


def run_adjoint(args, emit=True):
    """The differentiable form: forward raster vs one fwd+adjoint launch on the same
    frame; gradients checked against the FP64 reference adjoint and against central
    differences (h = 1e-2 px) of the loss on the largest point-gradient entries."""
    import torch
    from gudni_gb300 import adjoint as A
    from gudni_gb300 import lib as L
    from gudni_gb300 import scene as S
    from gudni_gb300.raster import Rasterizer

    torch.cuda.set_device(0)
    tile, tpt = tile_override(args, ADJ_SPEC["max_tile_size"], ADJ_SPEC["threads_per_tile"])
    adj_spec = dict(ADJ_SPEC, max_tile_size=tile, threads_per_tile=tpt)
    spec = L.make_spec(**adj_spec)
    side, n_sh = getattr(args, "adjoint_side", 1024), getattr(args, "adjoint_shapes", 500)
    frame = S.serialize_flat(adjoint_scene(0.0, side, n_sh), spec)
    tframe = S.serialize_flat(adjoint_scene(4.0, side, n_sh), spec)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    r = Rasterizer(spec)
    apply_coop(r, args)
    with torch.cuda.stream(stream):
        tr = A.FrameAdjoint(r, tframe)
        _, timg, _, _ = tr.loss_and_gradient(np.zeros((side, side, 4), np.float32))
        target = timg.clone()
        target[..., 3] = 0
        fa = A.FrameAdjoint(r, frame)
        out = torch.zeros(side * side, dtype=torch.int32, device=dev)

        def forward():
            r.raster_tiles_device(frame, fa.shapes.data_ptr(), fa.n_shapes, fa.tiles.data_ptr(),
                                  fa.tile_jobs.data_ptr(), fa.n_tiles, out.data_ptr(), stream=stream.cuda_stream)

        def fwd_adjoint():
            fa.enqueue(target)

        def timed(fn, steps):
            ts = []
            for _ in range(steps):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                flush.zero_()
                b.synchronize()
                ts.append(a.elapsed_time(b))
            return ts

        for _ in range(args.warmup):
            forward()
            fwd_adjoint()
        r.sync_status()
        launches0 = r.launch_count()
        with ClockSampler(0) as clocks:
            ft = timed(forward, args.steps)
            at = timed(fwd_adjoint, args.steps)
        r.sync_status()
        launches = r.launch_count() - launches0
        fwd_ms, adj_ms = statistics.median(ft), statistics.median(at)
        # the other mode: the backward regenerates the thresholds (same image and gradients)
        r.set_adjoint_regenerate(True)
        fwd_adjoint()
        regen_ms = statistics.median(timed(fwd_adjoint, args.steps))
        r.set_adjoint_regenerate(False)
        r.sync_status()
        loss, img, gg, gs = fa.loss_and_gradient(target)
        gg, gs = gg.cpu().numpy().astype(np.float64), gs.cpu().numpy().astype(np.float64)
        img = img.cpu().numpy()
        tnp = target.cpu().numpy()
    check = {}
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        t0 = time.perf_counter()
        loss_ref, g_geo, g_sub, _ = O.loss_and_gradient(frame, tnp)
        t_ref = time.perf_counter() - t0
        rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
        check["fp64_reference"] = {"geometry_rel_err": rel(gg, g_geo), "substance_rel_err": rel(gs.ravel(),
                                                                                              g_sub.ravel()),
                                   "loss": float(loss), "loss_fp64": loss_ref, "host_s": t_ref}
        # central differences of the GPU loss at h = 1e-2 px on the 8 largest point entries
        gp = S.pair_gradient(frame, gg)
        idx = np.argsort(-np.abs(gp.ravel()))[:8]
        h = 1e-2
        fd_rel = []
        with torch.cuda.stream(stream):
            for k in idx:
                p, c = divmod(int(k), 4)
                vals = []
                for sgn in (1, -1):
                    fl = adjoint_scene(0.0, side, n_sh)
                    fl.pairs[p, c] += sgn * h
                    f2 = S.serialize_flat(fl, spec)
                    vals.append(float(A.FrameAdjoint(r, f2).loss_and_gradient(target)[0]))
                fd = (vals[0] - vals[1]) / (2 * h)
                fd_rel.append(abs(gp[p, c] - fd) / max(abs(fd), 1e-12))
        check["central_differences_h1e-2"] = {"entries": len(fd_rel), "median_rel_err": float(np.median(fd_rel)),
                                              "max_rel_err": float(np.max(fd_rel))}
    pixels = side * side
    line = {"metric": WORKLOADS["adjoint1024"][1], "value": pixels / (adj_ms / 1000) / 1e6, "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": adj_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS["adjoint1024"][0] if (side, n_sh) == (1024, 500) else
                       f"random_{side}x{side}_shapes{n_sh}_seg16", "canvas": [side, side], "shapes": n_sh,
                       "segments": 16, "target": "same scene, control points jittered N(0, 4 px)",
                       "tiles": int(frame.n_tiles), **adj_spec, "l2": "flushed between steps (256 MB write)",
                       "data": "synthetic, seeded"},
            "forward_ms": fwd_ms, "fwd_adjoint_ms": adj_ms, "fwd_adjoint_over_forward": adj_ms / fwd_ms,
            "thresholds": "generated once per work unit: the forward scans a copy of the sorted queue, the "
                          "backward the queue itself",
            "regenerate": {"fwd_adjoint_ms": regen_ms, "fwd_adjoint_over_forward": regen_ms / fwd_ms,
                           "thresholds": "the forward generates its own, the backward generates them again "
                                         "(gudni_set_adjoint_regenerate)", "steps": args.steps},
            "gpu_launches": int(launches), "clocks": clocks.summary(), "gradient_check": check}
    if emit:
        print(json.dumps(line))
    r.close()
    return line


def run_dense(args):
    """The batched mix's densest scene (scene 25 of batch_mix(seed=2): 87x75 canvas,
    1817 canvas-wide random shapes, ~97,000 sections per pixel) rendered alone at the
    spec the autotuner picks for its bucket (8-pixel tiles, 64 threads: one-pixel
    columns), with or without the warp-cooperative scan of dense columns
    (--dense-columns).  Timed on the host clock around each blocking frame call (one
    launch is seconds long); the image is checked against the per-lane scan's."""
    from gudni_gb300 import autotune as A
    from gudni_gb300 import scene as S
    from gudni_gb300 import scenes as G
    from gudni_gb300.raster import Rasterizer
    flat = G.batch_mix(seed=2, n_scenes=26)[25]
    spec = A.spec_for(8, 64, BATCH_MAX_SHAPE, BATCH_MAX_THRESHOLDS, BATCH_STRANDS_PER_TILE)
    frame = S.serialize_flat(flat, spec)
    times, img = [], None
    with Rasterizer(spec) as r:
        apply_coop(r, args)
        if args.dense_columns:
            r.set_dense_columns(args.dense_columns)
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            img = r.raster_frame(frame)
            if i >= args.warmup:
                times.append(time.perf_counter() - t0)
        launches = r.launch_count()
    parity = None
    if args.dense_columns and not args.no_cpu_baseline:
        with Rasterizer(spec) as r:
            parity = lsb_parity(img, r.raster_frame(frame))
    s_frame = statistics.median(times)
    line = {"metric": WORKLOADS["densest"][1], "value": frame.canvas_w * frame.canvas_h / s_frame / 1e6, "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * s_frame,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS["densest"][0], "canvas": [frame.canvas_w, frame.canvas_h],
                       "shapes": int(frame.stats["shapes"]), "tile_size": 8, "threads_per_tile": 64,
                       "max_shape": BATCH_MAX_SHAPE, "dense_columns": args.dense_columns,
                       "timing": "host clock around gudni_raster_frame (blocking), median"},
            "gpu_launches": int(launches), "parity_vs_per_lane_scan": parity}
    print(json.dumps(line))
    return 0


def run_scene(args):
    """Scene to pixels on the device: the page's flattened scene (host arrays, what a
    host hands over) serialized by kernels (gudni_serialize_device) and rendered from
    the frame left on the device; the host serializer is timed beside it, sequential
    (gudni_serialize) and on all host threads (gudni_serialize_parallel).  A step is one serialization plus one render.  The piles are
    checked byte for byte against the host serializer's and the image against the
    render of the host-serialized frame."""
    import torch
    from gudni_gb300 import lib as L
    from gudni_gb300 import scene as S
    from gudni_gb300 import scenes as G
    from gudni_gb300.raster import Rasterizer

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    tile, tpt = tile_override(args, *PLAIN_TILES["page4k"])
    spec = L.make_spec(max_tile_size=tile, threads_per_tile=tpt, max_thresholds=4096, max_shape=127,
                       stack_sections=8)
    flat = G.glyph_page(seed=1)
    host_ms = {1: [], 0: []}  # the sequential restatement, and its passes on all host threads
    for threads in (1, 0):
        for _ in range(max(1, min(args.steps, 5))):
            t0 = time.perf_counter()
            host = S.serialize_flat(flat, spec, threads=threads)
            host_ms[threads].append(1000 * (time.perf_counter() - t0))
    shapes, tiles, jobs = S.concatenated_piles(host)
    w, h = flat.canvas_w, flat.canvas_h
    r = Rasterizer(spec)
    apply_coop(r, args)
    r.upload_pictures(flat.pictures)
    r.upload_random_field(host.random_field)
    out = torch.zeros(w * h, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize()

    def render(df):
        r.raster_device_frame(df, w, h, flat.background, out.data_ptr(), stream=stream.cuda_stream)

    for _ in range(args.warmup):
        render(r.serialize_device(flat))
        stream.synchronize()
    r.sync_status()
    ser_ms, ren_ms, tot_ms = [], [], []
    launches0 = r.launch_count()
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            df = r.serialize_device(flat)  # returns once the piles are on the device
            t1 = time.perf_counter()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            render(df)
            b.record(stream)
            b.synchronize()
            t2 = time.perf_counter()
            ser_ms.append(1000 * (t1 - t0))
            ren_ms.append(a.elapsed_time(b))
            tot_ms.append(1000 * (t2 - t0))
    launches = r.launch_count() - launches0
    r.sync_status()
    got = r.download_device_frame(df)
    piles = {"geometry": got["geometry"].tobytes() == host.geometry.tobytes(),
             "shapes": got["shapes"].tobytes() == shapes.tobytes(),
             "tiles": got["tiles"].tobytes() == tiles.tobytes(),
             "tile_jobs": bool(np.array_equal(got["tile_jobs"], jobs))}
    img = out.cpu().numpy().view(np.uint32).reshape(h, w)
    ref = r.raster_frame(host)  # the host-serialized frame through the plain path
    r.close()
    ms = statistics.median(tot_ms)
    line = {"metric": WORKLOADS["scene4k"][1], "value": w * h / (ms / 1000) / 1e6, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS["scene4k"][0], "canvas": [w, h], "tile": tile,
                       "threads_per_tile": tpt, "shapes": int(host.stats["shapes"]),
                       "tiles": int(host.stats["tiles"]), "l2": "flushed between steps (256 MB write)",
                       "inputs": "flattened scene arrays in host memory, uploaded inside each step"},
            "device_serialize_ms": statistics.median(ser_ms), "render_ms": statistics.median(ren_ms),
            "host_serialize_ms": {"sequential": statistics.median(host_ms[1]),
                                  "parallel": statistics.median(host_ms[0]), "host_threads": os.cpu_count()},
            "host_serializer_scene_to_pixels_ms": statistics.median(host_ms[0]) + statistics.median(ren_ms),
            "gpu_launches": int(launches), "clocks": clocks.summary(),
            "parity": {"piles_identical_to_host_serializer": piles, "image_vs_host_frame": lsb_parity(img, ref)}}
    print(json.dumps(line))
    return 0


# 16x16 tiles of 64 threads (4-row column slices): of (32, 256), (16, 64) and (16, 128),
# the fastest fitting step on GB300 (1.68 s against 1.76 s and 2.02 s)
FIT_SPEC = dict(max_tile_size=16, threads_per_tile=64, max_thresholds=4096, max_shape=255,
                max_strands_per_tile=1 << 24)


def fit_scenes(n=64, side=256, shapes=128, jitter_px=0.0, color_sigma=0.0, seed=100):
    from gudni_gb300 import scenes as G
    out = []
    for i in range(n):
        f = G.random_shapes(seed=seed + i, width=side, height=side, n_shapes=shapes)
        if jitter_px or color_sigma:
            rng = np.random.default_rng(10_000 + seed + i)
            f.pairs = (f.pairs + rng.normal(0, jitter_px, f.pairs.shape)).astype(np.float32)
            c = f.substance_color + rng.normal(0, color_sigma, f.substance_color.shape)
            f.substance_color = np.clip(c, 0.0, 1.0).astype(np.float32)
        out.append(f)
    return out


def run_fit(args, emit=True):
    """Batched fitting: 64 independent 256x256 scenes of 128 shapes fitted by Adam (lr
    0.5 px on points, 0.01 on colours) to targets rendered from perturbed copies
    (points N(0, 4 px), colours N(0, 0.1)); each step serializes the scenes, runs every
    scene's forward and adjoint in one launch and updates every scene's points and
    colours by Adam on the device.  --fit-checkpoint / --fit-resume split a long fit
    over several processes (BatchFit.save / load)."""
    import torch
    from gudni_gb300 import adjoint as A
    from gudni_gb300 import fit as F
    from gudni_gb300 import lib as L
    from gudni_gb300 import scene as S
    from gudni_gb300.raster import Rasterizer

    torch.cuda.set_device(0)
    tile, tpt = tile_override(args, FIT_SPEC["max_tile_size"], FIT_SPEC["threads_per_tile"])
    fit_spec = {**FIT_SPEC, "max_tile_size": tile, "threads_per_tile": tpt}
    spec = L.make_spec(**fit_spec)
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    targets = []
    with Rasterizer(spec) as r:
        for f in fit_scenes(jitter_px=4.0, color_sigma=0.1):
            fa = A.FrameAdjoint(r, S.serialize_flat(f, spec))
            _, img, _, _ = fa.loss_and_gradient(np.zeros((f.canvas_h, f.canvas_w, 4), np.float32))
            targets.append(img.cpu().numpy())
    fit = F.BatchFit(fit_scenes(), targets, spec, lr_points=0.5, lr_colors=0.01)
    resume = getattr(args, "fit_resume", None)
    if resume:
        fit.load(resume)
    resumed_steps = fit.steps
    pixels = 64 * 256 * 256
    for _ in range(args.warmup):  # warm-up steps are fitting steps too; they are counted in `steps_total`
        fit.step()
    fit.timings = {k: 0.0 for k in fit.timings}  # the split below covers the timed steps only
    first = None
    total = getattr(args, "fit_total_steps", None)
    limit = getattr(args, "fit_time_limit", None)
    t0 = time.perf_counter()
    losses = []
    for k in range(args.steps):
        if (total is not None and fit.steps >= total) or (limit is not None and time.perf_counter() - t0 > limit):
            break
        loss = fit.step()
        losses.append(loss)
        if first is None:
            first = loss
        if k % max(1, args.steps // 10) == 0:
            log(f"step {fit.steps}: loss {loss:.4f} per-pixel L2 {loss / (pixels * 3):.6f}")
    wall = time.perf_counter() - t0
    steps = len(losses)
    if steps == 0:
        raise SystemExit("fit64: no timed step (the fit had already reached --fit-total-steps)")
    final = losses[-1]
    timings = dict(fit.timings)
    after = fit.evaluate()  # the loss after the last update (untimed)
    line = {"metric": WORKLOADS["fit64"][1], "value": steps / wall, "unit": "steps/s", "n_gpus": 1,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS["fit64"][0], "scenes": 64, "canvas": [256, 256], "shapes": 128,
                       **fit_spec, "lr_points_px": 0.5, "lr_colors": 0.01,
                       "targets": "perturbed copies: points N(0, 4 px), colours N(0, 0.1)",
                       "data": "synthetic, seeded"},
            "steps_total": fit.steps,
            "resumed_from_step": resumed_steps,
            "loss": {"first_timed": first, "final": final, "per_pixel_l2_first": first / (pixels * 3),
                     "per_pixel_l2_final": final / (pixels * 3),
                     "after_last_update": after, "per_pixel_l2_after_last_update": after / (pixels * 3),
                     "note": "each step's loss is taken before its update: `final` is the loss after "
                             "steps_total - 1 updates, `after_last_update` after steps_total"},
            "seconds": timings}
    checkpoint = getattr(args, "fit_checkpoint", None)
    if checkpoint:
        fit.save(checkpoint)
    if emit:
        print(json.dumps(line))
    fit.close()
    return line


def time_plain(workload: str, coop: str, steps: int) -> float:
    """Median ms of the workload's frame launch (gudni_raster_tiles_device, resident
    piles) with the given --cooperative-units choice; the image is checked against the
    per-column kernel's."""
    import torch
    from gudni_gb300 import scene as S
    from gudni_gb300.raster import Rasterizer
    frame = make_frame(workload, False, *PLAIN_TILES[workload])
    shapes, tiles, tile_jobs = S.concatenated_piles(frame)
    dev = torch.device("cuda", 0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    d_shapes = torch.from_numpy(shapes.view(np.uint8).copy()).to(dev)
    d_tiles = torch.from_numpy(tiles.view(np.uint8).copy()).to(dev)
    d_jobs = torch.from_numpy(tile_jobs.copy()).to(dev)
    d_out = torch.zeros(frame.canvas_w * frame.canvas_h, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(dev)
    with Rasterizer(frame.spec) as r:
        r.set_cooperative_units({"on": True, "off": False, "auto": None}[coop])
        r.upload_common(frame)
        torch.cuda.synchronize()

        def step():
            r.raster_tiles_device(frame, d_shapes.data_ptr(), len(shapes), d_tiles.data_ptr(), d_jobs.data_ptr(),
                                  len(tiles), d_out.data_ptr(), stream=stream.cuda_stream)

        for _ in range(3):
            step()
        ts = []
        for _ in range(steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            with torch.cuda.stream(stream):
                flush.zero_()
            b.synchronize()
            ts.append(a.elapsed_time(b))
        r.sync_status()
        img = d_out.cpu().numpy()
        r.set_cooperative_units(False)
        ref = r.raster_frame(frame).reshape(-1)
    if not np.array_equal(img.view(np.uint32), ref):
        raise RuntimeError(f"{workload}: the {coop} image differs from the per-column kernel's")
    return statistics.median(ts)


def form_records(args) -> dict:
    """The three systems forms beside the plain page, each run briefly (timed repeats
    stated in each record), as sub-records of the page's line: the batched form on the
    256-scene mix against the per-scene path over the same resident piles, fwd+adjoint
    against forward on the 1024x1024 scene with gradients checked against the FP64
    reference, and a few steps of the batched fitting.  A form that fails records its
    error instead."""
    import copy
    out = {}

    def guarded(name, fn):
        t0 = time.perf_counter()
        try:
            out[name] = fn()
        except Exception as e:  # noqa: BLE001
            out[name] = {"error": f"{type(e).__name__}: {e}"[:300]}
        out[name]["wall_s"] = time.perf_counter() - t0

    def batched():
        b = copy.copy(args)
        b.steps, b.warmup, b.scenes, b.plain_untimed_pass = 1, 1, 256, 0
        b.dense_columns = args.form_dense_columns
        ln = run_batch(b, emit=False)
        keys = ("metric", "value", "unit", "ms_per_step", "mpixels_per_s", "plain_per_scene", "batched_over_plain",
                "parity_vs_oracle", "gpu_launches", "clocks", "host_s")
        rec = {k: ln[k] for k in keys}
        rec.update(steps=1, warmup=1, timing="one batched pass timed after one warm-up pass (the graph is captured "
                   "in the warm-up); the per-scene path: every scene's launch pair timed alone, summed",
                   autotune=ln["config"]["autotune"], dense_columns=b.dense_columns,
                   scenes=ln["config"]["scenes"], pixels=ln["config"]["pixels"])
        return rec

    def adjoint():
        # the ratio depends on the spec (a slow forward flatters it): every spec of the
        # autotuner's candidates that fits the scene is timed, and the headline is the
        # spec with the fastest forward
        specs = []
        for tile, tpt in ((32, 256), (16, 64), (32, 32)):
            a = copy.copy(args)
            a.steps, a.warmup, a.tile, a.threads_per_tile = 3, 3, tile, tpt
            a.no_cpu_baseline = args.no_cpu_baseline or bool(specs)  # gradients checked on the first spec
            specs.append(run_adjoint(a, emit=False))
        best = min(specs, key=lambda ln: ln["forward_ms"])
        keys = ("metric", "value", "unit", "forward_ms", "fwd_adjoint_ms", "fwd_adjoint_over_forward",
                "thresholds", "regenerate", "gpu_launches", "clocks")
        rec = {k: best[k] for k in keys}
        rec.update(steps=3, warmup=3, timing="median of 3 timed launches of each", config=best["config"],
                   gradient_check=specs[0]["gradient_check"],
                   gradient_check_spec=[specs[0]["config"]["max_tile_size"], specs[0]["config"]["threads_per_tile"]],
                   by_spec=[{"tile": ln["config"]["max_tile_size"], "threads_per_tile": ln["config"]["threads_per_tile"],
                             "forward_ms": ln["forward_ms"], "fwd_adjoint_ms": ln["fwd_adjoint_ms"],
                             "fwd_adjoint_over_forward": ln["fwd_adjoint_over_forward"],
                             "regenerate_fwd_adjoint_ms": ln["regenerate"]["fwd_adjoint_ms"]} for ln in specs],
                   headline="the spec with the fastest forward")
        return rec

    def fitting():
        f = copy.copy(args)
        f.steps, f.warmup = args.fit_steps, 1
        f.tile = f.threads_per_tile = f.fit_resume = f.fit_checkpoint = None  # the fit's own spec, from step 0
        ln = run_fit(f, emit=False)
        keys = ("metric", "value", "unit", "ms_per_step", "loss", "steps_total", "seconds")
        rec = {k: ln[k] for k in keys}
        rec.update(steps=f.steps, warmup=1, note="a short run of --workload fit64 (the same step); the full "
                   "2000-step fit is --workload fit64 --steps 2000")
        return rec

    def cooperative():
        """The warp-cooperative units against the per-column kernel on the page and on
        the quarter page (device-resident piles, CUDA events, median of 5 launches)."""
        rec = {"timing": "median of 5 launches each after 3 warm-up launches, L2 flushed between launches"}
        for wl in ("page4k", "page1080"):
            ms = {m: time_plain(wl, m, 5) for m in ("off", "on")}
            rec[wl] = {"per_column_ms": ms["off"], "cooperative_ms": ms["on"],
                       "cooperative_over_per_column": ms["on"] / ms["off"]}
        return rec

    guarded("cooperative_units", cooperative)
    guarded("batched", batched)
    guarded("adjoint", adjoint)
    guarded("fit", fitting)
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch256":
        run_batch(args)
        return 0
    if args.workload == "adjoint1024":
        run_adjoint(args)
        return 0
    if args.workload == "fit64":
        run_fit(args)
        return 0
    if args.workload == "scene4k":
        return run_scene(args)
    if args.workload == "densest":
        return run_dense(args)

    import torch

    from gudni_gb300 import replicas as R

    rank, world, local = R.ranks()
    R.init(world, "nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from gudni_gb300 import lib as L
    from gudni_gb300 import scene as S
    from gudni_gb300.raster import Rasterizer

    frame = make_frame(args.workload, False, *tile_override(args, *PLAIN_TILES[args.workload]))
    shapes, tiles, tile_jobs = S.concatenated_piles(frame)
    r = Rasterizer(frame.spec, device=local)
    apply_coop(r, args)
    if args.device_strand_table:
        r.set_device_strand_table(True)
    if args.dense_columns:
        r.set_dense_columns(args.dense_columns)
    r.upload_common(frame)
    d_shapes = torch.from_numpy(shapes.view(np.uint8).copy()).to(dev)
    d_tiles = torch.from_numpy(tiles.view(np.uint8).copy()).to(dev)
    d_jobs = torch.from_numpy(tile_jobs.copy()).to(dev)
    d_out = torch.zeros(frame.canvas_w * frame.canvas_h, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # one dedicated stream for the kernels, the events and the L2 flushes
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize()  # inputs were copied on the default stream
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0

    def step():
        r.raster_tiles_device(frame, d_shapes.data_ptr(), len(shapes), d_tiles.data_ptr(), d_jobs.data_ptr(),
                              len(tiles), d_out.data_ptr(), stream=stream.cuda_stream)

    # one counted launch (untimed) for the work figures
    r.enable_counters(True)
    step()
    torch.cuda.synchronize()
    counters = r.read_counters()
    r.enable_counters(False)
    r.sync_status()

    for _ in range(args.warmup):
        step()
        flush.zero_()
    torch.cuda.synchronize()
    r.sync_status()

    def barrier():
        R.barrier(world)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = r.launch_count()
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            starts[i].record(stream)
            step()
            ends[i].record(stream)
            flush.zero_()  # L2 flush between timed steps (outside the events)
        torch.cuda.synchronize()
    barrier()
    launches = r.launch_count() - launches0
    r.sync_status()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = R.max_over_ranks(sum(step_ms) / len(step_ms), world, dev)
    pixels = frame.canvas_w * frame.canvas_h
    value = R.job_rate(pixels, world, ms / 1000) / 1e6

    # end to end through the frame-level C ABI with pinned host buffers
    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = a.view(np.uint8).reshape(-1)
        return t

    import copy
    hframe = copy.copy(frame)
    keep = []
    for name in ("geometry", "substances", "pictures", "picture_uses", "radials", "random_field"):
        a = getattr(frame, name)
        t = pinned(np.ascontiguousarray(a))
        keep.append(t)
        setattr(hframe, name, t.numpy().view(a.dtype).reshape(a.shape))
    hjobs = []
    for j in frame.jobs:
        ts, tt = pinned(j.shapes), pinned(j.tiles)
        keep += [ts, tt]
        hjobs.append(S.Job(ts.numpy().view(L.SHAPE_DTYPE), tt.numpy().view(L.TILE_DTYPE), j.columns))
    hframe.jobs = hjobs
    out_pin = torch.empty(pixels * 4, dtype=torch.uint8, pin_memory=True)
    out_np = out_pin.numpy().view(np.uint32).reshape(frame.canvas_h, frame.canvas_w)
    for _ in range(args.warmup):
        r.raster_frame(hframe, out=out_np)
    barrier()
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.raster_frame(hframe, out=out_np)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = R.max_over_ranks(sum(e2e_times) / len(e2e_times), world, dev)
    h2d = (frame.geometry.nbytes + frame.substances.nbytes + frame.pictures.nbytes + frame.picture_uses.nbytes +
           frame.radials.nbytes + frame.random_field.nbytes + shapes.nbytes + tiles.nbytes + tile_jobs.nbytes)
    e2e = {"value": world * pixels / e2e_s / 1e6, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(pixels * 4), "ms_per_step": 1000 * e2e_s,
           "call": "gudni_upload_common + gudni_raster_frame (host buffers)",
           "strand_table": "device" if args.device_strand_table else "host"}

    if rank != 0:
        r.close()
        return 0

    gpu_img = d_out.cpu().numpy().view(np.uint32).reshape(frame.canvas_h, frame.canvas_w)
    b_alg = algorithmic_bytes(frame, counters["texels"])
    peak, peak_src = measured_peaks()
    achieved = b_alg / (ms / 1000) / 1e9
    traffic, prof = profile_traffic(args.workload)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "algorithmic_bytes_per_launch": b_alg,
                "peak_source": f"{peak_src} (hbm_gbs burst)",
                "kernel": "raster_tiles_kernel (the fast pass: 99.8 % of a frame's device time; the frame's "
                          "three tile-order kernels and the full-capacity pass are inside the timed step)",
                "note": "the scan is divergent scalar FP32/INT work in serial per-column chains; SM issue and "
                        "the longest columns, not HBM, bound it"}
    if prof:
        roofline["profile"] = {k: prof[k] for k in prof if k != "dram_bytes_per_launch"}

    line = {"metric": WORKLOADS[args.workload][1], "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(config_dict(frame, args.workload), dense_columns=args.dense_columns,
                           cooperative_units=args.cooperative_units),
            "frames_per_s": 1000.0 / ms * world, "e2e": e2e, "gpu_launches": int(launches),
            "clocks": clocks.summary(), "roofline": roofline,
            "work": {"thresholds": counters["thresholds"], "sections": counters["sections"],
                     "texels": counters["texels"], "max_shape_bits": counters["max_shape_bits"],
                     "sections_per_s": counters["sections"] / (ms / 1000)},
            "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)}}
    if world == 1 and not args.no_cpu_baseline:
        v, kind, cores, img, dt, ref_parity = cpu_baseline(args.workload, frame, args.cpu_sample_frames)
        sample = f"{args.cpu_sample_frames} full frame(s), {dt:.2f} s each"
        if kind == "reference" and len(frame.radials):
            sample += "; radial gradients baked into pictures (the reference has no radial substance)"
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample,
                                "build": " ".join(ref_build_flags()) if kind == "reference" else None}
        line["parity_vs_oracle"] = lsb_parity(gpu_img, img)
        line["parity_reference_vs_oracle"] = ref_parity
    r.close()
    if world == 1 and args.workload == "page4k" and not args.no_forms:
        line.update(form_records(args))
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
