"""Batched fitting: many independent scenes fitted to per-scene target images by Adam
on their curve points and solid colours, with every scene's forward and adjoint in
one persistent launch per step (gudni_batch_adjoint).  No counterpart in the
reference, which only renders.

Each step serializes the current scenes (the serializer's point provenance maps the
geometry pile back to the scene's curve points), uploads them as one batch, runs the
adjoint of all scenes at once, carries the pile gradient to the points
(scene.pair_gradient) and updates points and colours with Adam on the host.  The
loss is the per-pixel L2 of the adjoint module over every scene.
"""
from __future__ import annotations

import os
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import adjoint as A
from . import batch as B
from . import lib as L
from . import scene as S


@dataclass
class Adam:
    lr: float
    beta1: float = 0.9
    beta2: float = 0.999
    eps: float = 1e-8
    m: np.ndarray = None
    v: np.ndarray = None
    t: int = 0

    def step(self, x: np.ndarray, g: np.ndarray) -> np.ndarray:
        if self.m is None:
            self.m = np.zeros_like(g, dtype=np.float64)
            self.v = np.zeros_like(g, dtype=np.float64)
        self.t += 1
        self.m = self.beta1 * self.m + (1 - self.beta1) * g
        self.v = self.beta2 * self.v + (1 - self.beta2) * g * g
        mh = self.m / (1 - self.beta1 ** self.t)
        vh = self.v / (1 - self.beta2 ** self.t)
        return x - self.lr * mh / (np.sqrt(vh) + self.eps)


class BatchFit:
    """Fit `flats` (modified in place) to `targets` ((H, W, 3 or 4) float per scene)."""

    def __init__(self, flats: Sequence[S.FlatScene], targets: Sequence[np.ndarray], spec: L.Spec,
                 lr_points: float = 0.5, lr_colors: float = 0.01, device: int = 0):
        import torch
        self.torch = torch
        self.spec = spec
        self.flats = list(flats)
        self.targets = [A.target_from(t[..., :3]) for t in targets]
        self.point_opt = [Adam(lr_points) for _ in self.flats]
        self.color_opt = [Adam(lr_colors) for _ in self.flats]
        self.r = B.BatchRasterizer(spec, device)
        self.dev = torch.device("cuda", device)
        self.timings = {"serialize": 0.0, "upload": 0.0, "device": 0.0, "update": 0.0}
        # the serializer is native code called without the interpreter lock: scenes
        # serialize in parallel
        self.pool = ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))
        self._target = None

    def close(self):
        self.pool.shutdown()
        self.r.close()

    def _target_tensor(self, batch: B.Batch):
        if self._target is None:
            t = np.zeros((batch.out_pixels, 4), np.float32)
            for i, tg in enumerate(self.targets):
                o = int(batch.frame_offsets[i])
                t[o:o + tg.shape[0] * tg.shape[1]] = tg.reshape(-1, 4)
            self._target = self.torch.from_numpy(t).to(self.dev)
        return self._target

    def step(self) -> float:
        """One Adam step over every scene; returns the summed loss before the step."""
        torch = self.torch
        t0 = time.perf_counter()
        # one scene per pool thread: each serialized on its own thread (threads=1)
        frames = list(self.pool.map(lambda f: S.serialize_flat(f, self.spec, threads=1), self.flats))
        batch = B.build_batch(frames)
        t1 = time.perf_counter()
        self.r.upload(batch)
        target = self._target_tensor(batch)
        image = torch.empty_like(target)
        gg = torch.zeros(batch.geometry.size // 4, dtype=torch.float32, device=self.dev)
        gs = torch.zeros((len(batch.substances), 4), dtype=torch.float32, device=self.dev)
        t2 = time.perf_counter()
        self.r.adjoint(target, image, gg, gs)
        self.r.sync_status()
        d = image[:, :3] - target[:, :3]
        loss = float((d.double() * d.double()).sum())
        gg, gs = gg.cpu().numpy(), gs.cpu().numpy()
        t3 = time.perf_counter()
        for i, (f, fr) in enumerate(zip(self.flats, frames)):
            sg, ss = self.r.frame_slices(i)
            gp = S.pair_gradient(fr, gg[sg]).reshape(f.pairs.shape)
            f.pairs = self.point_opt[i].step(f.pairs.astype(np.float64), gp).astype(np.float32)
            gc = gs[ss].astype(np.float64)
            solid = f.substance_kind == 0
            col = f.substance_color.astype(np.float64)
            new = self.color_opt[i].step(col, np.where(solid[:, None], gc, 0.0))
            f.substance_color = np.clip(new, 0.0, 1.0).astype(np.float32)
        t4 = time.perf_counter()
        self.timings["serialize"] += t1 - t0
        self.timings["upload"] += t2 - t1
        self.timings["device"] += t3 - t2
        self.timings["update"] += t4 - t3
        return loss
