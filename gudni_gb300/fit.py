"""Batched fitting: many independent scenes fitted to per-scene target images by Adam
on their curve points and solid colours, with every scene's forward and adjoint in
one persistent launch per step (gudni_batch_adjoint).  No counterpart in the
reference, which only renders.

Each step serializes the current scenes (the serializer's point provenance maps the
geometry pile back to the scene's curve points), uploads them as one batch and runs
the adjoint of all scenes at once; on the device it then carries the pile gradient to
the curve points (the provenance as gather and scatter-add, scene.pair_gradient's
arithmetic) and updates every scene's points and colours with one Adam over their
concatenation (Adam is elementwise, so this is each scene's own optimiser), and only
the updated points and colours come back for the next serialization.  The loss is the
per-pixel L2 of the adjoint module over every scene.
"""
from __future__ import annotations

import os
import time
from concurrent.futures import ThreadPoolExecutor
from typing import Sequence

import numpy as np

from . import adjoint as A
from . import batch as B
from . import lib as L
from . import scene as S


class DeviceAdam:
    """Adam (Kingma and Ba 2015) over one float64 device tensor of parameters."""

    def __init__(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        self.lr, self.beta1, self.beta2, self.eps = lr, beta1, beta2, eps
        self.m = self.v = None
        self.t = 0

    def step(self, x, g):
        if self.m is None:
            self.m = g.new_zeros(g.shape)
            self.v = g.new_zeros(g.shape)
        self.t += 1
        self.m.mul_(self.beta1).add_(g, alpha=1 - self.beta1)
        self.v.mul_(self.beta2).addcmul_(g, g, value=1 - self.beta2)
        mh = self.m / (1 - self.beta1 ** self.t)
        vh = self.v / (1 - self.beta2 ** self.t)
        return x - self.lr * mh / (vh.sqrt() + self.eps)


def pair_gradients(frames, frame_geo_offsets, pair_start, grad_geometry):
    """dL/d(curve pairs) of every scene of a batch at once, on grad_geometry's device:
    scene.pair_gradient's gather of each pile point's x and y and scatter-add through
    its provenance (up to three weighted source points), with every frame's pile
    offsets shifted to its place in the batch (frame_geo_offsets, bytes) and its pair
    indices to its place in the concatenated pairs (pair_start).  Returns a float64
    (total pairs, 4) tensor."""
    import torch
    offs, srcs, wts = [], [], []
    for i, fr in enumerate(frames):
        offs.append(fr.point_offsets.astype(np.int64) + int(frame_geo_offsets[i]) // 4)
        src = fr.point_sources.astype(np.int64)
        srcs.append(np.where(src >= 0, src + 2 * int(pair_start[i]), -1))
        wts.append(fr.point_weights.astype(np.float64))
    dev = grad_geometry.device
    off = torch.from_numpy(np.concatenate(offs)).to(dev)
    src = torch.from_numpy(np.concatenate(srcs).reshape(-1, 3)).to(dev)
    wt = torch.from_numpy(np.concatenate(wts).reshape(-1, 3)).to(dev)
    g64 = grad_geometry.double()
    gxy = torch.stack([g64[off], g64[off + 1]], 1)
    gp = torch.zeros((2 * int(pair_start[-1]), 2), dtype=torch.float64, device=dev)
    for j in range(3):
        m = src[:, j] >= 0
        gp.index_add_(0, src[m, j], wt[m, j, None] * gxy[m])
    return gp.reshape(-1, 4)


class BatchFit:
    """Fit `flats` (modified in place) to `targets` ((H, W, 3 or 4) float per scene)."""

    def __init__(self, flats: Sequence[S.FlatScene], targets: Sequence[np.ndarray], spec: L.Spec,
                 lr_points: float = 0.5, lr_colors: float = 0.01, device: int = 0):
        import torch
        self.torch = torch
        self.spec = spec
        self.flats = list(flats)
        self.targets = [A.target_from(t[..., :3]) for t in targets]
        self.point_opt = DeviceAdam(lr_points)
        self.color_opt = DeviceAdam(lr_colors)
        # every scene's curve pairs and colours, concatenated, in float64 on the device
        self.pair_start = np.cumsum([0] + [len(f.pairs) for f in self.flats])
        self.sub_start = np.cumsum([0] + [len(f.substance_color) for f in self.flats])
        self.r = B.BatchRasterizer(spec, device)
        self.dev = torch.device("cuda", device)
        self.timings = {"serialize": 0.0, "upload": 0.0, "device": 0.0, "update": 0.0}
        # the serializer is native code called without the interpreter lock: scenes
        # serialize in parallel
        self.pool = ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))
        self._target = None
        self.steps = 0  # Adam steps taken, including those before a `load`

    def close(self):
        self.pool.shutdown()
        self.r.close()

    def save(self, path: str) -> None:
        """Write the fit's state (every scene's curve pairs and colours, both Adam
        moments and step counts, the steps taken) to an .npz file, so that a long fit
        can continue in another process with `load`."""
        def moments(opt):
            if opt.m is None:
                return np.zeros(0), np.zeros(0)
            return opt.m.cpu().numpy(), opt.v.cpu().numpy()
        pm, pv = moments(self.point_opt)
        cm, cv = moments(self.color_opt)
        np.savez(path, pairs=np.concatenate([f.pairs for f in self.flats]),
                 colors=np.concatenate([f.substance_color for f in self.flats]),
                 pair_start=self.pair_start, sub_start=self.sub_start,
                 point_m=pm, point_v=pv, point_t=self.point_opt.t,
                 color_m=cm, color_v=cv, color_t=self.color_opt.t, steps=self.steps)

    def load(self, path: str) -> None:
        """Continue from a state written by `save` for the same scenes (same curve and
        substance counts per scene); raises ValueError for another set of scenes."""
        z = np.load(path)
        if not (np.array_equal(z["pair_start"], self.pair_start) and np.array_equal(z["sub_start"], self.sub_start)):
            raise ValueError("checkpoint was written for other scenes")
        for i, f in enumerate(self.flats):
            f.pairs = z["pairs"][self.pair_start[i]:self.pair_start[i + 1]].astype(np.float32)
            f.substance_color = z["colors"][self.sub_start[i]:self.sub_start[i + 1]].astype(np.float32)
        for opt, key in ((self.point_opt, "point"), (self.color_opt, "color")):
            opt.t = int(z[key + "_t"])
            m = z[key + "_m"]
            if m.size:
                opt.m = self.torch.from_numpy(m).to(self.dev)
                opt.v = self.torch.from_numpy(z[key + "_v"]).to(self.dev)
            else:
                opt.m = opt.v = None
        self.steps = int(z["steps"])

    def _sub_slice(self, i: int):
        """(start, stop) of scene i's substances in the batch's substance pile."""
        _, ss = self.r.frame_slices(i)
        return ss.start, ss.stop

    def _target_tensor(self, batch: B.Batch):
        if self._target is None:
            t = np.zeros((batch.out_pixels, 4), np.float32)
            for i, tg in enumerate(self.targets):
                o = int(batch.frame_offsets[i])
                t[o:o + tg.shape[0] * tg.shape[1]] = tg.reshape(-1, 4)
            self._target = self.torch.from_numpy(t).to(self.dev)
        return self._target

    def evaluate(self) -> float:
        """The summed loss of the current scenes (no update)."""
        return self._forward()[-1]

    def _forward(self):
        """Serialize, upload and run every scene's forward and adjoint: (frames, batch,
        pile gradient, substance gradient, summed loss)."""
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
        t3 = time.perf_counter()
        self.timings["serialize"] += t1 - t0
        self.timings["upload"] += t2 - t1
        self.timings["device"] += t3 - t2
        return frames, batch, gg, gs, loss

    def step(self) -> float:
        """One Adam step over every scene; returns the summed loss before the step."""
        torch = self.torch
        frames, batch, gg, gs, loss = self._forward()
        t3 = time.perf_counter()
        dev = self.dev
        gp = pair_gradients(frames, batch.frame_geo_offsets, self.pair_start, gg)
        pairs = torch.from_numpy(np.concatenate([f.pairs for f in self.flats]).astype(np.float64)).to(dev)
        pairs = self.point_opt.step(pairs, gp)
        # colours: solid substances only (a texture's colour slot holds no colour)
        subs = torch.cat([gs[slice(*self._sub_slice(i))] for i in range(len(self.flats))]).double()
        solid = torch.from_numpy(np.concatenate([f.substance_kind == 0 for f in self.flats])).to(dev)
        cols = torch.from_numpy(np.concatenate([f.substance_color for f in self.flats]).astype(np.float64)).to(dev)
        cols = self.color_opt.step(cols, torch.where(solid[:, None], subs, torch.zeros_like(subs)))
        cols = cols.clamp_(0.0, 1.0).float().cpu().numpy()
        pairs = pairs.float().cpu().numpy()
        for i, f in enumerate(self.flats):
            f.pairs = pairs[self.pair_start[i]:self.pair_start[i + 1]].copy()
            f.substance_color = cols[self.sub_start[i]:self.sub_start[i + 1]].copy()
        self.timings["update"] += time.perf_counter() - t3
        self.steps += 1
        return loss
