"""Gradients of the per-pixel L2 loss through the raster path (no counterpart in the
reference, whose kernels only render).

  L = sum_p sum_{c in RGB} (I_c(p) - T_c(p))^2

with I(p) the pixel colour before the byte conversion (accumulated colour / area,
Kernels.cl:2017).  The CUDA adjoint (gudni_adjoint_tiles_device,
gudni_batch_adjoint) returns dL/d(every float of the geometry pile) and dL/d(every
substance colour); scene.pair_gradient carries the first back to the scene's curve
points through the serializer's point provenance.

Device memory is torch's; the kernels are libgudni_cuda.so's.  There is no CPU path.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np

from . import lib as L
from . import scene as S
from .raster import Rasterizer


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the adjoint needs a CUDA device")
    return torch


class FrameAdjoint:
    """One serialized frame resident on the device, ready for repeated adjoint calls.

    upload() puts the common piles and the concatenated job piles on the device;
    loss_and_gradient(target) enqueues one adjoint launch and returns torch tensors
    (loss, image (H, W, 4) float32 [I rgb, section area], grad_geometry
    (geometry_bytes/4,), grad_substances (n_substances, 4))."""

    def __init__(self, rasterizer: Rasterizer, frame: S.Frame):
        torch = _torch()
        self.r = rasterizer
        self.frame = frame
        self.dev = torch.device("cuda", torch.cuda.current_device())
        rasterizer.upload_common(frame)
        shapes, tiles, jobs = S.concatenated_piles(frame)
        self.n_shapes, self.n_tiles = len(shapes), len(tiles)
        self.shapes = torch.from_numpy(shapes.view(np.uint8).copy()).to(self.dev)
        self.tiles = torch.from_numpy(tiles.view(np.uint8).copy()).to(self.dev)
        self.tile_jobs = torch.from_numpy(jobs).to(self.dev)
        h, w = frame.canvas_h, frame.canvas_w
        self.image = torch.zeros((h, w, 4), dtype=torch.float32, device=self.dev)
        self.grad_geometry = torch.zeros(frame.geometry.size // 4, dtype=torch.float32, device=self.dev)
        self.grad_substances = torch.zeros((len(frame.substances), 4), dtype=torch.float32, device=self.dev)
        self.background = np.ascontiguousarray(frame.background, np.float32)

    def enqueue(self, target) -> None:
        """Zero the gradients and enqueue the adjoint, both on torch's current stream."""
        torch = _torch()
        f = self.frame
        self.grad_geometry.zero_()
        self.grad_substances.zero_()
        assert target.is_cuda and target.dtype == torch.float32 and target.is_contiguous()
        assert tuple(target.shape) == (f.canvas_h, f.canvas_w, 4)
        stream = L.current_stream_handle()
        self.r._check(self.r.lib.gudni_adjoint_tiles_device(
            self.r.ctx, self.shapes.data_ptr(), self.n_shapes, self.tiles.data_ptr(), self.tile_jobs.data_ptr(),
            self.n_tiles, f.canvas_w, f.canvas_h, f.compute_depth, self.background.ctypes.data, target.data_ptr(),
            self.image.data_ptr(), self.grad_geometry.data_ptr(), self.grad_substances.data_ptr(),
            stream or None))

    def loss_and_gradient(self, target):
        """One adjoint on torch's current stream; raises on a device-side error."""
        torch = _torch()
        if isinstance(target, np.ndarray):
            target = torch.from_numpy(np.ascontiguousarray(target, np.float32)).to(self.dev)
        if target.shape[-1] == 3:
            target = torch.cat([target, torch.zeros_like(target[..., :1])], -1).contiguous()
        self.enqueue(target)
        self.r.sync_status()
        d = self.image[..., :3] - target[..., :3]
        loss = (d.double() * d.double()).sum()
        return loss, self.image, self.grad_geometry, self.grad_substances


def frame_loss_and_gradient(rasterizer: Rasterizer, frame: S.Frame,
                            target: np.ndarray) -> Tuple[float, np.ndarray, np.ndarray, np.ndarray]:
    """Host-array convenience: (loss, grad_geometry, grad_substances (n, 4), image)."""
    fa = FrameAdjoint(rasterizer, frame)
    loss, img, gg, gs = fa.loss_and_gradient(target)
    return float(loss), gg.cpu().numpy(), gs.cpu().numpy(), img.cpu().numpy()


def pair_gradient(frame: S.Frame, grad_geometry) -> np.ndarray:
    """dL/d(scene curve pairs) from dL/d(geometry pile) (see scene.pair_gradient)."""
    if not isinstance(grad_geometry, np.ndarray):
        grad_geometry = grad_geometry.detach().cpu().numpy()
    return S.pair_gradient(frame, grad_geometry)


def target_from(image_rgb: np.ndarray, alpha: Optional[float] = 0.0) -> np.ndarray:
    """(H, W, 3) -> (H, W, 4) float32 target layout (alpha is not part of the loss)."""
    h, w = image_rgb.shape[:2]
    out = np.zeros((h, w, 4), np.float32)
    out[..., :3] = image_rgb
    out[..., 3] = alpha
    return out
