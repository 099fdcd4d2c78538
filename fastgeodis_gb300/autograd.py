"""Differentiable generalised geodesic distance (2D) behind torch.autograd.

The reference has no gradient.  The transform is a min-plus recurrence, so
its derivative is piecewise constant: every output cell's value is
``v * mask(x0) + Σ step costs`` along its optimal path.  The forward kernel
records which candidate won at every cell of every pass (a one-byte argmin
tape); the backward kernel walks the passes in reverse and routes
``dLoss/dD`` along the recorded choices:

* to the soft mask: ``dLoss/dmask = v * dLoss/dD0`` at each path's source;
* to the image: every step taken adds ``± l_grad * sign(I - I')`` per channel
  (the derivative of ``l_grad * |I - I'|``, with sign(0) = 0).

Forward values are bit-identical to :func:`generalised_geodesic2d`.

When memory is short, ``recompute=True`` keeps the tape of a single pass (1
byte per pixel instead of 4 per iteration) plus one scratch distance map, and
the backward recomputes the forward up to each pass before applying that
pass's adjoint (about (4 * iterations + 1) / 2 times the forward work); the
gradients are the same bits.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib

# fg_grad2d_item (include/fastgeodis_gb300.h)
GRAD_ITEM_DTYPE = np.dtype([
    ("image", np.uint64), ("mask", np.uint64), ("out", np.uint64), ("image_t", np.uint64), ("t1", np.uint64),
    ("tape", np.uint64), ("g_out", np.uint64), ("g_image", np.uint64), ("g_mask", np.uint64),
    ("g_r", np.uint64), ("g_t", np.uint64), ("gi_t", np.uint64),
    ("C", np.int32), ("H", np.int32), ("W", np.int32), ("reserved0", np.int32),
    ("v", np.float32), ("l_grad", np.float32), ("l_eucl", np.float32), ("reserved1", np.float32),
])
assert GRAD_ITEM_DTYPE.itemsize == 128


class _Buffers:
    def __init__(self, image, softmask, v, lamb, iterations, recompute=False):
        B, C, H, W = image.shape
        dev = image.device
        self.shape = (B, C, H, W)
        self.iterations = int(iterations)
        self.recompute = bool(recompute)
        self.image = image
        self.mask = softmask
        self.out = torch.empty((B, 1, H, W), device=dev)
        self.image_t = torch.empty((B, C, W, H), device=dev)
        self.t1 = torch.empty((B, W, H), device=dev)
        tape_passes = 1 if self.recompute else max(1, self.iterations) * 4
        self.tape = torch.empty((B, tape_passes * H * W), dtype=torch.uint8, device=dev)
        self.scratch = torch.empty((B, 1, H, W), device=dev) if self.recompute else None
        self.counter = torch.zeros(2, dtype=torch.int32, device=dev)
        self.items = np.zeros(B, dtype=GRAD_ITEM_DTYPE)
        P = H * W
        b = np.arange(B, dtype=np.uint64)
        it = self.items
        it["image"] = np.uint64(image.data_ptr()) + b * np.uint64(C * P * 4)
        it["mask"] = np.uint64(softmask.data_ptr()) + b * np.uint64(P * 4)
        it["out"] = np.uint64(self.out.data_ptr()) + b * np.uint64(P * 4)
        it["image_t"] = np.uint64(self.image_t.data_ptr()) + b * np.uint64(C * P * 4)
        it["t1"] = np.uint64(self.t1.data_ptr()) + b * np.uint64(P * 4)
        it["tape"] = np.uint64(self.tape.data_ptr()) + b * np.uint64(self.tape.shape[1])
        it["C"], it["H"], it["W"] = C, H, W
        it["v"] = np.float32(v)
        it["l_grad"] = np.float32(lamb)
        it["l_eucl"] = np.float32(1.0 - float(lamb))  # FastGeodis/__init__.py:63-65
        self.dev = dev
        self._pinned = []  # host copies of uploaded descriptors, alive until their copies are done

    def upload(self, items=None):
        """Descriptors to the device without a host synchronisation: pinned
        host memory, asynchronous copy on the current stream."""
        arr = self.items if items is None else items
        host = torch.from_numpy(arr.view(np.uint8).copy()).pin_memory()
        self._pinned.append(host)
        return host.to(self.dev, non_blocking=True)

    @property
    def npass(self):
        return 4 * self.iterations

    def forward(self):
        B, C, H, W = self.shape
        L = _lib.load()
        items = self.upload()
        stream = torch.cuda.current_stream(self.dev).cuda_stream
        if self.recompute and self.iterations > 0:
            # all passes, recording only the last one's tape
            rc = L.fg_grad_geodesic2d_forward_pass(items.data_ptr(), B, C, max(H, W), self.npass - 1,
                                                   self.counter.data_ptr(), self.counter.data_ptr() + 4, stream)
        else:
            rc = L.fg_grad_geodesic2d_forward(items.data_ptr(), B, C, max(H, W), self.iterations,
                                              self.counter.data_ptr(), self.counter.data_ptr() + 4, stream)
        _lib.check(rc)
        self._keep = items
        return self.out

    def backward(self, g_out):
        B, C, H, W = self.shape
        dev = self.dev
        P = H * W
        g_out = g_out.contiguous()
        g_image = torch.empty((B, C, H, W), device=dev)
        g_mask = torch.empty((B, 1, H, W), device=dev)
        g_r = torch.empty((B, H, W), device=dev)
        g_t = torch.empty((B, W, H), device=dev)
        gi_t = torch.empty((B, C, W, H), device=dev)
        b = np.arange(B, dtype=np.uint64)
        it = self.items
        it["g_out"] = np.uint64(g_out.data_ptr()) + b * np.uint64(P * 4)
        it["g_image"] = np.uint64(g_image.data_ptr()) + b * np.uint64(C * P * 4)
        it["g_mask"] = np.uint64(g_mask.data_ptr()) + b * np.uint64(P * 4)
        it["g_r"] = np.uint64(g_r.data_ptr()) + b * np.uint64(P * 4)
        it["g_t"] = np.uint64(g_t.data_ptr()) + b * np.uint64(P * 4)
        it["gi_t"] = np.uint64(gi_t.data_ptr()) + b * np.uint64(C * P * 4)
        L = _lib.load()
        items = self.upload()
        stream = torch.cuda.current_stream(dev).cuda_stream
        cnt, st = self.counter.data_ptr(), self.counter.data_ptr() + 4
        if not self.recompute or self.iterations <= 0:
            rc = L.fg_grad_geodesic2d_backward(items.data_ptr(), B, C, max(H, W), self.iterations, cnt, st, stream)
            _lib.check(rc)
            self._keep_b = (items, g_out, g_r, g_t, gi_t)
            return g_image, g_mask
        # recompute into scratch distance maps, so the forward output stays intact
        re = self.items.copy()
        re["out"] = np.uint64(self.scratch.data_ptr()) + np.arange(B, dtype=np.uint64) * np.uint64(H * W * 4)
        re_dev = self.upload(re)
        last = self.npass - 1
        for p in range(last, -1, -1):
            if p < last:  # the forward's tape holds the last pass; recompute the others
                _lib.check(L.fg_grad_geodesic2d_forward_pass(re_dev.data_ptr(), B, C, max(H, W), p, cnt, st, stream))
            _lib.check(L.fg_grad_geodesic2d_backward_pass(items.data_ptr(), B, C, max(H, W), p, int(p == last),
                                                          int(p == 0), cnt, stream))
        self._keep_b = (items, re_dev, g_out, g_r, g_t, gi_t)
        return g_image, g_mask


class GeneralisedGeodesic2dFunction(torch.autograd.Function):
    """autograd Function: (image [B,C,H,W], softmask [B,1,H,W]) -> D [B,1,H,W]."""

    @staticmethod
    def forward(ctx, image, softmask, v, lamb, iterations, recompute=False):
        buf = _Buffers(image, softmask, v, lamb, iterations, recompute)
        out = buf.forward()
        ctx.buf = buf
        return out

    @staticmethod
    def backward(ctx, g_out):
        g_image, g_mask = ctx.buf.backward(g_out)
        return g_image, g_mask, None, None, None, None


def generalised_geodesic2d_differentiable(image: torch.Tensor, softmask: torch.Tensor, v: float, lamb: float,
                                          iter: int = 2, recompute: bool = False) -> torch.Tensor:
    """Differentiable generalised geodesic distance of a batch of 2D images.

    Args:
        image: ``[B, C, H, W]`` float32 CUDA tensor (C <= 4, sides <= 2048).
        softmask: ``[B, 1, H, W]`` float32 CUDA tensor.
        v, lamb, iter: as in :func:`generalised_geodesic2d`.
        recompute: keep one pass's argmin tape instead of all of them and
            recompute the forward during the backward (less memory, more work,
            the same gradients).

    Returns ``[B, 1, H, W]``; gradients flow to ``image`` and ``softmask``.
    """
    if image.dim() != 4 or softmask.dim() != 4 or softmask.size(1) != 1:
        raise ValueError("expected image [B, C, H, W] and softmask [B, 1, H, W]")
    if image.shape[0] != softmask.shape[0] or image.shape[2:] != softmask.shape[2:]:
        raise ValueError("shapes of input tensors do not match")
    if image.dtype != torch.float32 or softmask.dtype != torch.float32:
        raise RuntimeError("expected scalar type Float")
    if not (image.is_cuda and softmask.is_cuda) or image.device != softmask.device:
        raise ValueError("image and softmask must be CUDA tensors on one device")
    if image.size(1) > 4 or max(image.shape[2], image.shape[3]) > 2048:
        raise RuntimeError("differentiable transforms handle up to 4 channels and sides up to 2048")
    with torch.cuda.device(image.device):
        return GeneralisedGeodesic2dFunction.apply(image.contiguous(), softmask.contiguous(), float(v),
                                                   float(lamb), int(iter), bool(recompute))
