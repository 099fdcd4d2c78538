"""Batched 2D transforms: many images of uneven sizes in one persistent launch.

The reference computes one image per call (its C++ layer rejects batch != 1,
FastGeodis/common.h:89-95).  Here a list of images -- each ``[1, C, H, W]``
with its own soft mask ``[1, 1, H, W]`` and its own ``lamb`` -- goes into a
single kernel launch whose CTAs pull images from a work queue, largest first,
and run each image's whole transform.  Per image the result is bit-identical
to :func:`fastgeodis_gb300.generalised_geodesic2d` /
:func:`fastgeodis_gb300.signed_generalised_geodesic2d`.

:class:`GeodesicBatch2d` fixes the shapes once, owns the buffers and replays
the launch from a captured CUDA graph.
"""
from __future__ import annotations

from typing import List, Optional, Sequence, Union

import numpy as np
import torch

from . import _lib

# fg_batch2d_item (include/fastgeodis_gb300.h)
ITEM_DTYPE = np.dtype([
    ("image", np.uint64), ("mask", np.uint64), ("out", np.uint64), ("image_t", np.uint64),
    ("d2", np.uint64), ("t1", np.uint64), ("t2", np.uint64),
    ("C", np.int32), ("H", np.int32), ("W", np.int32), ("reserved0", np.int32),
    ("v", np.float32), ("l_grad", np.float32), ("l_eucl", np.float32), ("reserved1", np.float32),
])
assert ITEM_DTYPE.itemsize == 88

MAX_SIDE = 2048
MAX_CHANNELS = 4


def _check_item(image: torch.Tensor, mask: torch.Tensor, device) -> None:
    if image.dim() != 4 or mask.dim() != 4:
        raise ValueError("batch items must be [1, C, H, W] images with [1, 1, H, W] soft masks")
    if image.size(0) != 1 or mask.size(0) != 1:
        raise ValueError("FastGeodis currently only supports single batch input.")
    if image.shape[2:] != mask.shape[2:]:
        raise ValueError("shapes of input tensors do not match")
    if mask.size(1) != 1:
        raise ValueError("batched transforms take single-channel soft masks")
    if image.dtype != torch.float32 or mask.dtype != torch.float32:
        raise RuntimeError("expected scalar type Float")
    if not (image.is_cuda and mask.is_cuda) or image.device != device or mask.device != device:
        raise ValueError("all batch tensors must be CUDA tensors on one device")
    C, H, W = image.shape[1], image.shape[2], image.shape[3]
    if C > MAX_CHANNELS or max(H, W) > MAX_SIDE:
        raise RuntimeError(f"batched transforms handle up to {MAX_CHANNELS} channels and sides up to {MAX_SIDE}")


class GeodesicBatch2d:
    """A batch of fixed shapes with preallocated buffers.

    Args:
        shapes: list of ``(C, H, W)``.
        signed: compute ``D(M) - D(1 - M)`` instead of ``D(M)``.
        iterations: raster-scan iterations (the reference's ``iter``).
        device: CUDA device.
        use_graph: replay the launch from a captured CUDA graph.

    Fill ``images[i]`` / ``masks[i]`` (in place), set ``v`` / ``lambs``, call
    :meth:`run`; results are in ``outputs[i]``.
    """

    def __init__(self, shapes: Sequence[Sequence[int]], signed: bool = False, iterations: int = 2,
                 device=None, use_graph: bool = True, inputs=None):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.signed = bool(signed)
        self.iterations = int(iterations)
        self.shapes = [tuple(int(x) for x in s) for s in shapes]
        for C, H, W in self.shapes:
            if C < 1 or C > MAX_CHANNELS or max(H, W) > MAX_SIDE or min(H, W) < 0:
                raise RuntimeError(f"unsupported batch item shape {(C, H, W)}")
        dev = self.device
        if inputs is not None:  # caller-owned tensors, used in place
            self.images, self.masks = list(inputs[0]), list(inputs[1])
        else:
            self.images = [torch.zeros((1, C, H, W), device=dev) for C, H, W in self.shapes]
            self.masks = [torch.ones((1, 1, H, W), device=dev) for _, H, W in self.shapes]
        self.outputs = [torch.empty((1, 1, H, W), device=dev) for _, H, W in self.shapes]
        self._scratch = []
        for C, H, W in self.shapes:
            s = {"image_t": torch.empty((C, W, H), device=dev), "t1": torch.empty((W, H), device=dev)}
            if self.signed:
                s["d2"] = torch.empty((H, W), device=dev)
                s["t2"] = torch.empty((W, H), device=dev)
            self._scratch.append(s)
        n = len(self.shapes)
        # largest first: the queue then finishes with the short jobs
        self.order = sorted(range(n), key=lambda i: -(self.shapes[i][1] + self.shapes[i][2]) *
                            max(self.shapes[i][1], self.shapes[i][2]))
        self._items_host = np.zeros(n, dtype=ITEM_DTYPE)
        self._items_dev = torch.empty(max(1, n * ITEM_DTYPE.itemsize), dtype=torch.uint8, device=dev)
        self._counter = torch.zeros(2, dtype=torch.int32, device=dev)
        self.max_C = max([s[0] for s in self.shapes], default=1)
        self.max_extent = max([max(s[1], s[2]) for s in self.shapes], default=1)
        self.v = 1e10
        self.lambs = [1.0] * n
        self._graph = None
        self._graph_key = None
        self.use_graph = bool(use_graph)

    def _fill_items(self):
        it = self._items_host
        for slot, i in enumerate(self.order):
            C, H, W = self.shapes[i]
            s = self._scratch[i]
            lamb = float(self.lambs[i])
            it[slot]["image"] = self.images[i].data_ptr()
            it[slot]["mask"] = self.masks[i].data_ptr()
            it[slot]["out"] = self.outputs[i].data_ptr()
            it[slot]["image_t"] = s["image_t"].data_ptr()
            it[slot]["t1"] = s["t1"].data_ptr()
            it[slot]["d2"] = s["d2"].data_ptr() if self.signed else 0
            it[slot]["t2"] = s["t2"].data_ptr() if self.signed else 0
            it[slot]["C"], it[slot]["H"], it[slot]["W"] = C, H, W
            it[slot]["v"] = np.float32(self.v)
            it[slot]["l_grad"] = np.float32(lamb)
            it[slot]["l_eucl"] = np.float32(1.0 - lamb)  # FastGeodis/__init__.py:63-65
        host = torch.from_numpy(it.view(np.uint8).copy())
        self._items_dev[: host.numel()].copy_(host, non_blocking=False)

    def _launch(self):
        L = _lib.load()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        cnt = self._counter
        rc = L.fg_batch_geodesic2d(self._items_dev.data_ptr(), len(self.shapes), self.max_C, self.max_extent,
                                   1 if self.signed else 0, self.iterations, cnt.data_ptr(),
                                   cnt.data_ptr() + 4, stream)
        _lib.check(rc)

    def run(self):
        """Compute all outputs (asynchronously on the current stream)."""
        if not self.shapes:
            return self.outputs
        with torch.cuda.device(self.device):
            key = (float(self.v), tuple(float(x) for x in self.lambs))
            if key != self._graph_key:
                self._fill_items()  # descriptors change only with v / lambs
                self._graph = None
                self._graph_key = key
            if not self.use_graph:
                self._launch()
                return self.outputs
            if self._graph is None:
                side = torch.cuda.Stream(self.device)
                side.wait_stream(torch.cuda.current_stream(self.device))
                with torch.cuda.stream(side):
                    self._launch()  # warm-up outside capture (function attributes, module load)
                torch.cuda.current_stream(self.device).wait_stream(side)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._launch()
                self._graph = g
            self._graph.replay()
            return self.outputs


def _as_list(x, n, name) -> List[float]:
    if isinstance(x, (list, tuple)):
        if len(x) != n:
            raise ValueError(f"{name} must have one value per image")
        return [float(a) for a in x]
    return [float(x)] * n


def _batch(images, softmasks, v, lamb, iterations, signed):
    if len(images) != len(softmasks):
        raise ValueError("images and softmasks must have the same length")
    if not images:
        return []
    device = images[0].device
    for im, m in zip(images, softmasks):
        _check_item(im, m, device)
    shapes = [(int(im.shape[1]), int(im.shape[2]), int(im.shape[3])) for im in images]
    plan = GeodesicBatch2d(shapes, signed=signed, iterations=iterations, device=device, use_graph=False,
                           inputs=([im.contiguous() for im in images], [m.contiguous() for m in softmasks]))
    plan.v = float(v)
    plan.lambs = _as_list(lamb, len(images), "lamb")
    return list(plan.run())


def generalised_geodesic2d_batch(images: Sequence[torch.Tensor], softmasks: Sequence[torch.Tensor], v: float,
                                 lamb: Union[float, Sequence[float]], iter: int = 2) -> List[torch.Tensor]:
    """Batched :func:`generalised_geodesic2d`: one output ``[1, 1, H, W]`` per
    image; ``lamb`` is one value or one per image."""
    return _batch(images, softmasks, v, lamb, iter, signed=False)


def signed_generalised_geodesic2d_batch(images: Sequence[torch.Tensor], softmasks: Sequence[torch.Tensor], v: float,
                                        lamb: Union[float, Sequence[float]], iter: int = 2) -> List[torch.Tensor]:
    """Batched :func:`signed_generalised_geodesic2d`."""
    return _batch(images, softmasks, v, lamb, iter, signed=True)
