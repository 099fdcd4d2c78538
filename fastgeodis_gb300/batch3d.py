"""Batched 3D transforms: many volumes of uneven sizes, run concurrently.

The reference computes one volume per call (its C++ layer rejects batch != 1,
FastGeodis/common.h:89-95).  Here a list of volumes -- each
``[1, C, D, H, W]`` with its own soft mask ``[1, 1, D, H, W]``, spacing and
``lamb`` -- is computed together: the transforms are spread over a pool of
CUDA streams, and every pass whose cross-section fits one thread-block
cluster runs on a cluster plan (one cluster of up to 16 CTAs owns the whole
cross-section; neighbour rows travel through distributed shared memory), so
each transform takes a few SMs and the device holds several at once.  Per
volume the result is bit-identical to
:func:`fastgeodis_gb300.generalised_geodesic3d` /
:func:`fastgeodis_gb300.signed_generalised_geodesic3d`.

:class:`GeodesicBatch3d` fixes the shapes once, owns the buffers and the
workspaces, and replays the whole batch from one captured CUDA graph.

Plans are the engine's per cross-section (``fg_plan_override``): pinning a
batch's plans also applies to other calls with the same cross-sections in the
process, until :meth:`GeodesicBatch3d.release_plans`.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence, Union

import torch

from . import _lib, tune


def _check_item(image: torch.Tensor, mask: torch.Tensor, device) -> None:
    if image.dim() != 5 or mask.dim() != 5:
        raise ValueError("batch items must be [1, C, D, H, W] volumes with [1, 1, D, H, W] soft masks")
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


def batch_plan_for(key, channels: int = 1):
    """The plan a batch pins for a pass cross-section ``(2, N1, N2)``, as
    fg_plan_override arguments (S, T1, T2, flags), for throughput with many
    transforms at once: the fewest SMs that hold the section, each with as
    many cells as a CTA takes.  A section that fits one CTA gets one tile; a
    larger one the cluster plan with the most cells per CTA (the cluster
    sweep kernel where it applies); None if no cluster holds it (the cost
    model's tile plan)."""
    cross, N1, N2 = key
    lean_ok = channels <= 1
    runs = N1 * -(-N2 // 4)
    if runs <= tune.THREADS:
        return (8, N1, N2, 0)
    if lean_ok and runs <= tune.THREADS_LEAN:
        return (8, N1, N2, _lib.FG_PLAN_LEAN)
    cands = tune.cluster_candidates(cross, N1, N2, lean_capable=lean_ok, one_channel=lean_ok)
    if not cands:
        return None
    # most rows per strip (fewest CTAs), the cluster sweep kernel first on ties
    return max(cands, key=lambda c: (c[1], bool(c[3] & _lib.FG_PLAN_RUNS2)))


class GeodesicBatch3d:
    """A batch of fixed volume shapes with preallocated buffers.

    Args:
        shapes: list of ``(C, D, H, W)``.
        signed: compute ``D(M) - D(1 - M)`` instead of ``D(M)``.
        iterations: raster-scan iterations (the reference's ``iter``).
        device: CUDA device.
        use_graph: replay the batch from a captured CUDA graph.
        streams: size of the stream pool (transform i runs on stream
            i mod streams; transforms on one stream share its workspace).
        plans: ``"cluster"`` pins plans for concurrent transforms on the
            batch's pass cross-sections (:func:`batch_plan_for`: one CTA or
            one cluster each), ``"tune"`` measures candidate plans on the batch's
            own shapes with its concurrency (``tune.autotune``), ``None``
            leaves the engine's plans as they are.

    Fill ``images[i]`` / ``masks[i]`` (in place), set ``v`` / ``lambs`` /
    ``spacings``, call :meth:`run`; results are in ``outputs[i]``.
    """

    def __init__(self, shapes: Sequence[Sequence[int]], signed: bool = False, iterations: int = 4, device=None,
                 use_graph: bool = True, inputs=None, streams: int = 8, plans: Optional[str] = "cluster"):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.signed = bool(signed)
        self.iterations = int(iterations)
        self.shapes = [tuple(int(x) for x in s) for s in shapes]
        for s in self.shapes:
            if len(s) != 4 or min(s) < 1:
                raise ValueError(f"batch item shapes are (C, D, H, W) with positive extents, got {s}")
        if plans not in ("cluster", "tune", None):
            raise ValueError("plans must be 'cluster', 'tune' or None")
        n = len(self.shapes)
        dev = self.device
        L = _lib.load()
        with torch.cuda.device(dev):
            if inputs is not None:  # caller-owned tensors, used in place
                self.images, self.masks = list(inputs[0]), list(inputs[1])
            else:
                self.images = [torch.zeros((1,) + s, device=dev) for s in self.shapes]
                self.masks = [torch.ones((1, 1) + s[1:], device=dev) for s in self.shapes]
            self.outputs = [torch.empty((1, 1) + s[1:], device=dev) for s in self.shapes]
            self.streams = [torch.cuda.Stream(dev) for _ in range(max(1, min(int(streams), n)))]
            # largest first, so that the pool finishes with the short transforms
            self.order = sorted(range(n), key=lambda i: -self.shapes[i][1] * self.shapes[i][2] * self.shapes[i][3])
            op = _lib.FG_OP_SIGNED if self.signed else _lib.FG_OP_PLAIN
            need = [0] * len(self.streams)
            for slot, i in enumerate(self.order):
                C, D, H, W = self.shapes[i]
                k = slot % len(self.streams)
                need[k] = max(need[k], int(L.fg_workspace_bytes(op, C, D, H, W)))
            self._ws = [torch.zeros(max(b, 1 << 16), dtype=torch.uint8, device=dev) for b in need]
        self.v = 1e10
        self.lambs = [0.5] * n
        self.spacings = [(1.0, 1.0, 1.0)] * n
        self.use_graph = bool(use_graph)
        self._graph = None
        self._graph_key = None
        self._pinned = set()
        if plans == "cluster":
            self.pin_cluster_plans()
        elif plans == "tune":
            self.tune_plans()

    # --- plans ---
    def _keys(self):
        keys = {}
        for C, D, H, W in self.shapes:
            for k in tune.pass_keys((D, H, W)):
                keys[k] = max(keys.get(k, 1), C)
        return keys

    def pin_cluster_plans(self) -> None:
        """Pin a plan for every pass cross-section of the batch (batch_plan_for)."""
        L = _lib.load()
        for key, C in self._keys().items():
            c = batch_plan_for(key, C)
            if c is not None:
                _lib.check(L.fg_plan_override(*key, *c))
                self._pinned.add(key)
        self._graph = None

    def tune_plans(self, repeats: int = 2) -> None:
        """Measure and pin plans for each distinct volume shape, with as many
        transforms running at once as the batch runs."""
        conc = min(len(self.streams), len(self.shapes))
        for D, H, W in sorted({s[1:] for s in self.shapes}):
            C = max(s[0] for s in self.shapes if s[1:] == (D, H, W))
            tune.autotune((D, H, W), channels=C, lambs=[0.5] * conc, iterations=1, repeats=repeats,
                          device=self.device)
            self._pinned.update(tune.pass_keys((D, H, W)))
        self._graph = None

    def release_plans(self) -> None:
        """Remove the plan overrides this batch set."""
        L = _lib.load()
        for key in self._pinned:
            _lib.check(L.fg_plan_override(*key, 0, 0, 0, 0))
        self._pinned.clear()
        self._graph = None

    # --- execution ---
    def _launch(self):
        L = _lib.load()
        fn = L.fg_signed_generalised_geodesic3d if self.signed else L.fg_generalised_geodesic3d
        main = torch.cuda.current_stream(self.device)
        for s in self.streams:
            s.wait_stream(main)
        for slot, i in enumerate(self.order):
            k = slot % len(self.streams)
            C, D, H, W = self.shapes[i]
            lamb = float(self.lambs[i])
            sp = (ctypes.c_float * 3)(*[float(x) for x in self.spacings[i]])
            ws = self._ws[k]
            rc = fn(self.images[i].data_ptr(), C, D, H, W, self.masks[i].data_ptr(), 1, sp,
                    self.outputs[i].data_ptr(), float(self.v), lamb, 1.0 - lamb,  # FastGeodis/__init__.py:93-96
                    self.iterations, ws.data_ptr(), ws.numel(), int(self.streams[k].cuda_stream))
            _lib.check(rc)
        for s in self.streams:
            main.wait_stream(s)

    def run(self):
        """Compute all outputs (asynchronously on the current stream)."""
        if not self.shapes:
            return self.outputs
        with torch.cuda.device(self.device):
            key = (float(self.v), tuple(float(x) for x in self.lambs),
                   tuple(tuple(float(y) for y in s) for s in self.spacings))
            if key != self._graph_key:
                self._graph = None  # v, lambs and spacings are launch arguments
                self._graph_key = key
            if not self.use_graph:
                self._launch()
                return self.outputs
            if self._graph is None:
                self._launch()  # warm-up outside capture: kernel attributes and cluster checks are cached
                torch.cuda.synchronize(self.device)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._launch()
                self._graph = g
            self._graph.replay()
            return self.outputs

    def check(self) -> None:
        """Synchronise and raise if a kernel of the batch gave up a bounded wait."""
        L = _lib.load()
        with torch.cuda.device(self.device):
            torch.cuda.synchronize(self.device)
            for ws, s in zip(self._ws, self.streams):
                _lib.check(L.fg_workspace_status(ws.data_ptr(), int(s.cuda_stream)))


def _as_list(x, n, name) -> list:
    if isinstance(x, (list, tuple)) and len(x) > 0 and isinstance(x[0], (list, tuple)):
        if len(x) != n:
            raise ValueError(f"{name} must have one value per volume")
        return list(x)
    if isinstance(x, (list, tuple)) and name == "spacing":
        return [tuple(x)] * n
    if isinstance(x, (list, tuple)):
        if len(x) != n:
            raise ValueError(f"{name} must have one value per volume")
        return [float(a) for a in x]
    return [float(x)] * n


def _batch(images, softmasks, spacing, v, lamb, iterations, signed):
    if len(images) != len(softmasks):
        raise ValueError("images and softmasks must have the same length")
    if not images:
        return []
    device = images[0].device
    for im, m in zip(images, softmasks):
        _check_item(im, m, device)
    shapes = [tuple(int(x) for x in im.shape[1:]) for im in images]
    spacings = _as_list(spacing, len(images), "spacing")
    for sp in spacings:
        if len(sp) != 3:
            raise ValueError("length of spacing must be 3 (one entry per spatial dimension)")
    plan = GeodesicBatch3d(shapes, signed=signed, iterations=iterations, device=device, use_graph=False,
                           inputs=([im.contiguous() for im in images], [m.contiguous() for m in softmasks]),
                           plans=None)
    plan.v = float(v)
    plan.lambs = _as_list(lamb, len(images), "lamb")
    plan.spacings = spacings
    out = list(plan.run())
    plan.check()
    return out


def generalised_geodesic3d_batch(images: Sequence[torch.Tensor], softmasks: Sequence[torch.Tensor],
                                 spacing, v: float, lamb: Union[float, Sequence[float]],
                                 iter: int = 4) -> List[torch.Tensor]:
    """Batched :func:`generalised_geodesic3d`: one output ``[1, 1, D, H, W]``
    per volume; ``spacing`` is one (s_D, s_H, s_W) or one per volume, ``lamb``
    one value or one per volume.  Runs with the engine's current plans (pin
    cluster plans with :class:`GeodesicBatch3d` for concurrent volumes)."""
    return _batch(images, softmasks, spacing, v, lamb, iter, signed=False)


def signed_generalised_geodesic3d_batch(images: Sequence[torch.Tensor], softmasks: Sequence[torch.Tensor],
                                        spacing, v: float, lamb: Union[float, Sequence[float]],
                                        iter: int = 4) -> List[torch.Tensor]:
    """Batched :func:`signed_generalised_geodesic3d`."""
    return _batch(images, softmasks, spacing, v, lamb, iter, signed=True)
