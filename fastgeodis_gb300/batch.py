"""Batched 2D transforms: many images of uneven sizes in one persistent launch.

The reference computes one image per call (its C++ layer rejects batch != 1,
FastGeodis/common.h:89-95).  Here a list of images -- each ``[1, C, H, W]``
with its own soft mask ``[1, 1, H, W]``, its own ``lamb`` and its own form
(plain or signed) -- goes into a single kernel launch whose CTAs pull jobs
from a work queue, largest first, and run each job whole.  A signed image is
one job (both distance maps in one CTA) or, when that job would set the
batch's critical path, two (one map each, on two CTAs).  Per image the result
is bit-identical to :func:`fastgeodis_gb300.generalised_geodesic2d` /
:func:`fastgeodis_gb300.signed_generalised_geodesic2d`.

:class:`GeodesicBatch2d` fixes the shapes once, owns the buffers and replays
the launch from a captured CUDA graph.

Images the persistent kernel does not take -- more than four channels, or a
side above 2048 -- are accepted too: they run through the per-call engine
(``fg_generalised_geodesic2d`` / ``fg_signed_generalised_geodesic2d``) on a
side stream beside the launch, outside the captured graph, with the same
bits as a single call.
"""
from __future__ import annotations

import ctypes
from typing import List, Sequence, Tuple, Union

import numpy as np
import torch

from . import _lib

# fg_batch2d_item (include/fastgeodis_gb300.h)
ITEM_DTYPE = np.dtype([
    ("image", np.uint64), ("mask", np.uint64), ("out", np.uint64), ("image_t", np.uint64),
    ("d2", np.uint64), ("t1", np.uint64), ("t2", np.uint64),
    ("C", np.int32), ("H", np.int32), ("W", np.int32), ("flags", np.int32),
    ("v", np.float32), ("l_grad", np.float32), ("l_eucl", np.float32), ("reserved1", np.float32),
])
assert ITEM_DTYPE.itemsize == 88
FG_BATCH_SIGNED, FG_BATCH_SPLIT, FG_BATCH_SECOND = 1, 2, 4

MAX_SIDE = 2048
MAX_CHANNELS = 4

# Microseconds per raster step of one job (one CTA sweeps a whole row per
# step) by (channels, maps), at rows of STEP_ROWS cells: measured on a GB300
# with square images, 2 iterations.
STEP_ROWS = (256, 512, 1024, 2048)
STEP_US = {
    (1, 1): (0.3196, 0.3633, 0.5081, 0.921),
    (1, 2): (0.3973, 0.4968, 0.7373, 1.7835),
    (2, 1): (0.3699, 0.4594, 0.6665, 1.4057),
    (2, 2): (0.4706, 0.5834, 0.9154, 2.3594),
    (3, 1): (0.4124, 0.5212, 0.8246, 2.0833),
    (3, 2): (0.5316, 0.667, 1.071, 2.8031),
    (4, 1): (0.4831, 0.6196, 0.9951, 2.5186),
    (4, 2): (0.5957, 0.7626, 1.2446, 3.8202),
}


def step_us(C: int, maps: int, row: int) -> float:
    """Estimated microseconds of one step over a row of `row` cells."""
    t = STEP_US[(min(max(C, 1), MAX_CHANNELS), maps)]
    return float(np.interp(row, STEP_ROWS, t))


def job_cost(C: int, H: int, W: int, maps: int, iterations: int) -> float:
    """Estimated microseconds of one job: per iteration two passes of H steps
    over rows of W cells and two of W steps over rows of H cells."""
    return 2.0 * max(iterations, 1) * (H * step_us(C, maps, W) + W * step_us(C, maps, H))


def plan_jobs(shapes: Sequence[Tuple[int, int, int]], signed: Sequence[bool], iterations: int, sms: int,
              split: Union[str, bool] = "auto") -> List[Tuple[int, int]]:
    """Queue order of the batch's jobs, largest first: ``(image, part)`` with
    part 0 for a whole image (plain, or signed with both maps in one CTA) and
    1 / 2 for the halves of a split signed image (adjacent, first first).

    ``split="auto"`` splits a signed image only when its one-CTA job would
    outlast the batch's lower bound on time, max(longest job, total work / SMs)
    with every signed image split: the others keep both maps in one CTA,
    which reads the image once for both."""
    n = len(shapes)
    whole = [job_cost(C, H, W, 2 if signed[i] else 1, iterations) for i, (C, H, W) in enumerate(shapes)]
    half = [job_cost(C, H, W, 1, iterations) for (C, H, W) in shapes]
    sgn = [i for i in range(n) if signed[i]]
    if split is True or split == "always":
        halves = set(sgn)
    elif split is False or split == "never":
        halves = set()
    else:
        halves = set(sgn)
        costs = [half[i] if i in halves else whole[i] for i in range(n)]
        total = sum(whole[i] for i in range(n) if not signed[i]) + sum(2 * half[i] for i in sgn)
        bound = max(max(costs, default=0.0), total / max(1, sms))
        for i in sorted(sgn, key=lambda k: whole[k]):
            if whole[i] <= bound:
                halves.discard(i)
    units = sorted(range(n), key=lambda i: -(half[i] if i in halves else whole[i]))
    jobs: List[Tuple[int, int]] = []
    for i in units:
        jobs.extend([(i, 1), (i, 2)] if i in halves else [(i, 0)])
    return jobs


# A tiled strip's hand-off of its edges through L2, once per HANDOFF_STEPS
# steps (its halo: HANDOFF_STEPS cells at each end of the strip), and the
# CTAs per tiled image tried.  On the uneven 2D batch (GB300): with a hand-off
# every 8 steps, 11 images at 3 CTAs took 19.5 ms, at 4 CTAs 16.8, at 6 16.6
# (about 5 us per hand-off of an image's two maps); with one every 32 steps
# 11 images at 6 CTAs 16.5 ms, 16 at 4 16.5, 22-26 at 4 15.4-15.5, 28 at 4
# 16.0, and 32 at 4 (128 CTAs) or 24 at 5 22-24 ms: the persistent launch
# then lacks SMs for the rest (MAX_TILED_SM_SHARE).
HANDOFF_US = 5.0
HANDOFF_STEPS = 32
TILE_COUNTS = (4, 6, 8)
MAX_TILED = 32  # images per tiled launch (fg_batch_geodesic2d_tiled)
MAX_TILED_SM_SHARE = 0.7  # tiled CTAs per SM at most


def tiled_width(n2: int, k: int, s: int = HANDOFF_STEPS) -> int:
    """Strip width of a row of n2 cells over k CTAs (fg_batch_tiled.cu)."""
    return max(((n2 + k - 1) // k + 3) & ~3, s)


def tiled_cost(C: int, H: int, W: int, maps: int, iterations: int, k: int) -> float:
    """Estimated microseconds of an image whose rows are split over k CTAs."""
    h = HANDOFF_US / HANDOFF_STEPS
    halo = 2 * HANDOFF_STEPS
    return 2.0 * max(iterations, 1) * (H * (step_us(C, maps, tiled_width(W, k) + halo) + h) +
                                       W * (step_us(C, maps, tiled_width(H, k) + halo) + h))


def _rest_bound(shapes, signed, iterations, sms) -> float:
    """Lower bound on the time of a batch: its longest job or its work over the SMs."""
    jobs = plan_jobs(shapes, signed, iterations, sms)
    cost = [job_cost(*shapes[i], 1 if p else (2 if signed[i] else 1), iterations) for i, p in jobs]
    return max(max(cost, default=0.0), sum(cost) / max(1, sms))


def plan_tiles(shapes: Sequence[Tuple[int, int, int]], signed: Sequence[bool], iterations: int, sms: int,
               max_images: int = MAX_TILED) -> dict:
    """Images to run tiled beside the batch, ``{image: CTAs}``: the largest
    images, as many and as finely split as lowers the estimated time of the
    whole (the tiled images' longest against the rest of the batch on the
    SMs left to it); none when tiling does not pay."""
    n = len(shapes)
    whole = [job_cost(C, H, W, 2 if signed[i] else 1, iterations) for i, (C, H, W) in enumerate(shapes)]
    order = [i for i in sorted(range(n), key=lambda i: -whole[i]) if max(shapes[i][1], shapes[i][2]) >= 256]
    best, best_t = {}, _rest_bound(shapes, signed, iterations, sms)
    for count in range(1, min(max_images, len(order)) + 1):
        top = order[:count]
        rest = [i for i in range(n) if i not in set(top)]
        for k in TILE_COUNTS:
            if count * k > int(MAX_TILED_SM_SHARE * sms):
                break
            t_tiled = max(tiled_cost(*shapes[i], 2 if signed[i] else 1, iterations, k) for i in top)
            t_rest = _rest_bound([shapes[i] for i in rest], [signed[i] for i in rest], iterations, sms - count * k)
            t = max(t_tiled, t_rest)
            if t < best_t * 0.97:
                best, best_t = {i: k for i in top}, t
    return best


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
    if image.size(1) < 1:
        raise RuntimeError("batch items need at least one image channel")


class GeodesicBatch2d:
    """A batch of fixed shapes with preallocated buffers.

    Args:
        shapes: list of ``(C, H, W)``.
        signed: compute ``D(M) - D(1 - M)`` instead of ``D(M)``: one value for
            every image, or one per image (plain and signed in one launch).
        iterations: raster-scan iterations (the reference's ``iter``).
        device: CUDA device.
        use_graph: replay the launch from a captured CUDA graph.
        inputs: optional caller-owned ``(images, masks)`` lists, used in place.
        split: ``"auto"`` (see :func:`plan_jobs`), ``True`` (every signed image
            as two jobs) or ``False`` (every signed image as one job).
        tiles: ``"auto"`` (see :func:`plan_tiles`), ``None`` (no tiled images)
            or ``{image: CTAs}``: images whose rows are split over several
            CTAs of a cooperative launch beside the batch.

    Fill ``images[i]`` / ``masks[i]`` (in place), set ``v`` / ``lambs``, call
    :meth:`run`; results are in ``outputs[i]``.
    """

    def __init__(self, shapes: Sequence[Sequence[int]], signed: Union[bool, Sequence[bool]] = False,
                 iterations: int = 2, device=None, use_graph: bool = True, inputs=None,
                 split: Union[str, bool] = "auto", tiles: Union[str, dict, None] = "auto"):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.iterations = int(iterations)
        self.shapes = [tuple(int(x) for x in s) for s in shapes]
        n = len(self.shapes)
        if isinstance(signed, (list, tuple)):
            if len(signed) != n:
                raise ValueError("signed must be one value or one per image")
            self.signed = [bool(x) for x in signed]
        else:
            self.signed = [bool(signed)] * n
        for C, H, W in self.shapes:
            if C < 1 or min(H, W) < 0:
                raise RuntimeError(f"unsupported batch item shape {(C, H, W)}")
        # images the persistent kernel does not take: the per-call engine
        self.percall = [i for i, (C, H, W) in enumerate(self.shapes) if C > MAX_CHANNELS or max(H, W) > MAX_SIDE]
        pc = set(self.percall)
        batched = [i for i in range(n) if i not in pc]
        dev = self.device
        if inputs is not None:  # caller-owned tensors, used in place
            self.images, self.masks = list(inputs[0]), list(inputs[1])
        else:
            self.images = [torch.zeros((1, C, H, W), device=dev) for C, H, W in self.shapes]
            self.masks = [torch.ones((1, 1, H, W), device=dev) for _, H, W in self.shapes]
        self.outputs = [torch.empty((1, 1, H, W), device=dev) for _, H, W in self.shapes]
        self._scratch = []
        for i, ((C, H, W), sg) in enumerate(zip(self.shapes, self.signed)):
            if i in pc:
                self._scratch.append(None)
                continue
            s = {"image_t": torch.empty((C, W, H), device=dev), "t1": torch.empty((W, H), device=dev)}
            if sg:
                s["d2"] = torch.empty((H, W), device=dev)
                s["t2"] = torch.empty((W, H), device=dev)
            self._scratch.append(s)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        self.sms = sms
        if tiles == "auto":
            sub = plan_tiles([self.shapes[i] for i in batched], [self.signed[i] for i in batched], self.iterations,
                             sms)
            self.tiled = {batched[i]: k for i, k in sub.items()}
        else:
            self.tiled = {int(i): int(k) for i, k in (tiles or {}).items()}
        for i, k in self.tiled.items():
            if not (0 <= i < n) or not (2 <= k <= 16) or i in pc:
                raise ValueError("tiles: {image: 2 to 16 CTAs} (images of up to 4 channels and sides up to 2048)")
        rest = [i for i in batched if i not in self.tiled]
        sub = plan_jobs([self.shapes[i] for i in rest], [self.signed[i] for i in rest], self.iterations,
                        sms - sum(self.tiled.values()), split)
        self.jobs = [(rest[i], part) for i, part in sub]
        # tiled images grouped by channel count, one cooperative launch each
        self._tiled_groups = []
        for C in sorted({self.shapes[i][0] for i in self.tiled}):
            idx = [i for i in sorted(self.tiled) if self.shapes[i][0] == C]
            for g0 in range(0, len(idx), MAX_TILED):
                g = idx[g0:g0 + MAX_TILED]
                ext = max(max(self.shapes[i][1], self.shapes[i][2]) for i in g)
                scratch = torch.empty(max(1, _lib.load().fg_batch2d_tiled_scratch_bytes(len(g), ext)),
                                      dtype=torch.uint8, device=dev)
                self._tiled_groups.append({
                    "images": g, "C": C, "ext": ext, "scratch": scratch,
                    "tiles": (ctypes.c_int * len(g))(*[self.tiled[i] for i in g]),
                    "host": np.zeros(len(g), dtype=ITEM_DTYPE),
                    "dev": torch.empty(len(g) * ITEM_DTYPE.itemsize, dtype=torch.uint8, device=dev),
                    "stream": torch.cuda.Stream(dev)})
        nj = len(self.jobs)
        self._items_host = np.zeros(nj, dtype=ITEM_DTYPE)
        self._items_dev = torch.empty(max(1, nj * ITEM_DTYPE.itemsize), dtype=torch.uint8, device=dev)
        self._counter = torch.zeros(1 + nj, dtype=torch.int32, device=dev)  # queue + one word per split image
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.max_C = max([self.shapes[i][0] for i in batched], default=1)
        self.max_extent = max([max(self.shapes[i][1], self.shapes[i][2]) for i in batched], default=1)
        # per-call images run one after another on one side stream: one workspace
        L = _lib.load()
        need = [int(L.fg_workspace_bytes(_lib.FG_OP_SIGNED if self.signed[i] else _lib.FG_OP_PLAIN, C, 1, H, W))
                for i, (C, H, W) in enumerate(self.shapes) if i in pc]
        self._pc_ws = torch.zeros(max(need), dtype=torch.uint8, device=dev) if need else None
        self._pc_stream = torch.cuda.Stream(dev) if need else None
        self.v = 1e10
        self.lambs = [1.0] * n
        self._graph = None
        self._graph_key = None
        self.use_graph = bool(use_graph)

    def _describe(self, rec, i, flags):
        """Descriptor of image i (fg_batch2d_item) into the record rec."""
        C, H, W = self.shapes[i]
        s = self._scratch[i]
        lamb = float(self.lambs[i])
        sg = self.signed[i]
        rec["image"] = self.images[i].data_ptr()
        rec["mask"] = self.masks[i].data_ptr()
        rec["out"] = self.outputs[i].data_ptr()
        rec["image_t"] = s["image_t"].data_ptr()
        rec["t1"] = s["t1"].data_ptr()
        rec["d2"] = s["d2"].data_ptr() if sg else 0
        rec["t2"] = s["t2"].data_ptr() if sg else 0
        rec["C"], rec["H"], rec["W"] = C, H, W
        rec["flags"] = flags
        rec["v"] = np.float32(self.v)
        rec["l_grad"] = np.float32(lamb)
        rec["l_eucl"] = np.float32(1.0 - lamb)  # FastGeodis/__init__.py:63-65

    def _fill_items(self):
        for g in self._tiled_groups:
            for slot, i in enumerate(g["images"]):
                self._describe(g["host"][slot], i, FG_BATCH_SIGNED if self.signed[i] else 0)
            g["dev"].copy_(torch.from_numpy(g["host"].view(np.uint8).copy()), non_blocking=False)
        it = self._items_host
        for slot, (i, part) in enumerate(self.jobs):
            flags = (FG_BATCH_SIGNED if self.signed[i] else 0) | (FG_BATCH_SPLIT if part else 0) | \
                (FG_BATCH_SECOND if part == 2 else 0)
            self._describe(it[slot], i, flags)
        host = torch.from_numpy(it.view(np.uint8).copy())
        self._items_dev[: host.numel()].copy_(host, non_blocking=False)

    def _launch(self):
        L = _lib.load()
        main = torch.cuda.current_stream(self.device)
        for g in self._tiled_groups:  # beside the batch, on their own streams
            g["stream"].wait_stream(main)
            with torch.cuda.stream(g["stream"]):
                rc = L.fg_batch_geodesic2d_tiled(g["dev"].data_ptr(), g["tiles"], len(g["images"]), g["C"], g["ext"],
                                                 self.iterations, g["scratch"].data_ptr(), g["scratch"].numel(),
                                                 self._status.data_ptr(), g["stream"].cuda_stream)
            _lib.check(rc)
        if self.jobs:
            rc = L.fg_batch_geodesic2d(self._items_dev.data_ptr(), len(self.jobs), self.max_C, self.max_extent, 0,
                                       self.iterations, self._counter.data_ptr(), self._status.data_ptr(),
                                       max(1, self.sms - sum(self.tiled.values())), main.cuda_stream)
            _lib.check(rc)
        for g in self._tiled_groups:
            main.wait_stream(g["stream"])

    def _launch_percall(self):
        """The images the persistent kernel does not take, through the per-call
        engine on a side stream (not captured: it runs beside the graph)."""
        if not self.percall:
            return
        L = _lib.load()
        main = torch.cuda.current_stream(self.device)
        side = self._pc_stream
        side.wait_stream(main)
        ws = self._pc_ws
        for i in self.percall:
            C, H, W = self.shapes[i]
            lamb = float(self.lambs[i])
            fn = L.fg_signed_generalised_geodesic2d if self.signed[i] else L.fg_generalised_geodesic2d
            rc = fn(self.images[i].data_ptr(), C, H, W, self.masks[i].data_ptr(), 1, self.outputs[i].data_ptr(),
                    float(np.float32(self.v)), lamb, 1.0 - lamb, self.iterations, ws.data_ptr(), ws.numel(),
                    side.cuda_stream)
            _lib.check(rc)
        main.wait_stream(side)

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
            self._launch_percall()
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

    def check(self) -> None:
        """Synchronise and raise if a launch recorded an error (a wait that
        timed out, or a malformed split pair)."""
        code = int(self._status.item())
        if code:
            self._status.zero_()
            raise _lib.EngineError(f"fastgeodis_gb300 batch error {code}")
        if self._pc_ws is not None:
            _lib.check(_lib.load().fg_workspace_status(self._pc_ws.data_ptr(), self._pc_stream.cuda_stream))


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
