"""Serving interactive geodesic-distance requests with continuous batching.

A request is "distance map of image X given these click seeds": 2D or 3D,
plain or GSF, with its own weights.  The server

* keeps images resident on the device (registered once, reused by every
  click on them) and rasterises each request's clicks into its soft mask on
  the device (0 inside a ball of `radius` around each click, 1 elsewhere);
* admits queued requests as soon as an in-flight slot and enough of the HBM
  budget are free (first come, first served; a request that does not fit
  waits, later ones do not overtake it);
* runs admitted requests concurrently on a pool of CUDA streams, so work of
  requests that arrive while others are running overlaps on the GPU;
* releases a request's memory when its completion event fires and records its
  latency from submission to result.

Every request is computed exactly as a standalone call would compute it (same
kernels, same arithmetic): results are identical alone and in the mix.

The scheduling (`Scheduler`) is independent of the GPU: it drives any
executor with ``start(request, slot) -> handle``, ``done(handle) -> bool`` and
``finish(handle)``; `GpuExecutor` is the real one.
"""
from __future__ import annotations

import collections
import threading
import time
from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Sequence

import numpy as np


@dataclass
class Request:
    image_id: Any
    clicks: Sequence[Sequence[int]]          # (y, x) or (z, y, x) voxel coordinates
    op: str = "plain"                          # "plain" or "gsf"
    v: float = 1e10
    lamb: float = 1.0
    iterations: int = 2
    spacing: Optional[Sequence[float]] = None  # 3D only
    theta: float = 0.5                         # GSF only
    radius: int = 2
    # filled in by the server
    id: int = -1
    t_submit: float = 0.0
    t_start: float = 0.0
    t_done: float = 0.0
    nbytes: int = 0
    result: Any = None
    error: Optional[BaseException] = None
    event: threading.Event = field(default_factory=threading.Event)

    @property
    def latency_ms(self) -> float:
        return (self.t_done - self.t_submit) * 1e3


def click_mask(shape, clicks, radius: int, device=None):
    """Soft mask [1, 1, *shape] (2D (H, W) or 3D (D, H, W)) that is 0 within
    Euclidean distance `radius` of any click and 1 elsewhere, written on the
    device by one kernel (fg_click_mask) on the current stream."""
    import ctypes

    import torch

    from . import _lib

    shape = tuple(int(s) for s in shape)
    if len(shape) not in (2, 3):
        raise ValueError("shape must be (H, W) or (D, H, W)")
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    D, H, W = shape if len(shape) == 3 else (1,) + shape
    flat = []
    for c in clicks:
        c = [int(v) for v in c]
        if len(c) != len(shape):
            raise ValueError(f"click {c} does not match a {len(shape)}D shape")
        flat += c if len(c) == 3 else [0] + c
    arr = (ctypes.c_int * max(1, len(flat)))(*flat)
    with torch.cuda.device(dev):
        m = torch.empty((1, 1) + shape, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _lib.check(_lib.load().fg_click_mask(m.data_ptr(), D, H, W, arr, len(flat) // 3, int(radius), stream))
    return m


class Scheduler:
    """Continuous-batching admission: FIFO queue, in-flight slots, memory budget."""

    def __init__(self, executor, budget_bytes: int, max_inflight: int = 8, poll_s: float = 2e-4):
        self.ex = executor
        self.budget = int(budget_bytes)
        self.max_inflight = int(max_inflight)
        self.poll_s = poll_s
        self.queue: collections.deque = collections.deque()
        self.inflight: Dict[int, tuple] = {}
        self.in_use = 0
        self.peak_in_use = 0
        self.peak_inflight = 0
        self.completed: List[Request] = []
        self._lock = threading.Lock()
        self._wake = threading.Event()
        self._stop = False
        self._next_id = 0
        self._free_slots = list(range(self.max_inflight))
        self._thread = threading.Thread(target=self._loop, daemon=True)
        self._thread.start()

    def submit(self, req: Request) -> Request:
        req.nbytes = int(self.ex.bytes_needed(req))
        if req.nbytes > self.budget:
            raise ValueError(f"request needs {req.nbytes} bytes, more than the whole budget {self.budget}")
        with self._lock:
            req.id = self._next_id
            self._next_id += 1
            req.t_submit = time.perf_counter()
            self.queue.append(req)
        self._wake.set()
        return req

    def _admit(self):
        while True:
            with self._lock:
                if not self.queue or not self._free_slots:
                    return
                req = self.queue[0]
                if self.in_use + req.nbytes > self.budget:
                    return  # the head waits for memory; FIFO order is kept
                self.queue.popleft()
                slot = self._free_slots.pop()
                self.in_use += req.nbytes
                self.peak_in_use = max(self.peak_in_use, self.in_use)
            req.t_start = time.perf_counter()
            try:
                handle = self.ex.start(req, slot)
            except BaseException as exc:  # delivered to the caller, not raised in the loop
                req.error = exc
                self._complete(req, slot)
                continue
            with self._lock:
                self.inflight[req.id] = (req, slot, handle)
                self.peak_inflight = max(self.peak_inflight, len(self.inflight))

    def _complete(self, req, slot):
        req.t_done = time.perf_counter()
        with self._lock:
            self.in_use -= req.nbytes
            self._free_slots.append(slot)
            self.completed.append(req)
        req.event.set()

    def _reap(self) -> bool:
        with self._lock:
            items = list(self.inflight.values())
        progressed = False
        for req, slot, handle in items:
            if self.ex.done(handle):
                try:
                    req.result = self.ex.finish(handle)
                except BaseException as exc:
                    req.error = exc
                with self._lock:
                    self.inflight.pop(req.id, None)
                self._complete(req, slot)
                progressed = True
        return progressed

    def _loop(self):
        while not self._stop:
            progressed = self._reap()
            self._admit()
            with self._lock:
                idle = not self.queue and not self.inflight
            if idle:
                self._wake.wait(0.01)
                self._wake.clear()
            elif not progressed:
                time.sleep(self.poll_s)

    def drain(self, timeout: float = 300.0) -> None:
        t0 = time.perf_counter()
        while True:
            with self._lock:
                if not self.queue and not self.inflight:
                    return
            if time.perf_counter() - t0 > timeout:
                raise TimeoutError("requests did not complete in time")
            time.sleep(1e-3)

    def close(self):
        self._stop = True
        self._wake.set()
        self._thread.join(timeout=5)

    def latency_percentiles(self, qs=(50, 99)) -> Dict[str, float]:
        lat = [r.latency_ms for r in self.completed if r.error is None]
        if not lat:
            return {f"p{q}": float("nan") for q in qs}
        return {f"p{q}": float(np.percentile(lat, q)) for q in qs}


class GpuExecutor:
    """Runs requests on a pool of CUDA streams with the engine's per-call API."""

    def __init__(self, device=None, streams: int = 4, copy_back: bool = False):
        import torch

        self.torch = torch
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.streams = [torch.cuda.Stream(self.device) for _ in range(max(1, streams))]
        self.images: Dict[Any, Any] = {}
        self.copy_back = copy_back

    def register_image(self, image_id, image) -> None:
        """Make an image ([1, C, H, W] or [1, C, D, H, W]) resident on the device."""
        self.images[image_id] = image.to(self.device).contiguous()

    def bytes_needed(self, req: Request) -> int:
        from . import _lib

        img = self.images[req.image_id]
        C = int(img.shape[1])
        dims = [int(s) for s in img.shape[2:]]
        D, H, W = dims if len(dims) == 3 else [1] + dims
        P = D * H * W
        op = _lib.FG_OP_GSF if req.op == "gsf" else _lib.FG_OP_PLAIN
        ws = int(_lib.load().fg_workspace_bytes(op, C, D, H, W))
        return 2 * P * 4 + ws  # soft mask + output + workspace

    def _mask(self, img, req):
        return click_mask(tuple(img.shape[2:]), req.clicks, req.radius, self.device)

    def start(self, req: Request, slot: int):
        import fastgeodis_gb300 as fg

        torch = self.torch
        s = self.streams[slot % len(self.streams)]
        img = self.images[req.image_id]
        with torch.cuda.device(self.device), torch.cuda.stream(s):
            m = self._mask(img, req)
            if img.dim() == 4:
                out = (fg.GSF2d(img, m, req.theta, req.v, req.lamb, req.iterations) if req.op == "gsf"
                       else fg.generalised_geodesic2d(img, m, req.v, req.lamb, req.iterations))
            else:
                sp = list(req.spacing or [1.0, 1.0, 1.0])
                out = (fg.GSF3d(img, m, req.theta, sp, req.v, req.lamb, req.iterations) if req.op == "gsf"
                       else fg.generalised_geodesic3d(img, m, sp, req.v, req.lamb, req.iterations))
            if self.copy_back:
                host = torch.empty(out.shape, pin_memory=True)
                host.copy_(out, non_blocking=True)
                out = host
            ev = torch.cuda.Event()
            ev.record(s)
        return (ev, out, m)

    def done(self, handle) -> bool:
        return handle[0].query()

    def finish(self, handle):
        return handle[1]


class GeodesicServer:
    """A Scheduler over a GpuExecutor."""

    def __init__(self, device=None, budget_bytes: int = 8 << 30, max_inflight: int = 8, streams: int = 4,
                 copy_back: bool = False):
        self.executor = GpuExecutor(device, streams, copy_back)
        self.scheduler = Scheduler(self.executor, budget_bytes, max_inflight)

    def register_image(self, image_id, image) -> None:
        self.executor.register_image(image_id, image)

    def submit(self, req: Request) -> Request:
        return self.scheduler.submit(req)

    def drain(self, timeout: float = 300.0) -> None:
        self.scheduler.drain(timeout)

    def close(self) -> None:
        self.scheduler.close()
