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


def _voxels(shape: Sequence[int]) -> int:
    return shape[1] * shape[2] * shape[3]


def _slot_key(shape: Sequence[int]):
    return (-_voxels(shape), tuple(shape))


def slot_order(shapes: Sequence[Sequence[int]]) -> List[int]:
    """Order of a batch's stream slots: largest volumes first, equal shapes
    together (a slot's workspace depends on the shape only)."""
    return sorted(range(len(shapes)), key=lambda i: _slot_key(shapes[i]))


def launch_order(shapes: Sequence[Sequence[int]], lambs: Sequence[float]) -> List[int]:
    """The order a batch launches its transforms in: the slot order, and
    among equal shapes the costlier arithmetic first (on the higher-priority
    streams).  Position k holds a volume of the same shape as in
    :func:`slot_order`, so the slots' workspaces fit whatever the weights."""
    return sorted(range(len(shapes)), key=lambda i: (_slot_key(shapes[i]), -transform_cost(shapes[i], lambs[i])))


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


def batch_general_plan_for(key, channels: int = 1):
    """The plan a batch pins for passes of the general arithmetic (0 < lamb
    < 1) on a cross-section whose batch plan runs the cluster sweep kernel:
    the same strips with one run per thread (twice the warps), or None.
    Measured on eight 256^3 volumes with mixed lambdas: 12.92 -> 12.70 ms per
    batch (the l_eucl = 0 and l_grad = 0 passes are faster on the sweep kernel)."""
    c = batch_plan_for(key, channels)
    if c is None or not c[3] & _lib.FG_PLAN_RUNS2 or channels > 1:
        return None
    S, T1, N2 = c[0], c[1], key[2]
    threads = T1 * -(-N2 // 4)
    if threads > tune.THREADS_LEAN:
        return None
    return (S, T1, N2, _lib.FG_PLAN_CLUSTER | (_lib.FG_PLAN_LEAN if threads > tune.THREADS else 0))


# Relative time of a pass per cell by arithmetic mode, measured on GB300
# (256^3 passes on the cluster plan: 0.261 / 0.395 / 0.471 ms for l_grad = 0,
# l_eucl = 0 and l_grad = 1, general).
MODE_COST = {tune.MODE_EUCLID: 1.0, tune.MODE_GEO: 1.5, tune.MODE_GENERAL: 1.8}


def transform_cost(shape: Sequence[int], lamb: float) -> float:
    """Estimated relative time of one transform of a (C, D, H, W) volume
    with weight ``lamb``: cells x the pass cost of its arithmetic mode."""
    C, D, H, W = shape
    return float(D) * H * W * MODE_COST[tune.mode_of(lamb)] * (1.0 + 0.3 * (C - 1))


def priority_streams(n: int, device=None) -> List[torch.cuda.Stream]:
    """n CUDA streams in decreasing priority (as far as the device's range
    goes): launch the costliest transforms of a batch on the first ones, so
    that when SMs free up the block scheduler serves the batch's critical
    path first (the batch ends with its slowest transform).  Measured on a
    batch of eight 256^3 volumes: 229 -> 243 Gvoxel-passes/s."""
    least, greatest = torch.cuda.Stream.priority_range()
    return [torch.cuda.Stream(device, priority=min(least, greatest + k)) for k in range(n)]


class GeodesicBatch3d:
    """A batch of fixed volume shapes with preallocated buffers.

    Args:
        shapes: list of ``(C, D, H, W)``.
        signed: compute ``D(M) - D(1 - M)`` instead of ``D(M)``.
        iterations: raster-scan iterations (the reference's ``iter``).
        device: CUDA device.
        use_graph: replay the batch from a captured CUDA graph (worth it for
            many small volumes; on eight 256^3 volumes host launches were 5%
            faster, 12.9 against 13.6 ms: the replay's kernels do not follow
            the streams' priorities).
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
            self.streams = priority_streams(max(1, min(int(streams), n)), dev)
            # largest first, so that the pool finishes with the short transforms
            self.order = slot_order(self.shapes)
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
            g = batch_general_plan_for(key, C)
            if g is not None:
                _lib.check(L.fg_plan_override(*key, *g[:3], g[3] | _lib.FG_PLAN_MODE(tune.MODE_GENERAL)))
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
            for m in (tune.MODE_GENERAL, tune.MODE_EUCLID, tune.MODE_GEO):
                _lib.check(L.fg_plan_override(*key, 0, 0, 0, _lib.FG_PLAN_MODE(m)))
        self._pinned.clear()
        self._graph = None

    # --- execution ---
    def _launch(self):
        L = _lib.load()
        fn = L.fg_signed_generalised_geodesic3d if self.signed else L.fg_generalised_geodesic3d
        main = torch.cuda.current_stream(self.device)
        for s in self.streams:
            s.wait_stream(main)
        order = launch_order(self.shapes, self.lambs)
        for slot, i in enumerate(order):
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


class _Item3d(ctypes.Structure):
    """fg_batch3d_item (include/fastgeodis_gb300.h)."""
    _fields_ = [("image", ctypes.c_void_p), ("mask", ctypes.c_void_p), ("out", ctypes.c_void_p),
                ("image_t", ctypes.c_void_p), ("t1", ctypes.c_void_p), ("d2", ctypes.c_void_p),
                ("t2", ctypes.c_void_p), ("C", ctypes.c_int), ("D", ctypes.c_int), ("H", ctypes.c_int),
                ("W", ctypes.c_int), ("flags", ctypes.c_int), ("v", ctypes.c_float), ("l_grad", ctypes.c_float),
                ("l_eucl", ctypes.c_float), ("spacing", ctypes.c_float * 3), ("reserved1", ctypes.c_float)]


FG_BATCH_SIGNED = 1
CLUSTER_SIZES = (16, 8, 4, 2, 1)


class PersistentBatch3d:
    """A batch of volumes in ONE persistent launch (fg_batch3d_plan /
    fg_batch3d_launch).

    Every volume's transform is a chain of jobs in one queue -- initial
    distances and the transposed image, its passes in order, and for the
    signed form the difference -- and the launch holds as many thread-block
    clusters as the device co-schedules; each cluster runs one job at a time
    (a pass: the cross-section's rows split into strips over the cluster's
    CTAs, rows exchanged through distributed shared memory), a job starting
    once its volume's previous one has finished.  Volumes of any sizes that
    fit a cluster; per volume the result is bit-identical to
    :func:`fastgeodis_gb300.generalised_geodesic3d` /
    :func:`fastgeodis_gb300.signed_generalised_geodesic3d`.

    Args:
        shapes: list of ``(C, D, H, W)``; C = 1 (the cluster body reads one
            image channel; C > 1 is accepted when every lamb is 0).
        signed: every volume signed, or every volume plain.
        iterations: raster-scan iterations (the reference's ``iter``).
        device: CUDA device.
        use_graph: replay the launch from a captured CUDA graph.
        inputs: optional caller-owned ``(images, masks)`` lists, used in place.
        cluster_size: CTAs per cluster (1-16); default: the largest size whose
            co-resident clusters still number at least the volumes, else the
            smallest that holds every cross-section.

    Fill ``images[i]`` / ``masks[i]`` (in place), set ``v`` / ``lambs`` /
    ``spacings``, call :meth:`run`; results are in ``outputs[i]``.
    """

    def __init__(self, shapes: Sequence[Sequence[int]], signed: bool = False, iterations: int = 4, device=None,
                 use_graph: bool = True, inputs=None, cluster_size: Optional[int] = None):
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.signed = bool(signed)
        self.iterations = int(iterations)
        self.shapes = [tuple(int(x) for x in s) for s in shapes]
        for s in self.shapes:
            if len(s) != 4 or min(s) < 1:
                raise ValueError(f"batch item shapes are (C, D, H, W) with positive extents, got {s}")
        n = len(self.shapes)
        dev = self.device
        L = _lib.load()
        with torch.cuda.device(dev):
            if inputs is not None:
                self.images, self.masks = list(inputs[0]), list(inputs[1])
            else:
                self.images = [torch.zeros((1,) + s, device=dev) for s in self.shapes]
                self.masks = [torch.ones((1, 1) + s[1:], device=dev) for s in self.shapes]
            self.outputs = [torch.empty((1, 1) + s[1:], device=dev) for s in self.shapes]
            self._scratch = []
            for C, D, H, W in self.shapes:
                sc = {"image_t": torch.empty((C, W, D, H), device=dev), "t1": torch.empty((W, D, H), device=dev)}
                if self.signed:
                    sc["d2"] = torch.empty((D, H, W), device=dev)
                    sc["t2"] = torch.empty((W, D, H), device=dev)
                self._scratch.append(sc)
            self._counters = torch.zeros(n + 1, dtype=torch.int32, device=dev)
            self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.job_bytes = int(L.fg_batch3d_job_bytes())
        self.v = 1e10
        self.lambs = [0.5] * n
        self.spacings = [(1.0, 1.0, 1.0)] * n
        self.use_graph = bool(use_graph)
        self._graph = None
        self._key = None
        self._jobs = None
        self.info = None
        self.cluster_size = int(cluster_size) if cluster_size else None

    def _items(self):
        items = (_Item3d * max(1, len(self.shapes)))()
        for i, (C, D, H, W) in enumerate(self.shapes):
            sc = self._scratch[i]
            it = items[i]
            it.image, it.mask, it.out = self.images[i].data_ptr(), self.masks[i].data_ptr(), self.outputs[i].data_ptr()
            it.image_t, it.t1 = sc["image_t"].data_ptr(), sc["t1"].data_ptr()
            it.d2 = sc["d2"].data_ptr() if self.signed else None
            it.t2 = sc["t2"].data_ptr() if self.signed else None
            it.C, it.D, it.H, it.W = C, D, H, W
            it.flags = FG_BATCH_SIGNED if self.signed else 0
            lamb = float(self.lambs[i])
            it.v, it.l_grad, it.l_eucl = float(self.v), lamb, 1.0 - lamb  # FastGeodis/__init__.py:93-96
            for k in range(3):
                it.spacing[k] = float(self.spacings[i][k])
        return items

    def _plan_with(self, items, G):
        L = _lib.load()
        n = len(self.shapes)
        cap = max(1, n * (2 + 10 * max(self.iterations, 0)))  # fg_batch3d_plan's bound
        buf = (ctypes.c_ubyte * (cap * self.job_bytes))()
        info = (ctypes.c_int * 5)()
        rc = L.fg_batch3d_plan(items, n, self.iterations, G, self._status.data_ptr(), buf, len(buf), info)
        return rc, buf, [int(x) for x in info]

    def _plan(self):
        """Job records for the current v / lambs / spacings, copied to the device."""
        L = _lib.load()
        items = self._items()
        sizes = [self.cluster_size] if self.cluster_size else list(CLUSTER_SIZES)
        fits = []
        for G in sizes:
            rc, buf, info = self._plan_with(items, G)
            if rc == _lib.FG_OK:
                fits.append((G, buf, info))
            elif self.cluster_size:
                _lib.check(rc)
        if not fits:
            raise _lib.EngineError("no cluster size holds every cross-section of this batch: " + _lib.last_error())
        choice = fits[-1]  # the smallest size that holds every cross-section
        n = len(self.shapes)
        with torch.cuda.device(self.device):
            for G, buf, info in fits:  # largest first: enough co-resident clusters for every volume
                c = ctypes.c_int()
                _lib.check(L.fg_batch3d_capacity(info[3], info[4], G, info[1], info[2], ctypes.byref(c)))
                if c.value >= n:
                    choice = (G, buf, info)
                    break
            G, buf, info = choice
            host = torch.frombuffer(bytearray(bytes(buf)[: info[0] * self.job_bytes]), dtype=torch.uint8)
            self._jobs = host.to(self.device) if info[0] else torch.zeros(1, dtype=torch.uint8, device=self.device)
        self.cluster_size_used = G
        self.info = {"jobs": info[0], "threads": info[1], "smem": info[2], "maps": info[3], "mode": info[4],
                     "cluster_size": G}

    def _launch(self):
        L = _lib.load()
        i = self.info
        rc = L.fg_batch3d_launch(self._jobs.data_ptr(), i["jobs"], len(self.shapes), i["maps"], i["mode"],
                                 i["cluster_size"], i["threads"], i["smem"], self._counters.data_ptr(),
                                 self._status.data_ptr(), int(torch.cuda.current_stream(self.device).cuda_stream))
        _lib.check(rc)

    def run(self):
        """Compute all outputs (asynchronously on the current stream)."""
        if not self.shapes:
            return self.outputs
        with torch.cuda.device(self.device):
            key = (float(self.v), tuple(float(x) for x in self.lambs),
                   tuple(tuple(float(y) for y in s) for s in self.spacings))
            if key != self._key:
                self._plan()  # the job records hold v, the weights and the step lengths
                self._graph = None
                self._key = key
            if not self.use_graph:
                self._launch()
                return self.outputs
            if self._graph is None:
                self._launch()  # outside capture first: kernel attributes, cluster capacity
                torch.cuda.synchronize(self.device)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._launch()
                self._graph = g
            self._graph.replay()
            return self.outputs

    def check(self) -> None:
        """Synchronise and raise if a wait of the launch ran out (its results are void)."""
        code = int(self._status.item())
        if code:
            self._status.zero_()
            raise _lib.EngineError(f"fastgeodis_gb300 batch3d error {code}")


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
