"""Serving: admission logic on the CPU with a fake executor, and on the GPU a
mixed stream whose every result must equal the standalone call bit for bit."""
import threading
import time

import numpy as np
import pytest
import torch

from fastgeodis_gb300.serving import Request, Scheduler


class FakeExecutor:
    """Requests take `duration` seconds; image_id is the request's byte size."""

    def __init__(self, duration=0.02):
        self.duration = duration
        self.lock = threading.Lock()
        self.running = 0
        self.max_running = 0
        self.order = []

    def bytes_needed(self, req):
        return int(req.image_id)

    def start(self, req, slot):
        with self.lock:
            self.running += 1
            self.max_running = max(self.max_running, self.running)
            self.order.append(req.id)
        return time.perf_counter() + self.duration

    def done(self, h):
        return time.perf_counter() >= h

    def finish(self, h):
        with self.lock:
            self.running -= 1
        return "ok"


def test_scheduler_budget_slots_and_fifo():
    ex = FakeExecutor(0.02)
    sch = Scheduler(ex, budget_bytes=100, max_inflight=3)
    try:
        reqs = [sch.submit(Request(image_id=s, clicks=[])) for s in [40, 40, 40, 10, 90, 10, 10, 60]]
        sch.drain(timeout=30)
    finally:
        sch.close()
    assert all(r.result == "ok" and r.error is None for r in reqs)
    assert sch.peak_in_use <= 100
    assert sch.peak_inflight <= 3 and ex.max_running <= 3
    assert ex.order == sorted(ex.order)  # admission never lets a later request overtake the queue head
    assert ex.max_running >= 2          # requests did overlap
    p = sch.latency_percentiles()
    assert p["p50"] > 0 and p["p99"] >= p["p50"]


def test_scheduler_rejects_oversized_and_reports_errors():
    class Failing(FakeExecutor):
        def start(self, req, slot):
            if req.image_id == 7:
                raise RuntimeError("launch failed")
            return super().start(req, slot)

    sch = Scheduler(Failing(0.005), budget_bytes=50, max_inflight=2)
    try:
        with pytest.raises(ValueError):
            sch.submit(Request(image_id=51, clicks=[]))
        ok = sch.submit(Request(image_id=5, clicks=[]))
        bad = sch.submit(Request(image_id=7, clicks=[]))
        sch.drain(timeout=30)
    finally:
        sch.close()
    assert ok.error is None and isinstance(bad.error, RuntimeError)
    assert sch.in_use == 0


@pytest.mark.gpu
def test_gpu_mix_equals_standalone_calls():
    import fastgeodis_gb300 as fg
    from fastgeodis_gb300.serving import GeodesicServer

    g = torch.Generator().manual_seed(2)
    srv = GeodesicServer(budget_bytes=1 << 30, max_inflight=6, streams=3)
    imgs = {
        "a": torch.rand((1, 1, 300, 257), generator=g) * 255,
        "b": torch.rand((1, 3, 128, 520), generator=g) * 255,
        "v": torch.rand((1, 1, 40, 64, 48), generator=g),
        "w": torch.rand((1, 1, 33, 20, 70), generator=g),
    }
    for k, t in imgs.items():
        srv.register_image(k, t)
    rng = np.random.default_rng(5)
    reqs = []
    try:
        for i in range(24):
            key = ["a", "b", "v", "w"][i % 4]
            shape = imgs[key].shape[2:]
            clicks = [[int(rng.integers(0, n)) for n in shape] for _ in range(int(rng.integers(1, 5)))]
            op = "gsf" if i % 7 == 3 else "plain"
            sp = [float(x) for x in rng.uniform(0.5, 3.0, 3)] if len(shape) == 3 else None
            reqs.append(srv.submit(Request(image_id=key, clicks=clicks, op=op, v=1e10, lamb=float(rng.random()),
                                           iterations=2, spacing=sp, theta=0.5, radius=2)))
        srv.drain(timeout=120)
        assert srv.scheduler.peak_inflight >= 2
        for r in reqs:
            assert r.error is None, r.error
            img = srv.executor.images[r.image_id]
            m = srv.executor._mask(img, r)
            if img.dim() == 4:
                ref = (fg.GSF2d(img, m, r.theta, r.v, r.lamb, r.iterations) if r.op == "gsf"
                       else fg.generalised_geodesic2d(img, m, r.v, r.lamb, r.iterations))
            else:
                ref = (fg.GSF3d(img, m, r.theta, r.spacing, r.v, r.lamb, r.iterations) if r.op == "gsf"
                       else fg.generalised_geodesic3d(img, m, r.spacing, r.v, r.lamb, r.iterations))
            assert torch.equal(r.result.view(torch.int32), ref.view(torch.int32)), (r.id, r.image_id, r.op)
        fg.check_status()
    finally:
        srv.close()


def _torch_click_mask(shape, clicks, radius):
    """Plain PyTorch reference of the click mask (on the CPU)."""
    grids = torch.meshgrid(*[torch.arange(n) for n in shape], indexing="ij")
    m = torch.ones(shape)
    for c in clicks:
        d2 = sum((g - int(ci)) ** 2 for g, ci in zip(grids, c))
        m[d2 <= radius * radius] = 0.0
    return m[None, None]


def test_click_mask_argument_errors():
    import ctypes

    from fastgeodis_gb300 import _lib
    from fastgeodis_gb300.serving import click_mask

    L = _lib.load()
    arr = (ctypes.c_int * 3)(0, 0, 0)
    assert L.fg_click_mask(None, 1, 4, 4, arr, 1, 1, None) == _lib.FG_ERR_INVALID_ARGUMENT
    big = (ctypes.c_int * 195)()
    buf = (ctypes.c_float * 16)()
    assert L.fg_click_mask(ctypes.cast(buf, ctypes.c_void_p), 1, 4, 4, big, 65, 1, None) == _lib.FG_ERR_UNSUPPORTED
    assert L.fg_click_mask(ctypes.cast(buf, ctypes.c_void_p), 1, 4, 4, arr, 1, -1, None) == _lib.FG_ERR_INVALID_ARGUMENT
    with pytest.raises(ValueError):
        click_mask((4, 4), [(1, 2, 3)], 1, device="cpu")


@pytest.mark.gpu
@pytest.mark.parametrize("shape,clicks,radius", [
    ((300, 257), [(0, 0), (150, 100), (299, 256)], 3),
    ((64, 65), [(10, 70), (-3, 5)], 4),           # clicks outside the image still mark what they reach
    ((40, 64, 48), [(0, 0, 0), (20, 31, 47), (39, 63, 10)], 2),
    ((17, 9, 33), [(8, 4, 16)], 0),               # radius 0: the click voxel only
    ((5, 6, 7), [], 3),                           # no clicks: all ones
])
def test_click_mask_matches_torch(shape, clicks, radius):
    from fastgeodis_gb300.serving import click_mask

    got = click_mask(shape, clicks, radius).cpu()
    assert torch.equal(got, _torch_click_mask(shape, clicks, radius))
