"""Chunked tile plans: a pass run as one ordinary launch per chunk of S steps
over any number of tiles, each launch's CTAs starting from the previous row
that the launch before published.  The planner takes such a plan for volume
slices whose tiles cannot all be resident at once (about 600 thousand cells
and more on 152 SMs); here it is also forced onto small volumes and images
with fg_plan_override(FG_PLAN_CHUNKED), through every kernel variant a
chunk can run on (one or two maps, 1, 3 or 6 channels, the three arithmetic
modes, transposed writes).  The bar is the oracle's bits."""
import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib, tune
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu

CH = _lib.FG_PLAN_CHUNKED


def _case(shape, C, seed, soft=False):
    rng = np.random.default_rng(seed)
    img = (rng.random((C,) + tuple(shape)) * 50).astype(np.float32)
    m = rng.random((1,) + tuple(shape)).astype(np.float32) if soft else np.ones((1,) + tuple(shape), np.float32)
    for _ in range(4):
        m[(0,) + tuple(int(rng.integers(0, n)) for n in shape)] = 0
    return img, m


def _pin_chunked(shape, S, T1, T2, lean=0):
    tune.pin({k: (S, T1 if k[0] == 2 else 1, T2, CH | lean) for k in tune.pass_keys(shape)})
    for k in tune.pass_keys(shape):
        p = _lib.plan_describe(*k)
        assert p["lean"] & CH and p["tiles1"] * p["tiles2"] > 1, (k, p)


SP = [1.3, 0.9, 1.1]


@pytest.mark.parametrize("op,C,lamb,S,T1,T2,lean", [
    ("plain", 1, 0.6, 4, 8, 12, 0),
    ("plain", 1, 0.6, 8, 8, 16, 1),   # the 64-register kernel
    ("plain", 1, 0.0, 2, 4, 8, 0),    # l_grad == 0: no image term
    ("plain", 3, 0.5, 4, 6, 8, 0),
    ("plain", 6, 0.7, 4, 8, 8, 0),    # more than 4 channels: image read through L1
    ("signed", 1, 1.0, 4, 8, 12, 0),  # two maps; l_eucl == 0, l_grad == 1
    ("signed", 2, 0.4, 8, 9, 20, 0),
    ("gsf", 1, 0.5, 4, 8, 12, 0),
])
def test_forced_chunked_volume(op, C, lamb, S, T1, T2, lean):
    shape = (22, 37, 45)
    img, m = _case(shape, C, 3 + C, soft=op == "gsf")
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    try:
        _pin_chunked(shape, S, T1, T2, lean)
        if op == "plain":
            got = fg.generalised_geodesic3d(ti, tm, SP, 1e10, lamb, 2)
            want = oracle.geodesic3d(img, m, SP, 1e10, lamb, 2)
        elif op == "signed":
            got = fg.signed_generalised_geodesic3d(ti, tm, SP, 1e10, lamb, 2)
            want = oracle.signed3d(img, m, SP, 1e10, lamb, 2)
        else:
            got = fg.GSF3d(ti, tm, 0.3, SP, 1e10, lamb, 1)
            want = oracle.gsf3d(img, m, 0.3, SP, 1e10, lamb, 1)
        got = got[0].cpu().numpy()
        assert bits_equal(got, want), float(np.nanmax(np.abs(got - want)))
        fg.check_status()
    finally:
        tune.clear(shape)


@pytest.mark.parametrize("op,C,lamb,S,T2", [("plain", 1, 0.6, 4, 32), ("signed", 3, 0.5, 8, 24), ("plain", 5, 0.8, 2, 16)])
def test_forced_chunked_image(op, C, lamb, S, T2):
    shape = (70, 301)
    img, m = _case(shape, C, 7 + C)
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    try:
        _pin_chunked(shape, S, 1, T2)
        if op == "plain":
            got = fg.generalised_geodesic2d(ti, tm, 1e10, lamb, 2)
            want = oracle.geodesic2d(img, m, 1e10, lamb, 2)
        else:
            got = fg.signed_generalised_geodesic2d(ti, tm, 1e10, lamb, 2)
            want = oracle.signed2d(img, m, 1e10, lamb, 2)
        assert bits_equal(got[0].cpu().numpy(), want)
        fg.check_status()
    finally:
        tune.clear(shape)


def test_planner_chunks_a_volume_with_large_slices():
    """12 slices of 800 x 900: the sweep along the slices has a cross-section
    of 720,000 cells, more than the SMs' co-resident regions hold, so the
    planner runs it chunked; the other passes keep cooperative plans."""
    shape = (12, 800, 900)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    p = _lib.plan_describe(2, 800, 900, sms=sms)
    assert p["lean"] & CH and p["tiles1"] * p["tiles2"] > sms
    assert not _lib.plan_describe(2, 12, 900, sms=sms)["lean"] & CH
    img, m = _case(shape, 1, 21)
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    for lamb in (0.5, 1.0):
        got = fg.generalised_geodesic3d(ti, tm, SP, 1e10, lamb, 1)[0].cpu().numpy()
        assert bits_equal(got, oracle.geodesic3d(img, m, SP, 1e10, lamb, 1)), lamb
    got = fg.signed_generalised_geodesic3d(ti, tm, SP, 1e10, 0.5, 1)[0].cpu().numpy()
    assert bits_equal(got, oracle.signed3d(img, m, SP, 1e10, 0.5, 1))
    fg.check_status()


@pytest.mark.parametrize("seed", range(6))
def test_random_shapes_chunked_and_cluster_plans(seed):
    """Seeded random volumes, each pass cross-section pinned to a random
    chunked tile plan or cluster plan (whose layout-changing passes run in
    place and are followed by a transpose), random weights, plain or signed:
    the oracle's bits."""
    rng = np.random.default_rng(100 + seed)
    shape = tuple(int(x) for x in rng.integers(5, 41, 3))
    C = int(rng.choice([1, 1, 2, 5]))
    lamb = float(rng.choice([0.0, 0.35, 1.0]))
    signed = bool(rng.integers(0, 2))
    img, m = _case(shape, C, 200 + seed, soft=True)
    plans = {}
    for key in tune.pass_keys(shape):
        _, N1, N2 = key
        if rng.integers(0, 2) and N1 >= 2 and C == 1:
            G = int(rng.integers(2, min(N1, 16) + 1))
            plans[key] = (8, -(-N1 // G), N2, _lib.FG_PLAN_CLUSTER | (_lib.FG_PLAN_RUNS2 if rng.integers(0, 2) else 0))
        else:
            S = int(rng.choice([2, 4, 8]))
            T1 = max(S, int(rng.integers(S, max(S + 1, N1))))
            T2 = max(4, (int(rng.integers(S, max(S + 1, N2))) + 3) // 4 * 4)
            plans[key] = (S, T1, T2, CH)
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    try:
        tune.pin(plans)
        if signed:
            got = fg.signed_generalised_geodesic3d(ti, tm, SP, 1e10, lamb, 2)
            want = oracle.signed3d(img, m, SP, 1e10, lamb, 2)
        else:
            got = fg.generalised_geodesic3d(ti, tm, SP, 1e10, lamb, 2)
            want = oracle.geodesic3d(img, m, SP, 1e10, lamb, 2)
        got = got[0].cpu().numpy()
        assert bits_equal(got, want), (shape, C, lamb, signed, plans)
        fg.check_status()
    finally:
        tune.clear(shape)


def test_pass_of_more_than_65536_chunks():
    """A 70000 x 64 image on two tiles with a hand-off every step: the passes
    along H have 70000 chunks, more epochs than one counter value spans; each
    pass reserves its own range, so no pass reads another's exchange words."""
    shape = (70000, 64)
    img, m = _case(shape, 1, 31)
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    L = _lib.load()
    try:
        _lib.check(L.fg_plan_override(1, 1, 64, 1, 1, 32, 0))
        p = _lib.plan_describe(1, 1, 64)
        assert (p["S"], p["tiles2"]) == (1, 2)
        got = fg.generalised_geodesic2d(ti, tm, 1e10, 0.7, 2)[0].cpu().numpy()
        assert bits_equal(got, oracle.geodesic2d(img, m, 1e10, 0.7, 2))
        fg.check_status()
    finally:
        tune.clear(shape)
