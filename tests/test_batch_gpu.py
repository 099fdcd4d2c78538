"""Batched 2D transforms (one persistent launch, work queue of images) against
the per-call path: each image's result must be bit-identical alone and in the
batch."""
import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg

pytestmark = pytest.mark.gpu


def make_batch(seed, n, sides, channels, odd=False):
    rng = np.random.default_rng(seed)
    imgs, masks, lambs = [], [], []
    for _ in range(n):
        H = int(rng.integers(sides[0], sides[1]))
        W = int(rng.integers(sides[0], sides[1]))
        if not odd:
            H, W = H // 4 * 4 or 4, W // 4 * 4 or 4
        C = int(rng.choice(channels))
        img = torch.from_numpy((rng.random((1, C, H, W)) * 255).astype(np.float32)).cuda()
        m = torch.ones((1, 1, H, W))
        for _ in range(int(rng.integers(1, 4))):
            y, x = int(rng.integers(0, H)), int(rng.integers(0, W))
            m[0, 0, max(0, y - 2):y + 2, max(0, x - 2):x + 2] = 0
        imgs.append(img)
        masks.append(m.cuda())
        lambs.append(float(rng.random()))
    return imgs, masks, lambs


@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("odd", [False, True])
def test_batch_matches_per_call(signed, odd):
    imgs, masks, lambs = make_batch(3 + odd + 2 * signed, 12, (1, 300), [1, 3], odd=odd)
    f = fg.signed_generalised_geodesic2d_batch if signed else fg.generalised_geodesic2d_batch
    g = fg.signed_generalised_geodesic2d if signed else fg.generalised_geodesic2d
    outs = f(imgs, masks, 1e10, lambs, 2)
    for im, m, l, o in zip(imgs, masks, lambs, outs):
        ref = g(im, m, 1e10, l, 2)
        assert o.shape == ref.shape
        assert torch.equal(o.view(torch.int32), ref.view(torch.int32)), (im.shape, l)
    fg.check_status()


def test_batch_large_sides_and_graph_replay():
    imgs, masks, lambs = make_batch(11, 6, (1000, 2049), [1], odd=False)
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im in imgs]
    plan = fg.GeodesicBatch2d(shapes, signed=False, iterations=2, use_graph=True)
    for i in range(len(imgs)):
        plan.images[i].copy_(imgs[i])
        plan.masks[i].copy_(masks[i])
    plan.v, plan.lambs = 1e10, lambs
    for _ in range(3):  # capture once, replay twice
        outs = plan.run()
    torch.cuda.synchronize()
    for im, m, l, o in zip(imgs, masks, lambs, outs):
        ref = fg.generalised_geodesic2d(im, m, 1e10, l, 2)
        assert torch.equal(o.view(torch.int32), ref.view(torch.int32))


def test_batch_rejects_bad_items():
    a = torch.rand(1, 1, 8, 8, device="cuda")
    with pytest.raises(ValueError):
        fg.generalised_geodesic2d_batch([a], [torch.rand(1, 1, 8, 9, device="cuda")], 1e10, 1.0)
    with pytest.raises(ValueError):
        fg.generalised_geodesic2d_batch([a], [torch.rand(1, 2, 8, 8, device="cuda")], 1e10, 1.0)
    with pytest.raises(RuntimeError):
        fg.generalised_geodesic2d_batch([torch.rand(1, 1, 8, 8, device="cuda", dtype=torch.float64)],
                                        [torch.rand(1, 1, 8, 8, device="cuda")], 1e10, 1.0)
    assert fg.generalised_geodesic2d_batch([], [], 1e10, 1.0) == []


@pytest.mark.parametrize("graph", [False, True])
def test_batch_takes_any_channel_count_and_side(graph):
    """Images of more than four channels and a side above 2048 go through the
    per-call engine beside the persistent launch: every output equals the
    oracle's bits, plain and signed, mixed with ordinary images."""
    from golden_cases import bits_equal
    from oracle import oracle

    rng = np.random.default_rng(40)
    shapes = [(5, 37, 61), (1, 90, 70), (8, 50, 33), (2, 8, 2100), (3, 64, 64), (6, 2050, 6)]
    signed = [False, True, True, False, False, True]
    imgs = [torch.from_numpy((rng.random((1,) + s) * 255).astype(np.float32)).cuda() for s in shapes]
    msks = []
    for _, H, W in shapes:
        m = np.ones((1, 1, H, W), np.float32)
        m[0, 0, H // 2, W // 3] = 0
        msks.append(torch.from_numpy(m).cuda())
    lambs = [0.6, 0.3, 1.0, 0.8, 0.0, 0.5]
    plan = fg.GeodesicBatch2d(shapes, signed=signed, iterations=2, use_graph=graph, inputs=(imgs, msks))
    assert sorted(plan.percall) == [0, 2, 3, 5]
    plan.v, plan.lambs = 1e10, lambs
    for _ in range(2):
        outs = plan.run()
    torch.cuda.synchronize()
    plan.check()
    for im, m, l, sg, o in zip(imgs, msks, lambs, signed, outs):
        f = oracle.signed2d if sg else oracle.geodesic2d
        want = f(im[0].cpu().numpy(), m[0].cpu().numpy(), 1e10, l, 2)
        assert bits_equal(o[0].cpu().numpy(), want), (im.shape, l, sg)


@pytest.mark.parametrize("split", [True, False, "auto"])
def test_mixed_plain_and_signed_in_one_launch(split):
    """Plain and signed images in one plan, signed images split over two CTAs
    or not: every output bit-identical to its per-call transform."""
    imgs, masks, lambs = make_batch(21, 10, (1, 400), [1, 2, 3, 4], odd=True)
    n = len(imgs)
    signed = [bool(i % 2) for i in range(n)] + [True] * n
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im in imgs] * 2
    plan = fg.GeodesicBatch2d(shapes, signed=signed, iterations=2, use_graph=True, split=split,
                              inputs=(imgs * 2, masks * 2))
    plan.v, plan.lambs = 1e10, lambs * 2
    halves = sum(1 for _, p in plan.jobs if p == 1)
    if split is True:
        assert halves == sum(signed)
    if split is False:
        assert halves == 0
    for _ in range(2):  # capture, replay
        outs = plan.run()
    plan.check()
    for i, o in enumerate(outs):
        g = fg.signed_generalised_geodesic2d if signed[i] else fg.generalised_geodesic2d
        ref = g(imgs[i % n], masks[i % n], 1e10, lambs[i % n], 2)
        assert torch.equal(o.view(torch.int32), ref.view(torch.int32)), (i, shapes[i], signed[i])


def test_split_halves_large_images():
    """Split signed images whose second half reaches its first pass along W
    long after the first half published the transposed image."""
    imgs, masks, lambs = make_batch(5, 4, (1500, 2049), [1, 3])
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im in imgs]
    plan = fg.GeodesicBatch2d(shapes, signed=True, iterations=1, use_graph=False, split=True,
                              inputs=(imgs, masks))
    plan.v, plan.lambs = 1e10, lambs
    outs = plan.run()
    plan.check()
    for im, m, l, o in zip(imgs, masks, lambs, outs):
        ref = fg.signed_generalised_geodesic2d(im, m, 1e10, l, 1)
        assert torch.equal(o.view(torch.int32), ref.view(torch.int32))


def test_split_halves_more_jobs_than_the_grid():
    """240 jobs (120 split signed images) for a grid of one CTA per SM: halves
    claimed late still find their first half published."""
    imgs, masks, lambs = make_batch(13, 120, (8, 96), [1, 3], odd=True)
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im in imgs]
    plan = fg.GeodesicBatch2d(shapes, signed=True, iterations=2, use_graph=True, split=True, inputs=(imgs, masks))
    plan.v, plan.lambs = 1e10, lambs
    assert len(plan.jobs) == 240
    for _ in range(2):
        outs = plan.run()
    plan.check()
    for im, m, l, o in zip(imgs, masks, lambs, outs):
        ref = fg.signed_generalised_geodesic2d(im, m, 1e10, l, 2)
        assert torch.equal(o.view(torch.int32), ref.view(torch.int32))


def test_split_pair_without_partner_is_reported():
    """A descriptor marked as the first half of a split image whose partner is
    missing runs nothing and records FG_ERR_INVALID_ARGUMENT."""
    from fastgeodis_gb300 import _lib
    from fastgeodis_gb300.batch import FG_BATCH_SIGNED, FG_BATCH_SPLIT

    imgs, masks, lambs = make_batch(9, 2, (16, 40), [1])
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im in imgs]
    plan = fg.GeodesicBatch2d(shapes, signed=True, iterations=1, use_graph=False, split=False,
                              inputs=(imgs, masks))
    plan.v, plan.lambs = 1e10, lambs
    plan.run()
    plan.check()
    plan._items_host[0]["flags"] = FG_BATCH_SIGNED | FG_BATCH_SPLIT  # no FG_BATCH_SECOND copy follows
    host = torch.from_numpy(plan._items_host.view(np.uint8).copy())
    plan._items_dev[: host.numel()].copy_(host)
    plan._launch()
    with pytest.raises(_lib.EngineError):
        plan.check()
    plan.check()  # cleared: the context stays usable


@pytest.mark.parametrize("signed", [False, True])
def test_tiled_images_beside_the_batch(signed):
    """Images whose rows are split over 2-8 CTAs of the cooperative launch
    beside the batch (odd sizes, 1-4 channels): bit-identical to per call."""
    imgs, masks, lambs = make_batch(31 + signed, 9, (40, 700), [1, 2, 3, 4], odd=True)
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im in imgs]
    tiles = {0: 2, 2: 3, 3: 8, 5: 4, 6: 2, 8: 6}
    plan = fg.GeodesicBatch2d(shapes, signed=signed, iterations=2, use_graph=True, tiles=tiles,
                              inputs=(imgs, masks))
    plan.v, plan.lambs = 1e10, lambs
    assert {i for i, _ in plan.jobs} == {1, 4, 7}
    for _ in range(3):  # capture, replay
        outs = plan.run()
    plan.check()
    g = fg.signed_generalised_geodesic2d if signed else fg.generalised_geodesic2d
    for i, (im, m, l, o) in enumerate(zip(imgs, masks, lambs, outs)):
        ref = g(im, m, 1e10, l, 2)
        assert torch.equal(o.view(torch.int32), ref.view(torch.int32)), (i, shapes[i], tiles.get(i))


def test_tiled_auto_plan_large_images():
    """The automatic plan tiles the largest images of a batch like the
    uneven-batch workload's; every output still matches its per-call one."""
    imgs, masks, lambs = make_batch(41, 24, (200, 2049), [1, 3])
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im in imgs]
    plan = fg.GeodesicBatch2d(shapes * 2, signed=[False] * 24 + [True] * 24, iterations=2, use_graph=True,
                              inputs=(imgs * 2, masks * 2))
    plan.v, plan.lambs = 1e10, lambs * 2
    assert plan.tiled  # the largest images run tiled
    outs = plan.run()
    plan.check()
    for i, o in enumerate(outs):
        g = fg.signed_generalised_geodesic2d if i >= 24 else fg.generalised_geodesic2d
        ref = g(imgs[i % 24], masks[i % 24], 1e10, lambs[i % 24], 2)
        assert torch.equal(o.view(torch.int32), ref.view(torch.int32)), (i, shapes[i % 24], plan.tiled.get(i))


def test_tiled_degenerate_shapes():
    """Tiled images with one row, one column, rows narrower than a halo and
    more CTAs than strips: every CTA still meets the barriers, results match."""
    shapes = [(1, 1, 700), (3, 600, 1), (1, 5, 7), (2, 3, 900), (1, 64, 40)]
    rng = np.random.default_rng(17)
    imgs, masks = [], []
    for C, H, W in shapes:
        imgs.append(torch.from_numpy((rng.random((1, C, H, W)) * 255).astype(np.float32)).cuda())
        m = torch.ones((1, 1, H, W))
        m[0, 0, H // 2, W // 2] = 0
        masks.append(m.cuda())
    lambs = [0.3, 0.9, 0.5, 1.0, 0.0]
    for signed in (False, True):
        plan = fg.GeodesicBatch2d(shapes, signed=signed, iterations=2, use_graph=False,
                                  tiles={0: 4, 1: 8, 2: 3, 3: 16, 4: 2}, inputs=(imgs, masks))
        plan.v, plan.lambs = 1e10, lambs
        outs = plan.run()
        plan.check()
        g = fg.signed_generalised_geodesic2d if signed else fg.generalised_geodesic2d
        for i, o in enumerate(outs):
            ref = g(imgs[i], masks[i], 1e10, lambs[i], 2)
            assert torch.equal(o.view(torch.int32), ref.view(torch.int32)), (shapes[i], signed)
