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
        fg.generalised_geodesic2d_batch([torch.rand(1, 1, 8, 4096, device="cuda")],
                                        [torch.rand(1, 1, 8, 4096, device="cuda")], 1e10, 1.0)
    assert fg.generalised_geodesic2d_batch([], [], 1e10, 1.0) == []
