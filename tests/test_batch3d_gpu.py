"""Batched 3D transforms (GeodesicBatch3d): volumes of uneven sizes run
concurrently on plans for many transforms at once, replayed from one CUDA
graph; every output is bit-identical to the single call and to the oracle."""
import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib, tune
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu

SHAPES = [(1, 20, 33, 27), (1, 16, 64, 64), (2, 12, 30, 44), (1, 24, 40, 72), (1, 8, 100, 36), (1, 10, 256, 64)]
LAMBS = [0.0, 0.3, 0.6, 1.0, 0.8, 0.5]
SPACINGS = [(1.5, 0.8, 1.1), (1.0, 1.0, 1.0), (2.0, 0.5, 0.5), (0.7, 1.3, 2.2), (1.0, 0.6, 0.9), (3.0, 1.0, 1.0)]


def volume(shape, seed, soft=False):
    rng = np.random.default_rng(seed)
    C, D, H, W = shape
    img = rng.random((1, C, D, H, W)).astype(np.float32)
    if soft:
        m = rng.random((1, 1, D, H, W)).astype(np.float32)
    else:
        m = np.ones((1, 1, D, H, W), np.float32)
        for _ in range(3):
            m[0, 0, rng.integers(0, D), rng.integers(0, H), rng.integers(0, W)] = 0
    return img, m


@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_single_calls_and_oracle(signed, use_graph):
    vols = [volume(s, 30 + i, soft=signed) for i, s in enumerate(SHAPES)]
    b = fg.GeodesicBatch3d(SHAPES, signed=signed, iterations=2, use_graph=use_graph, streams=4)
    try:
        for i, (img, m) in enumerate(vols):
            b.images[i].copy_(torch.from_numpy(img))
            b.masks[i].copy_(torch.from_numpy(m))
        b.v, b.lambs, b.spacings = 1e10, LAMBS, SPACINGS
        for rep in range(2):
            outs = [o.clone() for o in b.run()]
            b.check()
            single = fg.signed_generalised_geodesic3d if signed else fg.generalised_geodesic3d
            for i, (img, m) in enumerate(vols):
                want = single(torch.from_numpy(img).cuda(), torch.from_numpy(m).cuda(), list(SPACINGS[i]), 1e10,
                              LAMBS[i], 2)
                assert torch.equal(outs[i].view(torch.int32), want.view(torch.int32)), (rep, i)
            # a new image in place: the captured graph reads the same buffers
            img0 = np.ascontiguousarray(vols[0][0][:, :, ::-1])
            vols[0] = (img0, vols[0][1])
            b.images[0].copy_(torch.from_numpy(img0))
        for i in (0, 2):  # the oracle on two of them
            img, m = vols[i]
            f = oracle.signed3d if signed else oracle.geodesic3d
            got = fg.signed_generalised_geodesic3d if signed else fg.generalised_geodesic3d
            out = got(torch.from_numpy(img).cuda(), torch.from_numpy(m).cuda(), list(SPACINGS[i]), 1e10,
                      LAMBS[i], 2)[0].cpu().numpy()
            assert bits_equal(out, f(img[0], m[0], list(SPACINGS[i]), 1e10, LAMBS[i], 2))
        fg.check_status()
    finally:
        b.release_plans()


def test_batch_pins_plans_for_concurrency_and_releases_them():
    b = fg.GeodesicBatch3d([(1, 12, 256, 256), (1, 8, 48, 40)], iterations=1, use_graph=False, streams=2)
    try:
        # l_grad = 0 and l_eucl = 0 passes: the cluster sweep kernel (two runs per thread)
        for mode in (1, 2):
            d = _lib.plan_describe(2, 256, 256, mode=mode)
            assert d["lean"] & _lib.FG_PLAN_CLUSTER and d["lean"] & _lib.FG_PLAN_RUNS2
        # general passes: the same strips, one run per thread
        d = _lib.plan_describe(2, 256, 256, mode=0)
        assert d["lean"] & _lib.FG_PLAN_CLUSTER and not d["lean"] & _lib.FG_PLAN_RUNS2 and d["tiles1"] == 16
        assert _lib.plan_describe(2, 48, 40)["tiles1"] * _lib.plan_describe(2, 48, 40)["tiles2"] == 1
    finally:
        b.release_plans()
    for mode in (0, 1, 2):
        assert not _lib.plan_describe(2, 256, 256, mode=mode)["lean"] & _lib.FG_PLAN_CLUSTER


def test_functional_batch_api():
    vols = [volume(s, 50 + i) for i, s in enumerate(SHAPES[:3])]
    imgs = [torch.from_numpy(v[0]).cuda() for v in vols]
    msks = [torch.from_numpy(v[1]).cuda() for v in vols]
    outs = fg.generalised_geodesic3d_batch(imgs, msks, [list(s) for s in SPACINGS[:3]], 1e10, LAMBS[:3], 2)
    souts = fg.signed_generalised_geodesic3d_batch(imgs, msks, (1.0, 1.0, 1.0), 1e10, 0.5, 2)
    for i in range(3):
        want = fg.generalised_geodesic3d(imgs[i], msks[i], list(SPACINGS[i]), 1e10, LAMBS[i], 2)
        assert torch.equal(outs[i], want)
        want = fg.signed_generalised_geodesic3d(imgs[i], msks[i], [1.0, 1.0, 1.0], 1e10, 0.5, 2)
        assert torch.equal(souts[i], want)


def test_batch_with_tuned_plans():
    shapes = [(1, 12, 40, 48)] * 3 + [(1, 8, 24, 32)]
    vols = [volume(s, 70 + i) for i, s in enumerate(shapes)]
    b = fg.GeodesicBatch3d(shapes, iterations=1, use_graph=True, streams=4, plans="tune")
    try:
        for i, (img, m) in enumerate(vols):
            b.images[i].copy_(torch.from_numpy(img))
            b.masks[i].copy_(torch.from_numpy(m))
        b.lambs = [0.0, 0.5, 1.0, 0.7]
        outs = [o.clone() for o in b.run()]
        b.check()
        for i, (img, m) in enumerate(vols):
            assert bits_equal(outs[i][0].cpu().numpy(), oracle.geodesic3d(img[0], m[0], [1.0, 1.0, 1.0], 1e10,
                                                                         b.lambs[i], 1)), i
    finally:
        b.release_plans()
