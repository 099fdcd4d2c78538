"""Parity at the configurations the benchmark times, against the oracle
(the C restatement of the reference's CPU path, itself pinned bit for bit to
the reference's own CPU build by tests/test_oracle_golden.py).

* The 3D workload 1x1x128x256x256 (spacing 2, 0.5, 0.5; lamb 0, 0.5, 1;
  iterations 4) under the cost model's plans, under plans the autotuner picks
  for the three transforms running together on three streams (the bench's
  step), and under the plans a bench run pinned on a GB300.
* One 256^3 volume under the cluster-sweep plan of the batch of 256^3
  volumes (16 strips of 16 rows, two runs per thread), and three volumes of
  that batch through GeodesicBatch3d on concurrent streams.
* The 64-image uneven 2D batch of the bench (seed 3): every image whose rows
  are tiled over several CTAs, every signed image split over two CTAs and a
  spread of the rest, plain and signed, each against the oracle.

The bar is bit-identity (both sides evaluate the same float32 operations in
the same order).
"""
import numpy as np
import pytest
import torch

import bench
import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib, tune
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c2():
    return bench.workload("c2")


def run_concurrent(w, d_img, d_msk):
    """The bench's step: one transform per lamb, each on its own stream."""
    main = torch.cuda.current_stream()
    streams = [torch.cuda.Stream() for _ in w["lambs"]]
    outs = []
    for s in streams:
        s.wait_stream(main)
    for lamb, s in zip(w["lambs"], streams):
        with torch.cuda.stream(s):
            outs.append(fg.generalised_geodesic3d(d_img, d_msk, w["spacing"], w["v"], lamb, w["iters"]))
    for s in streams:
        main.wait_stream(s)
    torch.cuda.synchronize()
    return [o[0].cpu().numpy() for o in outs]


def check_c2(w, outs):
    for lamb, got in zip(w["lambs"], outs):
        want = oracle.geodesic3d(w["image"][0], w["mask"][0], w["spacing"], w["v"], lamb, w["iters"])
        assert bits_equal(got, want), (lamb, float(np.abs(got - want).max()))


def test_c2_cost_model_plans(c2):
    tune.clear(c2["image"].shape[2:])
    d_img, d_msk = torch.from_numpy(c2["image"]).cuda(), torch.from_numpy(c2["mask"]).cuda()
    check_c2(c2, run_concurrent(c2, d_img, d_msk))
    fg.check_status()


def test_c2_autotuned_plans(c2):
    shape = c2["image"].shape[2:]
    try:
        res = tune.autotune(shape, channels=1, lambs=c2["lambs"], spacing=c2["spacing"], iterations=1)
        assert set(res) == set(tune.pass_keys(shape))
        d_img, d_msk = torch.from_numpy(c2["image"]).cuda(), torch.from_numpy(c2["mask"]).cuda()
        check_c2(c2, run_concurrent(c2, d_img, d_msk))
        fg.check_status()
    finally:
        tune.clear(shape)


def test_c2_plans_pinned_by_a_bench_run(c2):
    # (cross, N1, N2) -> (S, T1, T2, flags) as recorded in a bench line on a GB300
    plans = {(2, 256, 256): (4, 18, 52, _lib.FG_PLAN_LEAN), (2, 128, 256): (8, 22, 32, 0)}
    shape = c2["image"].shape[2:]
    try:
        tune.pin(plans)
        d_img, d_msk = torch.from_numpy(c2["image"]).cuda(), torch.from_numpy(c2["mask"]).cuda()
        check_c2(c2, run_concurrent(c2, d_img, d_msk))
        fg.check_status()
    finally:
        tune.clear(shape)


B256_PLAN = (8, 16, 256, _lib.FG_PLAN_CLUSTER | _lib.FG_PLAN_RUNS2)


def test_vol256_on_the_batch_cluster_plan():
    w = bench.workload("vol256", seed=1)
    shape = w["image"].shape[2:]
    try:
        tune.pin({k: B256_PLAN for k in tune.pass_keys(shape)})
        for k in tune.pass_keys(shape):
            assert _lib.plan_describe(*k, 1, 1, 0)["lean"] & _lib.FG_PLAN_RUNS2
        d_img, d_msk = torch.from_numpy(w["image"]).cuda(), torch.from_numpy(w["mask"]).cuda()
        for lamb in w["lambs"]:
            got = fg.generalised_geodesic3d(d_img, d_msk, w["spacing"], w["v"], lamb, w["iters"])[0].cpu().numpy()
            want = oracle.geodesic3d(w["image"][0], w["mask"][0], w["spacing"], w["v"], lamb, w["iters"])
            assert bits_equal(got, want), (lamb, float(np.abs(got - want).max()))
        fg.check_status()
    finally:
        tune.clear(shape)


def test_b256_volumes_through_the_batch_api():
    vols = [bench.workload("vol256", seed=1 + k) for k in range(3)]
    shape = vols[0]["image"].shape[2:]
    lambs = [0.0, 0.5, 1.0]
    try:
        tune.pin({k: B256_PLAN for k in tune.pass_keys(shape)})
        imgs = [torch.from_numpy(v["image"]).cuda() for v in vols]
        msks = [torch.from_numpy(v["mask"]).cuda() for v in vols]
        b = fg.GeodesicBatch3d([tuple(im.shape[1:]) for im in imgs], iterations=4, use_graph=True, streams=3,
                               inputs=(imgs, msks))
        b.v, b.lambs, b.spacings = 1e10, lambs, [(1.0, 1.0, 1.0)] * 3
        for _ in range(2):  # capture, then replay
            outs = b.run()
        torch.cuda.synchronize()
        b.check()
        for v, lamb, o in zip(vols, lambs, outs):
            want = oracle.geodesic3d(v["image"][0], v["mask"][0], v["spacing"], 1e10, lamb, 4)
            assert bits_equal(o[0].cpu().numpy(), want), lamb
    finally:
        tune.clear(shape)


def test_c3_batch_against_the_oracle():
    items = bench.batch_workload()
    shapes = [(im.shape[1], im.shape[2], im.shape[3]) for im, _, _ in items]
    n = len(items)
    plan = fg.GeodesicBatch2d(shapes + shapes, signed=[False] * n + [True] * n, iterations=2, use_graph=True,
                              inputs=([im for im, _, _ in items] * 2, [m for _, m, _ in items] * 2))
    plan.v, plan.lambs = 1e10, [l for _, _, l in items] * 2
    for _ in range(2):  # capture, then replay
        plan.run()
    torch.cuda.synchronize()
    plan.check()
    tiled = set(plan.tiled)
    split = {i for i, part in plan.jobs if part == 1}
    assert tiled, "the bench batch tiles its largest images"
    spread = set(range(0, 2 * n, 7))
    chosen = sorted(tiled | split | spread)
    for j in chosen:
        im, m, lamb = items[j % n]
        img, msk = im[0].cpu().numpy(), m[0].cpu().numpy()
        want = oracle.signed2d(img, msk, 1e10, lamb, 2) if j >= n else oracle.geodesic2d(img, msk, 1e10, lamb, 2)
        got = plan.outputs[j][0].cpu().numpy()
        kind = "tiled" if j in tiled else "split" if j in split else "one CTA"
        assert bits_equal(got, want), (j, shapes[j % n], kind, float(np.abs(got - want).max()))
