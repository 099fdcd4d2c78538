"""Cluster plans on the GPU: every volume pass of a transform pinned to a
cluster plan (one thread-block cluster owns the cross-section; boundary rows
travel through distributed shared memory) gives the oracle's bits, for the
three arithmetic modes, one and several image channels, the 64-register and
128-register kernels, transposed writes, signed and GSF transforms, and
cluster sizes from 2 to 16."""
import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib, tune
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu


def case(shape, C, seed):
    rng = np.random.default_rng(seed)
    img = rng.random((C,) + tuple(shape)).astype(np.float32)
    m = np.ones((1,) + tuple(shape), np.float32)
    for _ in range(3):
        m[(0,) + tuple(int(rng.integers(0, n)) for n in shape)] = 0
    return img, m


RUNS = {1: 0, 2: _lib.FG_PLAN_RUNS2}


def pin_cluster(shape, G, lean=False, rpt=1, S=4):
    """Pins a cluster plan of about G strips on every pass of a volume shape
    (rpt runs per thread: 1 the pass kernel, 2 the cluster sweep kernel)."""
    L = _lib.load()
    for cross, N1, N2 in tune.pass_keys(shape):
        T1 = -(-N1 // G)
        flags = _lib.FG_PLAN_CLUSTER | (_lib.FG_PLAN_LEAN if lean else 0) | RUNS[rpt]
        _lib.check(L.fg_plan_override(cross, N1, N2, S, T1, N2, flags))


def uses_cluster(shape, C=1, maps=1, mode=0, flag=_lib.FG_PLAN_CLUSTER):
    return all(_lib.plan_describe(*k, C, maps, mode)["lean"] & flag for k in tune.pass_keys(shape))


def t(a):
    return torch.from_numpy(np.ascontiguousarray(a))[None].cuda()


@pytest.mark.parametrize("shape", [(20, 33, 27), (24, 64, 64), (7, 18, 40)])
@pytest.mark.parametrize("G", [2, 5, 16])
def test_cluster_plans_give_the_oracle_bits(shape, G):
    img, m = case(shape, 1, sum(shape) + G)
    sp = [1.5, 0.8, 1.1]
    try:
        pin_cluster(shape, G)
        assert uses_cluster(shape)
        for lamb in (0.0, 0.6, 1.0):
            got = fg.generalised_geodesic3d(t(img), t(m), sp, 1e10, lamb, 2)[0].cpu().numpy()
            want = oracle.geodesic3d(img, m, sp, 1e10, lamb, 2)
            assert bits_equal(got, want), (shape, G, lamb, np.abs(got - want).max())
        fg.check_status()
    finally:
        tune.clear(shape)


def test_cluster_plans_lean_kernel_and_full_strips():
    # 16 strips of 16 rows x 256 columns: 1024 threads per CTA, 64-register kernel
    shape = (24, 256, 256)
    img, m = case(shape, 1, 5)
    sp = [1.0, 1.0, 1.0]
    try:
        pin_cluster(shape, 16, lean=True)
        assert _lib.plan_describe(2, 256, 256)["threads"] == 1024
        for lamb in (0.0, 0.5):
            got = fg.generalised_geodesic3d(t(img), t(m), sp, 1e10, lamb, 1)[0].cpu().numpy()
            assert bits_equal(got, oracle.geodesic3d(img, m, sp, 1e10, lamb, 1)), lamb
        fg.check_status()
    finally:
        tune.clear(shape)


def test_cluster_plans_channels_signed_gsf():
    shape = (12, 30, 44)
    img, m = case(shape, 3, 9)
    sp = [0.7, 1.3, 2.0]
    try:
        pin_cluster(shape, 4)
        assert uses_cluster(shape, C=3) and uses_cluster(shape, maps=2)
        got = fg.generalised_geodesic3d(t(img), t(m), sp, 1e10, 0.7, 2)[0].cpu().numpy()
        assert bits_equal(got, oracle.geodesic3d(img, m, sp, 1e10, 0.7, 2))
        img1, m1 = case(shape, 1, 10)
        m1 = np.random.default_rng(3).random(m1.shape).astype(np.float32)
        got = fg.signed_generalised_geodesic3d(t(img1), t(m1), sp, 1e10, 0.5, 2)[0].cpu().numpy()
        assert bits_equal(got, oracle.signed3d(img1, m1, sp, 1e10, 0.5, 2))
        got = fg.GSF3d(t(img1), t(m1), 0.5, sp, 1e10, 1.0, 2)[0].cpu().numpy()
        assert bits_equal(got, oracle.gsf3d(img1, m1, 0.5, sp, 1e10, 1.0, 2))
        fg.check_status()
    finally:
        tune.clear(shape)


def test_concurrent_cluster_transforms():
    # several transforms on their own streams, each a cluster at a time
    shape = (16, 64, 128)
    img, m = case(shape, 1, 21)
    sp = [2.0, 0.5, 0.5]
    lambs = [0.0, 0.3, 0.6, 1.0, 0.8, 0.1]
    try:
        pin_cluster(shape, 8)
        ti, tm = t(img), t(m)
        torch.cuda.synchronize()
        streams = [torch.cuda.Stream() for _ in lambs]
        outs = []
        for lamb, s in zip(lambs, streams):
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                outs.append(fg.generalised_geodesic3d(ti, tm, sp, 1e10, lamb, 2))
        torch.cuda.synchronize()
        for lamb, o in zip(lambs, outs):
            assert bits_equal(o[0].cpu().numpy(), oracle.geodesic3d(img, m, sp, 1e10, lamb, 2)), lamb
        fg.check_status()
    finally:
        tune.clear(shape)


@pytest.mark.parametrize("shape", [(20, 33, 27), (24, 64, 64), (7, 18, 40), (13, 100, 36)])
@pytest.mark.parametrize("G", [2, 5, 16])
@pytest.mark.parametrize("rpt", [2])
def test_cluster_sweep_kernel_gives_the_oracle_bits(shape, G, rpt):
    img, m = case(shape, 1, sum(shape) * rpt + G)
    sp = [1.5, 0.8, 1.1]
    try:
        pin_cluster(shape, G, rpt=rpt, S=8)
        for mode in (0, 1, 2):
            assert uses_cluster(shape, mode=mode, flag=RUNS[rpt]), mode
        for lamb in (0.0, 0.6, 1.0):
            got = fg.generalised_geodesic3d(t(img), t(m), sp, 1e10, lamb, 2)[0].cpu().numpy()
            want = oracle.geodesic3d(img, m, sp, 1e10, lamb, 2)
            assert bits_equal(got, want), (shape, G, rpt, lamb, np.abs(got - want).max())
        fg.check_status()
    finally:
        tune.clear(shape)


@pytest.mark.parametrize("rpt", [2])
def test_cluster_sweep_kernel_full_strips_signed_gsf_channels(rpt):
    shape = (20, 256, 256)
    img, m = case(shape, 1, 77 + rpt)
    sp = [1.0, 1.0, 1.0]
    try:
        pin_cluster(shape, 16, rpt=rpt, S=8)
        assert uses_cluster(shape, flag=RUNS[rpt])
        # two maps: the 20 x 256 sections on the sweep kernel (256 x 256 ones do not fit its rings)
        assert _lib.plan_describe(2, 20, 256, 1, 2, 0)["lean"] & RUNS[rpt]
        for lamb in (0.0, 0.5):
            got = fg.generalised_geodesic3d(t(img), t(m), sp, 1e10, lamb, 1)[0].cpu().numpy()
            assert bits_equal(got, oracle.geodesic3d(img, m, sp, 1e10, lamb, 1)), lamb
        m2 = np.random.default_rng(5).random(m.shape).astype(np.float32)
        got = fg.signed_generalised_geodesic3d(t(img), t(m2), sp, 1e10, 0.5, 1)[0].cpu().numpy()
        assert bits_equal(got, oracle.signed3d(img, m2, sp, 1e10, 0.5, 1))
        got = fg.GSF3d(t(img), t(m2), 0.5, sp, 1e10, 1.0, 1)[0].cpu().numpy()
        assert bits_equal(got, oracle.gsf3d(img, m2, 0.5, sp, 1e10, 1.0, 1))
        # three image channels: these passes keep a plan of the pass kernel
        img3, _ = case(shape, 3, 5)
        got = fg.generalised_geodesic3d(t(img3), t(m), sp, 1e10, 0.5, 1)[0].cpu().numpy()
        assert bits_equal(got, oracle.geodesic3d(img3, m, sp, 1e10, 0.5, 1))
        fg.check_status()
    finally:
        tune.clear(shape)


def test_cluster_capacity_matches_what_runs():
    # 16-CTA clusters of the b256 plan: the device runs at least one, at most 152 / 16
    n = _lib.cluster_capacity(16, 512, 188 * 1024)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert 1 <= n <= sms // 16
    assert _lib.cluster_capacity(2, 512, 188 * 1024) >= n
