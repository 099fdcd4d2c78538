"""GPU parity of Toivanen's raster scan (the wavefront kernel) against the C
oracle, which is pinned to the reference's own CPU output by the golden
vectors (tests/test_oracle_golden.py).  The golden cases themselves run in
tests/test_parity_gpu.py::test_golden_bits."""
import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu


def case(rng, shape, C, nseeds=3, soft=False):
    img = (rng.random((C,) + shape) * 255).astype(np.float32)
    if soft:
        m = rng.random((1,) + shape).astype(np.float32)
    else:
        m = np.ones((1,) + shape, np.float32)
        for _ in range(nseeds):
            m[(0,) + tuple(int(rng.integers(0, n)) for n in shape)] = 0
    return img, m


def t(a):
    return torch.from_numpy(np.ascontiguousarray(a))[None].cuda()


# up to 1024 rows: one thread per row; taller images: the wave kernel
# (rows of a multiple of 4 cells read and write their own cells four at a time)
@pytest.mark.parametrize("shape", [(1, 1), (1, 37), (29, 1), (2, 3), (130, 97), (64, 200), (257, 31), (1024, 9),
                                   (1100, 23), (1, 4), (5, 12), (300, 128), (1024, 16), (512, 512)])
@pytest.mark.parametrize("C", [1, 3])
def test_2d_vs_oracle(shape, C):
    rng = np.random.default_rng(sum(shape) * 7 + C)
    img, m = case(rng, shape, C)
    for lamb, it in [(0.0, 1), (0.6, 2), (1.0, 2)]:
        got = fg.generalised_geodesic2d_toivanen(t(img), t(m), 1e10, lamb, it)[0].cpu().numpy()
        want = oracle.toivanen2d(img, m, 1e10, lamb, it)
        assert bits_equal(got, want), (shape, C, lamb, it, np.abs(got - want).max())


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 9, 13), (9, 1, 13), (9, 13, 1), (5, 6, 7), (20, 33, 27),
                                   (11, 40, 9)])
@pytest.mark.parametrize("C", [1, 2])
def test_3d_vs_oracle(shape, C):
    rng = np.random.default_rng(sum(shape) * 11 + C)
    img, m = case(rng, shape, C)
    for sp, lamb, it in [([1.0, 1.0, 1.0], 0.0, 1), ([2.0, 0.5, 0.7], 0.5, 2), ([0.6, 1.3, 2.2], 1.0, 1)]:
        got = fg.generalised_geodesic3d_toivanen(t(img), t(m), sp, 1e10, lamb, it)[0].cpu().numpy()
        want = oracle.toivanen3d(img, m, sp, 1e10, lamb, it)
        assert bits_equal(got, want), (shape, C, sp, lamb, it, np.abs(got - want).max())


@pytest.mark.parametrize("shape", [(64, 128, 256)])
def test_3d_groups_vs_oracle(shape):
    """A volume whose waves hold more than 4096 cells (8192): a cooperative
    group of CTAs per map with a bounded barrier between waves; plain and
    signed."""
    rng = np.random.default_rng(sum(shape))
    img, m = case(rng, shape, 1)
    got = fg.generalised_geodesic3d_toivanen(t(img), t(m), [1.0, 0.7, 1.3], 1e10, 0.6, 1)[0].cpu().numpy()
    assert bits_equal(got, oracle.toivanen3d(img, m, [1.0, 0.7, 1.3], 1e10, 0.6, 1))
    got = fg.signed_generalised_geodesic3d_toivanen(t(img), t(m), [1.0, 1.0, 1.0], 1e10, 1.0, 1)[0].cpu().numpy()
    assert bits_equal(got, oracle.toivanen3d(img, m, [1.0, 1.0, 1.0], 1e10, 1.0, 1, signed=True))


def test_signed_gsf_many_channels_and_soft_masks():
    rng = np.random.default_rng(31)
    img, m = case(rng, (70, 45), 5, soft=True)  # five channels: no channel limit on this path
    got = fg.signed_generalised_geodesic2d_toivanen(t(img), t(m), 3.0, 0.4, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.toivanen2d(img, m, 3.0, 0.4, 2, signed=True))
    got = fg.GSF2d_toivanen(t(img), t(m), 0.3, 3.0, 0.9, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.gsf_toivanen2d(img, m, 0.3, 3.0, 0.9, 2))
    vol, vm = case(rng, (12, 15, 18), 1)
    sp = [1.5, 0.7, 1.1]
    got = fg.signed_generalised_geodesic3d_toivanen(t(vol), t(vm), sp, 1e10, 0.5, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.toivanen3d(vol, vm, sp, 1e10, 0.5, 2, signed=True))
    got = fg.GSF3d_toivanen(t(vol), t(vm), 0.5, sp, 1e10, 1.0, 1)[0].cpu().numpy()
    assert bits_equal(got, oracle.gsf_toivanen3d(vol, vm, 0.5, sp, 1e10, 1.0, 1))
    fg.check_status()


def test_host_tensors_and_mask_channels():
    rng = np.random.default_rng(8)
    img, _ = case(rng, (40, 52), 1)
    m = rng.random((2, 40, 52)).astype(np.float32)  # two mask channels: only channel 0 is swept
    got = fg.generalised_geodesic2d_toivanen(torch.from_numpy(img)[None], torch.from_numpy(m)[None], 2.0, 0.5, 2)
    assert not got.is_cuda and got.shape == (1, 2, 40, 52)
    assert bits_equal(got[0].numpy(), oracle.toivanen2d(img, m, 2.0, 0.5, 2))


def test_toivanen_and_raster_scans_reach_the_same_fixed_point():
    # two different scans of the same 8-connected graph with the same step
    # costs: they differ after few iterations and agree once both converge
    rng = np.random.default_rng(4)
    img, m = case(rng, (24, 31), 1)
    a1 = fg.generalised_geodesic2d_toivanen(t(img), t(m), 1e10, 0.7, 1)
    b1 = fg.generalised_geodesic2d(t(img), t(m), 1e10, 0.7, 1)
    assert not torch.equal(a1, b1)
    a = fg.generalised_geodesic2d_toivanen(t(img), t(m), 1e10, 0.7, 40)
    b = fg.generalised_geodesic2d(t(img), t(m), 1e10, 0.7, 40)
    assert torch.allclose(a, b, rtol=1e-5, atol=1e-4)


def test_large_volume_grouped_ctas():
    # 6400 cells per wave: each map is swept by a group of CTAs ordered by a
    # grid barrier; plain (one group), signed (two) and GSF (four at once)
    rng = np.random.default_rng(12)
    vol, vm = case(rng, (64, 200, 200), 1)
    sp = [1.0, 0.8, 1.2]
    got = fg.generalised_geodesic3d_toivanen(t(vol), t(vm), sp, 1e10, 0.5, 1)[0].cpu().numpy()
    assert bits_equal(got, oracle.toivanen3d(vol, vm, sp, 1e10, 0.5, 1))
    got = fg.signed_generalised_geodesic3d_toivanen(t(vol), t(vm), sp, 1e10, 1.0, 1)[0].cpu().numpy()
    assert bits_equal(got, oracle.toivanen3d(vol, vm, sp, 1e10, 1.0, 1, signed=True))
    got = fg.GSF3d_toivanen(t(vol), t(vm), 0.5, sp, 1e10, 0.7, 1)[0].cpu().numpy()
    assert bits_equal(got, oracle.gsf_toivanen3d(vol, vm, 0.5, sp, 1e10, 0.7, 1))
    fg.check_status()
