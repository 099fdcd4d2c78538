"""A batch of volumes in one persistent launch (PersistentBatch3d): uneven
sizes, spacings and lambs, plain and signed, replayed from a CUDA graph,
every output bit-identical to the oracle; the queue's ordering and the
per-volume progress counters are exercised by batches with more volumes
than co-resident clusters and by forced cluster sizes."""
import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu

SHAPES = [(20, 33, 27), (7, 18, 40), (24, 64, 64), (1, 12, 17), (9, 1, 13), (40, 8, 8), (16, 16, 16), (5, 30, 4)]
SPACINGS = [(1.5, 0.8, 1.1), (1.0, 1.0, 1.0), (2.0, 0.5, 0.5), (0.7, 1.3, 2.2), (1.0, 0.6, 0.9), (3.0, 1.0, 1.0),
            (1.0, 1.0, 1.0), (0.5, 2.0, 1.0)]
LAMBS = [0.5, 0.0, 1.0, 0.3, 0.8, 0.0, 1.0, 0.65]


def volumes(seed, shapes):
    rng = np.random.default_rng(seed)
    imgs, msks = [], []
    for s in shapes:
        imgs.append(rng.random((1, 1) + s).astype(np.float32))
        m = np.ones((1, 1) + s, np.float32)
        for _ in range(2):
            m[(0, 0) + tuple(int(rng.integers(0, n)) for n in s)] = 0
        msks.append(m)
    return imgs, msks


def run_batch(imgs, msks, lambs, spacings, signed, iterations=2, graph=True, cluster_size=None, repeat=2):
    ti = [torch.from_numpy(a).cuda() for a in imgs]
    tm = [torch.from_numpy(a).cuda() for a in msks]
    b = fg.PersistentBatch3d([tuple(a.shape[1:]) for a in imgs], signed=signed, iterations=iterations,
                             use_graph=graph, inputs=(ti, tm), cluster_size=cluster_size)
    b.v, b.lambs, b.spacings = 1e10, list(lambs), list(spacings)
    for _ in range(repeat):
        outs = b.run()
    torch.cuda.synchronize()
    b.check()
    return b, [o[0].cpu().numpy() for o in outs]


@pytest.mark.parametrize("signed", [False, True])
@pytest.mark.parametrize("graph", [False, True])
def test_uneven_volumes_one_launch(signed, graph):
    imgs, msks = volumes(7 + signed, SHAPES)
    b, outs = run_batch(imgs, msks, LAMBS, SPACINGS, signed, graph=graph)
    assert b.info["mode"] == 0  # mixed lambs: the general expression for every pass
    f = oracle.signed3d if signed else oracle.geodesic3d
    for im, m, sp, lamb, got in zip(imgs, msks, SPACINGS, LAMBS, outs):
        want = f(im[0], m[0], sp, 1e10, lamb, 2)
        assert bits_equal(got, want), (im.shape, sp, lamb, float(np.nanmax(np.abs(got - want))))


@pytest.mark.parametrize("lamb,mode", [(0.0, 1), (1.0, 2), (0.4, 0)])
def test_one_mode_batches_take_the_specialised_body(lamb, mode):
    shapes = [(12, 40, 36), (6, 20, 20), (18, 24, 52)]
    imgs, msks = volumes(11, shapes)
    sps = [(1.0, 1.0, 1.0), (2.0, 0.5, 0.5), (1.2, 0.9, 1.1)]
    b, outs = run_batch(imgs, msks, [lamb] * 3, sps, False)
    assert b.info["mode"] == mode
    for im, m, sp, got in zip(imgs, msks, sps, outs):
        assert bits_equal(got, oracle.geodesic3d(im[0], m[0], sp, 1e10, lamb, 2)), (im.shape, lamb)


@pytest.mark.parametrize("G", [1, 2, 4])
def test_more_volumes_than_clusters(G):
    """Small clusters and many volumes: chains interleave across clusters,
    jobs wait on their volume's progress counter."""
    shapes = [(10 + k, 12 + 2 * k, 16) for k in range(12)]
    imgs, msks = volumes(20 + G, shapes)
    lambs = [[0.0, 0.5, 1.0][k % 3] for k in range(12)]
    sps = [(1.0, 1.0, 1.0)] * 12
    b, outs = run_batch(imgs, msks, lambs, sps, False, iterations=3, cluster_size=G)
    assert b.info["cluster_size"] == G
    for im, m, lamb, got in zip(imgs, msks, lambs, outs):
        assert bits_equal(got, oracle.geodesic3d(im[0], m[0], (1.0, 1.0, 1.0), 1e10, lamb, 3)), (im.shape, lamb)


def test_large_volumes_one_launch():
    shapes = [(48, 128, 128), (64, 96, 160), (32, 256, 256)]
    imgs, msks = volumes(31, shapes)
    lambs = [0.5, 0.0, 1.0]
    sps = [(1.0, 1.0, 1.0), (2.0, 0.5, 0.5), (1.0, 0.7, 0.7)]
    b, outs = run_batch(imgs, msks, lambs, sps, False, iterations=2)
    for im, m, sp, lamb, got in zip(imgs, msks, sps, lambs, outs):
        assert bits_equal(got, oracle.geodesic3d(im[0], m[0], sp, 1e10, lamb, 2)), (im.shape, lamb)
    fg.check_status()
