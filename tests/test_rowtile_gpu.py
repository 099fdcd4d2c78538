"""Row tiles: 2D passes whose rows are split into tiles of T2 cells, one CTA
per tile and one thread per cell of the tile and its halos of S cells, with
a hand-off of the halos through exchange words every S steps
(fastgeodis_gb300/csrc/fg_rowtile2d.cu).  The planner takes them for every
2D pass of 1 to 4 image channels; here they are also forced with fg_plan_override
(FG_PLAN_ROWS) onto small images, through every variant (1 to 4 channels,
one or two maps, the three arithmetic modes, S from 1 to 32, hand-offs
through global memory or within a thread-block cluster; the passes that
change layout run in place and a transpose follows).  The bar is the
oracle's bits."""
import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib, tune
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu

ROWS = _lib.FG_PLAN_ROWS
CLU = _lib.FG_PLAN_CLUSTER


def _case(shape, C, seed, soft=False):
    rng = np.random.default_rng(seed)
    img = (rng.random((C,) + tuple(shape)) * 80).astype(np.float32)
    m = rng.random((1,) + tuple(shape)).astype(np.float32) if soft else np.ones((1,) + tuple(shape), np.float32)
    for _ in range(3):
        m[(0,) + tuple(int(rng.integers(0, n)) for n in shape)] = 0
    return img, m


def _pin(shape, S, T2, flags=ROWS):
    tune.pin({k: (S, 1, T2, flags) for k in tune.pass_keys(shape)})
    for k in tune.pass_keys(shape):
        p = _lib.plan_describe(*k)
        assert p["lean"] == flags and p["S"] == S and p["tiles2"] > 1, (k, p)


@pytest.mark.parametrize("op,C,lamb,S,T2", [
    ("plain", 1, 0.6, 8, 32),
    ("plain", 1, 0.0, 4, 20),    # l_grad == 0: no image term
    ("plain", 1, 1.0, 32, 64),   # l_eucl == 0, l_grad == 1
    ("plain", 3, 0.5, 16, 48),
    ("plain", 4, 0.3, 2, 12),
    ("plain", 2, 0.8, 1, 8),     # a hand-off every step
    ("plain", 1, 0.6, 1, 64),    # a hand-off every step, 3 warps per tile: two ring rows at least
    ("signed", 2, 0.7, 1, 40),
    ("signed", 1, 0.5, 32, 40),
    ("signed", 3, 1.0, 8, 44),
    ("gsf", 1, 0.7, 16, 36),
])
def test_forced_row_tiles(op, C, lamb, S, T2):
    _forced(op, C, lamb, S, T2, ROWS)


def _forced(op, C, lamb, S, T2, flags):
    shape = (97, 211)  # the passes along H have rows of 211 cells, those along W rows of 97
    img, m = _case(shape, C, 11 + C + S, soft=op == "gsf")
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    try:
        _pin(shape, S, T2, flags)
        if op == "plain":
            got = fg.generalised_geodesic2d(ti, tm, 1e10, lamb, 2)
            want = oracle.geodesic2d(img, m, 1e10, lamb, 2)
        elif op == "signed":
            got = fg.signed_generalised_geodesic2d(ti, tm, 1e10, lamb, 2)
            want = oracle.signed2d(img, m, 1e10, lamb, 2)
        else:
            got = fg.GSF2d(ti, tm, 0.4, 1e10, lamb, 1)
            want = oracle.gsf2d(img, m, 0.4, 1e10, lamb, 1)
        got = got[0].cpu().numpy()
        assert bits_equal(got, want), float(np.nanmax(np.abs(got - want)))
        fg.check_status()
    finally:
        tune.clear(shape)


@pytest.mark.parametrize("op,C,lamb,S,T2", [
    ("plain", 1, 0.6, 8, 32),
    ("plain", 1, 0.0, 4, 20),
    ("plain", 1, 1.0, 32, 64),
    ("plain", 3, 0.5, 16, 48),
    ("plain", 4, 0.3, 2, 16),
    ("plain", 2, 0.8, 1, 16),    # a hand-off every step
    ("plain", 1, 0.6, 1, 64),
    ("signed", 1, 0.5, 32, 40),
    ("signed", 3, 1.0, 8, 44),
    ("gsf", 1, 0.7, 16, 36),
])
def test_forced_cluster_row_tiles(op, C, lamb, S, T2):
    """Row tiles as one thread-block cluster (FG_PLAN_ROWS | FG_PLAN_CLUSTER):
    the halos handed over through distributed shared memory."""
    _forced(op, C, lamb, S, T2, ROWS | CLU)


@pytest.mark.parametrize("op,C,lamb", [("plain", 1, 0.6), ("plain", 3, 1.0), ("signed", 2, 0.4), ("gsf", 1, 0.8)])
def test_single_tile_row_tiles(op, C, lamb):
    """A row-tile plan of one tile (T2 >= the row): the whole row on one CTA,
    one thread per cell, no halos and no hand-off."""
    shape = (97, 211)
    img, m = _case(shape, C, 61 + C, soft=op == "gsf")
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    try:
        tune.pin({k: (32, 1, 512, ROWS) for k in tune.pass_keys(shape)})
        for k in tune.pass_keys(shape):
            p = _lib.plan_describe(*k)
            assert p["lean"] == ROWS and p["tiles2"] == 1 and p["K2"] == 0, (k, p)
        if op == "plain":
            got, want = fg.generalised_geodesic2d(ti, tm, 1e10, lamb, 2), oracle.geodesic2d(img, m, 1e10, lamb, 2)
        elif op == "signed":
            got, want = fg.signed_generalised_geodesic2d(ti, tm, 1e10, lamb, 2), oracle.signed2d(img, m, 1e10, lamb, 2)
        else:
            got, want = fg.GSF2d(ti, tm, 0.4, 1e10, lamb, 1), oracle.gsf2d(img, m, 0.4, 1e10, lamb, 1)
        assert bits_equal(got[0].cpu().numpy(), want)
        fg.check_status()
    finally:
        tune.clear(shape)


@pytest.mark.parametrize("shape,S", [((150, 492), 32), ((492, 150), 16), ((40, 512), 32)])
def test_cluster_row_tiles_with_a_short_last_tile(shape, S):
    """16 tiles of 32 cells whose last tile holds fewer cells than a halo
    (492 = 15 x 32 + 12), and 5 tiles of a 150-cell row: the cluster form
    expects only the cells that exist."""
    img, m = _case(shape, 1, 41 + S)
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    try:
        _pin(shape, S, 32, ROWS | CLU)
        for lamb in (0.4, 1.0):
            got = fg.generalised_geodesic2d(ti, tm, 1e10, lamb, 2)[0].cpu().numpy()
            assert bits_equal(got, oracle.geodesic2d(img, m, 1e10, lamb, 2)), lamb
        got = fg.signed_generalised_geodesic2d(ti, tm, 1e10, 0.6, 1)[0].cpu().numpy()
        assert bits_equal(got, oracle.signed2d(img, m, 1e10, 0.6, 1))
        fg.check_status()
    finally:
        tune.clear(shape)


@pytest.mark.parametrize("shape,C", [((1500, 1300), 1), ((700, 2100), 3), ((3000, 600), 1), ((512, 512), 1),
                                     ((200, 384), 4), ((128, 130), 2), ((90, 700), 1), ((64, 512), 1),
                                     ((40, 900), 2), ((100, 200), 1), ((3000, 20), 3), ((7, 4000), 1)])
def test_planner_row_tiles(shape, C):
    """The planner's own plan for every 2D pass: row tiles with a hand-off
    every 32 steps (one tile for rows of up to 32 cells, a cluster of up to
    16 tiles for rows of up to 1024)."""
    assert not _lib.runs_in_one_launch(shape)
    for k in tune.pass_keys(shape):
        p = _lib.plan_describe(*k, C=C)
        assert p["lean"] & ROWS and (p["tiles2"] == 1) == (k[2] <= 32), (k, p)
        assert bool(p["lean"] & CLU) == (32 < k[2] <= 1024), (k, p)
    img, m = _case(shape, C, 5 + C)
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    got = fg.generalised_geodesic2d(ti, tm, 1e10, 0.5, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.geodesic2d(img, m, 1e10, 0.5, 2))
    got = fg.signed_generalised_geodesic2d(ti, tm, 1e10, 1.0, 1)[0].cpu().numpy()
    assert bits_equal(got, oracle.signed2d(img, m, 1e10, 1.0, 1))
    fg.check_status()
