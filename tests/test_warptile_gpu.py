"""Warp tiles: a 2D pass over rows of up to 1024 cells in one CTA, a warp
per strip of the row with 4 cells per lane, neighbours by shuffles, halos of
S cells handed over through shared memory every S steps
(fastgeodis_gb300/csrc/fg_warptile2d.cu).  The planner takes them for rows of
up to 1024 cells with one image channel read (or none); here they are also
forced with fg_plan_override(FG_PLAN_WARPS) through every variant (one or
two maps, the three arithmetic modes, S from 4 to 32, rows that are not a
multiple of 4, a row of one warp, a short last warp).  The bar is the
oracle's bits."""
import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib, tune
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu

WARPS = _lib.FG_PLAN_WARPS


def _case(shape, C, seed, soft=False):
    rng = np.random.default_rng(seed)
    img = (rng.random((C,) + tuple(shape)) * 80).astype(np.float32)
    m = rng.random((1,) + tuple(shape)).astype(np.float32) if soft else np.ones((1,) + tuple(shape), np.float32)
    for _ in range(3):
        m[(0,) + tuple(int(rng.integers(0, n)) for n in shape)] = 0
    return img, m


def _run(op, img, m, lamb, it=2):
    ti, tm = (torch.from_numpy(a)[None].cuda() for a in (img, m))
    if op == "plain":
        return fg.generalised_geodesic2d(ti, tm, 1e10, lamb, it)[0].cpu().numpy(), \
            oracle.geodesic2d(img, m, 1e10, lamb, it)
    if op == "signed":
        return fg.signed_generalised_geodesic2d(ti, tm, 1e10, lamb, it)[0].cpu().numpy(), \
            oracle.signed2d(img, m, 1e10, lamb, it)
    return fg.GSF2d(ti, tm, 0.4, 1e10, lamb, 1)[0].cpu().numpy(), oracle.gsf2d(img, m, 0.4, 1e10, lamb, 1)


@pytest.mark.parametrize("op,lamb,S,shape", [
    ("plain", 0.6, 16, (97, 211)),
    ("plain", 0.0, 4, (97, 211)),     # l_grad == 0: no image term
    ("plain", 1.0, 32, (150, 300)),   # l_eucl == 0, l_grad == 1
    ("plain", 0.3, 8, (130, 257)),    # rows not a multiple of 4
    ("plain", 0.8, 16, (1024, 120)),  # one warp along W, 11 warps along H
    ("plain", -0.4, 16, (300, 1000)),
    ("signed", 0.5, 32, (97, 211)),
    ("signed", 1.0, 8, (200, 129)),   # 129 cells: two warps, the second holding one cell
    ("gsf", 0.7, 16, (61, 333)),
])
def test_forced_warp_tiles(op, lamb, S, shape):
    img, m = _case(shape, 1, 17 + S, soft=op == "gsf")
    try:
        tune.pin({k: (S, 1, 1, WARPS) for k in tune.pass_keys(shape)})
        for k in tune.pass_keys(shape):
            p = _lib.plan_describe(*k)
            assert p["lean"] == WARPS and p["K2"] == (S if k[2] > 128 else 0), (k, p)
        got, want = _run(op, img, m, lamb)
        assert bits_equal(got, want), float(np.nanmax(np.abs(got - want)))
        fg.check_status()
    finally:
        tune.clear(shape)


@pytest.mark.parametrize("shape", [(512, 512), (700, 1024), (128, 128), (3000, 40), (33, 999), (1, 600), (600, 1)])
def test_planner_warp_tiles(shape):
    """The planner's own plan: warp tiles for rows of up to 1024 cells with
    one image channel (halos of 16), row tiles beyond; plain, signed and
    GSF against the oracle."""
    for k in tune.pass_keys(shape):
        p = _lib.plan_describe(*k)
        assert bool(p["lean"] & WARPS) == (k[2] <= 1024), (k, p)
    img, m = _case(shape, 1, 3)
    for op, lamb in (("plain", 1.0), ("signed", 0.5), ("gsf", 0.8)):
        got, want = _run(op, img, m, lamb)
        assert bits_equal(got, want), (op, float(np.nanmax(np.abs(got - want))))
    fg.check_status()


def test_warp_tiles_refuse_more_channels():
    """Two or more image channels read: the planner keeps row tiles, and a
    pinned warp-tile plan falls back to the planner's."""
    shape = (90, 300)
    img, m = _case(shape, 3, 9)
    assert not _lib.plan_describe(1, 1, 300, C=3)["lean"] & WARPS
    try:
        tune.pin({k: (16, 1, 1, WARPS) for k in tune.pass_keys(shape)})
        assert not _lib.plan_describe(1, 1, 300, C=3)["lean"] & WARPS
        got, want = _run("plain", img, m, 0.5)
        assert bits_equal(got, want)
        got = fg.generalised_geodesic2d(*(torch.from_numpy(a)[None].cuda() for a in (img, m)), 1e10, 0.0, 2)
        assert bits_equal(got[0].cpu().numpy(), oracle.geodesic2d(img, m, 1e10, 0.0, 2))  # no image read: warp tiles
    finally:
        tune.clear(shape)
