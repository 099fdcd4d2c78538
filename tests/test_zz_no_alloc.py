"""The allocation-free entry point fg_generalised_geodesic2d_noalloc.

It serves callers that cannot allocate device memory when they need a
distance map (code inside a framework that owns the allocator and forbids
allocation during execution, or C callers without an allocator): its scratch
is a fixed 16 MiB device array inside the library.  Checked here through the
C ABI against the ordinary workspace entry point, on calls in a row with
different inputs, so leftover scratch contents of one call must not affect
the next -- including a 1024 x 1000 image swept on several tiles, whose halo
exchange words live in the fixed array -- and the array's status word must
read FG_OK afterwards (fg_noalloc_status).  This file is collected last on
purpose.
"""
import ctypes

import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib

pytestmark = pytest.mark.gpu


def noalloc(img, msk, v, lamb, iters):
    L = _lib.load()
    out = torch.empty_like(msk)
    C, H, W = img.shape[1], img.shape[2], img.shape[3]
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.fg_generalised_geodesic2d_noalloc(img.data_ptr(), C, H, W, msk.data_ptr(), msk.shape[1], out.data_ptr(),
                                             v, lamb, 1.0 - lamb, iters, stream)
    _lib.check(rc)
    return out


def case(seed, C, H, W):
    g = torch.Generator().manual_seed(seed)
    img = (torch.rand((1, C, H, W), generator=g) * 255).cuda()
    msk = torch.ones((1, 1, H, W))
    msk[0, 0, H // 3:H // 3 + 3, W // 2:W // 2 + 4] = 0
    return img, msk.cuda()


@pytest.fixture
def tiled_plans():
    """Planner limits that cut every row into regions of at most 256 cells,
    so rows above 512 cells run on several tiles with halo exchange words."""
    L = _lib.load()
    _lib.check(L.fg_set_tuning(256, 0))
    yield
    _lib.check(L.fg_set_tuning(0, 0))


def test_noalloc_matches_workspace_entry_on_two_calls():
    inputs = [(case(1, 1, 300, 417), 0.7, 2), (case(2, 3, 256, 200), 1.0, 3)]
    got = []
    for (img, msk), lamb, it in inputs:
        got.append(noalloc(img, msk, 1e10, lamb, it))
    torch.cuda.synchronize()
    for ((img, msk), lamb, it), a in zip(inputs, got):
        b = fg.generalised_geodesic2d(img, msk, 1e10, lamb, it)
        # the parity tests' bar: identical bits
        assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    _lib.check(_lib.load().fg_noalloc_status(torch.cuda.current_stream().cuda_stream))


def test_noalloc_multi_tile_after_a_smaller_call(tiled_plans):
    L = _lib.load()
    plan = _lib.plan_describe(1, 1, 1000, C=1, maps=1, mode=0)
    assert plan["tiles1"] * plan["tiles2"] > 1  # the exchange words are in use
    inputs = [(case(3, 1, 200, 180), 0.4, 2), (case(4, 1, 1024, 1000), 0.6, 2), (case(5, 1, 1024, 1000), 0.9, 2)]
    got = [noalloc(img, msk, 1e10, lamb, it) for (img, msk), lamb, it in inputs]
    _lib.check(L.fg_noalloc_status(torch.cuda.current_stream().cuda_stream))
    for ((img, msk), lamb, it), a in zip(inputs, got):
        b = fg.generalised_geodesic2d(img, msk, 1e10, lamb, it)
        assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    fg.check_status()


def test_noalloc_refuses_sizes_beyond_its_scratch():
    L = _lib.load()
    small = torch.zeros(16, device="cuda")
    p = small.data_ptr()
    rc = L.fg_generalised_geodesic2d_noalloc(p, 1, 4096, 4096, p, 1, p, 1e10, 1.0, 0.0, 2,
                                             torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.FG_ERR_UNSUPPORTED
    assert "scratch" in _lib.last_error()
