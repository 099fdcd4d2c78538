"""Failure detection on the GPU without a fault: the engine's bounded wait
routines, run on something that never happens (an exchange word nobody
publishes, an mbarrier phase whose bytes never arrive, a group counter that
never reaches its target), give up within their limit, record
FG_ERR_TIMEOUT in the workspace status word, and leave the context usable."""
import time

import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_bounded_wait_gives_up_and_reports(kind):
    L = _lib.load()
    ws = torch.zeros(1 << 16, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert L.fg_workspace_status(ws.data_ptr(), s) == _lib.FG_OK
    t0 = time.perf_counter()
    _lib.check(L.fg_selftest_wait(kind, ws.data_ptr(), ws.numel(), s))
    assert L.fg_workspace_status(ws.data_ptr(), s) == _lib.FG_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 10.0
    assert L.fg_workspace_status(ws.data_ptr(), s) == _lib.FG_OK  # read and cleared
    # the context is usable: a transform afterwards gives the oracle's bits
    rng = np.random.default_rng(kind)
    img = rng.random((1, 12, 30, 44)).astype(np.float32)
    m = np.ones((1, 12, 30, 44), np.float32)
    m[0, 3, 4, 5] = 0
    got = fg.generalised_geodesic3d(torch.from_numpy(img)[None].cuda(), torch.from_numpy(m)[None].cuda(),
                                    [1.0, 1.0, 1.0], 1e10, 0.5, 2)[0].cpu().numpy()
    assert bits_equal(got, oracle.geodesic3d(img, m, [1.0, 1.0, 1.0], 1e10, 0.5, 2))
    fg.check_status()


def test_selftest_arguments():
    L = _lib.load()
    ws = torch.zeros(1 << 16, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    assert L.fg_selftest_wait(3, ws.data_ptr(), ws.numel(), s) == _lib.FG_ERR_INVALID_ARGUMENT
    assert L.fg_selftest_wait(0, ws.data_ptr(), 64, s) == _lib.FG_ERR_WORKSPACE
