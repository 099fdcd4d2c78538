"""Every transform entry of the C ABI called directly (ctypes), the way a C
or C++ caller binds it: caller-owned device buffers and workspace, a stream
of the caller's, no Python layer in between.  Each result must equal the
oracle's bits; a workspace one byte short is refused before any launch; the
workspace status word reads FG_OK afterwards."""
import ctypes

import numpy as np
import pytest
import torch

from fastgeodis_gb300 import _lib
from golden_cases import bits_equal
from oracle import oracle

pytestmark = pytest.mark.gpu

F3 = ctypes.c_float * 3


def case(seed, C, shape, Cm=1):
    rng = np.random.default_rng(seed)
    img = (rng.random((C,) + shape) * 100).astype(np.float32)
    m = np.ones((Cm,) + shape, np.float32)
    if Cm > 1:
        m[1:] = rng.random((Cm - 1,) + shape).astype(np.float32)
    for _ in range(3):
        m[(0,) + tuple(int(rng.integers(0, n)) for n in shape)] = 0
    return img, m


def call(name, op, img, msk, *params, spacing=None, short=False):
    """Run the entry `name` on device copies of img [C, ...] / msk [Cm, ...]
    with a workspace from fg_workspace_bytes; returns the output (numpy)."""
    L = _lib.load()
    is3d = img.ndim == 4
    C, Cm = img.shape[0], msk.shape[0]
    D, H, W = img.shape[1:] if is3d else (1,) + img.shape[1:]
    di = torch.from_numpy(img).cuda()
    dm = torch.from_numpy(msk).cuda()
    out = torch.full(msk.shape, float("nan"), device="cuda")
    need = int(L.fg_workspace_bytes(op, C, D, H, W))
    ws = torch.zeros(need, dtype=torch.uint8, device="cuda")
    size = need - 1 if short else need
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    fn = getattr(L, name)
    dims = (C, D, H, W) if is3d else (C, H, W)
    sp = F3(*spacing) if is3d else None
    if name.startswith("fg_GSF"):
        theta, v, lamb, it = params
        if is3d:
            rc = fn(di.data_ptr(), *dims, dm.data_ptr(), Cm, theta, sp, v, lamb, it, out.data_ptr(), ws.data_ptr(),
                    size, sh)
        else:
            rc = fn(di.data_ptr(), *dims, dm.data_ptr(), Cm, theta, v, lamb, it, out.data_ptr(), ws.data_ptr(), size, sh)
    else:
        v, lamb, it = params
        lg, le = lamb, 1.0 - lamb
        if is3d:
            rc = fn(di.data_ptr(), *dims, dm.data_ptr(), Cm, sp, out.data_ptr(), v, lg, le, it, ws.data_ptr(), size,
                    sh)
        else:
            rc = fn(di.data_ptr(), *dims, dm.data_ptr(), Cm, out.data_ptr(), v, lg, le, it, ws.data_ptr(), size, sh)
    if short:
        return rc
    _lib.check(rc)
    _lib.check(L.fg_workspace_status(ws.data_ptr(), sh))
    stream.synchronize()
    return out.cpu().numpy()


P, S, G = _lib.FG_OP_PLAIN, _lib.FG_OP_SIGNED, _lib.FG_OP_GSF


@pytest.mark.parametrize("C,Cm,shape", [(1, 1, (37, 53)), (3, 2, (130, 96)), (5, 1, (600, 40))])
def test_2d_entries(C, Cm, shape):
    img, m = case(C * 10 + Cm, C, shape, Cm)
    v, lamb, it = 1e10, 0.6, 2
    assert bits_equal(call("fg_generalised_geodesic2d", P, img, m, v, lamb, it), oracle.geodesic2d(img, m, v, lamb, it))
    assert bits_equal(call("fg_signed_generalised_geodesic2d", S, img, m, v, lamb, it),
                      oracle.signed2d(img, m, v, lamb, it))
    assert bits_equal(call("fg_GSF2d", G, img, m, 0.5, v, lamb, 1), oracle.gsf2d(img, m, 0.5, v, lamb, 1))
    assert bits_equal(call("fg_generalised_geodesic2d_toivanen", P, img, m, v, lamb, it),
                      oracle.toivanen2d(img, m, v, lamb, it))
    assert call("fg_generalised_geodesic2d", P, img, m, v, lamb, it, short=True) == _lib.FG_ERR_WORKSPACE


@pytest.mark.parametrize("C,Cm,shape", [(1, 1, (9, 23, 31)), (2, 2, (16, 40, 36)), (6, 1, (12, 20, 24))])
def test_3d_entries(C, Cm, shape):
    img, m = case(C * 10 + Cm + 3, C, shape, Cm)
    v, lamb, it, sp = 1e10, 0.4, 2, (1.5, 0.7, 1.1)
    kw = dict(spacing=sp)
    assert bits_equal(call("fg_generalised_geodesic3d", P, img, m, v, lamb, it, **kw),
                      oracle.geodesic3d(img, m, sp, v, lamb, it))
    assert bits_equal(call("fg_signed_generalised_geodesic3d", S, img, m, v, lamb, it, **kw),
                      oracle.signed3d(img, m, sp, v, lamb, it))
    assert bits_equal(call("fg_GSF3d", G, img, m, 0.3, v, lamb, 1, **kw), oracle.gsf3d(img, m, 0.3, sp, v, lamb, 1))
    assert bits_equal(call("fg_generalised_geodesic3d_toivanen", P, img, m, v, lamb, it, **kw),
                      oracle.toivanen3d(img, m, sp, v, lamb, it))
    assert call("fg_signed_generalised_geodesic3d", S, img, m, v, lamb, it, short=True, **kw) == _lib.FG_ERR_WORKSPACE
