"""Batched 3D transforms: argument checks and the plans a batch pins (CPU)."""
import pytest
import torch

import fastgeodis_gb300 as fg
from fastgeodis_gb300 import _lib, batch3d


def test_argument_checks():
    a = torch.zeros(1, 1, 4, 5, 6)
    m = torch.ones(1, 1, 4, 5, 6)
    with pytest.raises(ValueError):
        fg.generalised_geodesic3d_batch([a], [m, m], (1, 1, 1), 1e10, 0.5)
    with pytest.raises(ValueError):
        fg.generalised_geodesic3d_batch([a[0]], [m[0]], (1, 1, 1), 1e10, 0.5)  # not 5D
    with pytest.raises(ValueError):
        fg.generalised_geodesic3d_batch([a], [torch.ones(1, 1, 4, 5, 7)], (1, 1, 1), 1e10, 0.5)
    with pytest.raises(ValueError):
        fg.generalised_geodesic3d_batch([a], [m], (1, 1, 1), 1e10, 0.5)  # host tensors
    assert fg.generalised_geodesic3d_batch([], [], (1, 1, 1), 1e10, 0.5) == []


@pytest.mark.parametrize("key", [(2, 256, 256), (2, 128, 256), (2, 64, 64), (2, 40, 72), (2, 100, 300), (2, 20, 27),
                                 (2, 512, 512)])
@pytest.mark.parametrize("C", [1, 3])
def test_batch_plans_fit(key, C):
    p = batch3d.batch_plan_for(key, C)
    cross, N1, N2 = key
    runs = N1 * -(-N2 // 4)
    if p is None:
        # no cluster holds it: even 16 strips need more threads than a CTA has
        assert -(-N1 // 16) * -(-N2 // 4) > (1024 if C == 1 else 512)
        return
    S, T1, T2, flags = p
    if flags & _lib.FG_PLAN_CLUSTER:
        rpt = 2 if flags & _lib.FG_PLAN_RUNS2 else 1
        g = -(-N1 // T1)
        assert 2 <= g <= 16 and T2 == N2 and T1 % rpt == 0
        assert T1 // rpt * -(-N2 // 4) <= (1024 if rpt == 1 and C == 1 else 512)
        if rpt == 2:
            assert C == 1
    else:
        assert (T1, T2) == (N1, N2) and runs <= (1024 if C == 1 else 512)
    _lib.check(_lib.load().fg_plan_override(*key, *p))  # a valid override
    _lib.check(_lib.load().fg_plan_override(*key, 0, 0, 0, 0))


def _items(shapes, lambs, signed=False, C=1):
    import ctypes

    from fastgeodis_gb300 import batch3d

    arr = (batch3d._Item3d * len(shapes))()
    base = 1 << 20
    for k, (s, lamb) in enumerate(zip(shapes, lambs)):
        it = arr[k]
        for nm in ("image", "mask", "out", "image_t", "t1", "d2", "t2"):
            setattr(it, nm, base)  # placeholders: planning only records the addresses
            base += 1 << 24
        it.C, (it.D, it.H, it.W) = C, s
        it.flags = 1 if signed else 0
        it.v, it.l_grad, it.l_eucl = 1e10, lamb, 1.0 - lamb
        for j in range(3):
            it.spacing[j] = 1.0
    return arr


def _plan(shapes, lambs, signed=False, C=1, G=16, iterations=4):
    import ctypes

    from fastgeodis_gb300 import _lib

    L = _lib.load()
    info = (ctypes.c_int * 5)()
    buf = (ctypes.c_ubyte * (len(shapes) * (2 + 10 * iterations) * L.fg_batch3d_job_bytes()))()
    rc = L.fg_batch3d_plan(_items(shapes, lambs, signed, C), len(shapes), iterations, G, None, buf, len(buf), info)
    return rc, list(info)


def test_one_launch_plan_jobs_and_shape():
    """The one-launch batch's job list (built on the host, no GPU): a prologue,
    every pass, a transpose of each map after the pass that hands over to the
    passes along W and after the last of those, and (signed) an epilogue per
    volume; the launch's arithmetic mode is the shared one or the general
    expression; refusals."""
    from fastgeodis_gb300 import _lib

    rc, info = _plan([(20, 33, 27), (7, 18, 40)], [0.5, 0.0])
    assert rc == 0 and info[0] == 2 * (1 + 24 + 2 * 4) and info[3] == 1 and info[4] == 0
    rc, info = _plan([(8, 8, 8)], [1.0], signed=True, G=4)
    assert rc == 0 and info[0] == 1 + 24 + 4 * 4 + 1 and info[3] == 2 and info[4] == 2
    rc, info = _plan([(16, 16, 16)] * 3, [0.0] * 3)
    assert rc == 0 and info[4] == 1 and info[1] <= 512 and info[2] <= 227 * 1024
    rc, info = _plan([(1, 9, 13)], [0.5], iterations=2)  # D = 1: the passes along D move no data
    assert rc == 0 and info[0] == 1 + 2 * (4 + 2)
    assert _plan([(8, 8, 8)], [0.5], C=2)[0] == _lib.FG_ERR_UNSUPPORTED  # one image channel read
    assert _plan([(8, 8, 8)], [0.0], C=3)[0] == 0                        # ... unless lamb = 0
    assert _plan([(64, 256, 256)], [0.5], G=2)[0] == _lib.FG_ERR_UNSUPPORTED  # section too large for 2 CTAs
    rc, info = _plan([(8, 8, 8)] * 2, [0.5, 0.5], G=16, iterations=1)
    assert rc == 0


def test_launch_order_keeps_each_slot_shape():
    """The launch order (costliest arithmetic first among equal shapes) puts
    a volume of the same shape at every slot position as the order the slots'
    workspaces were sized in, whatever the weights; the costliest mode leads
    its shape group."""
    import numpy as np

    from fastgeodis_gb300.batch3d import launch_order, slot_order, transform_cost

    rng = np.random.default_rng(5)
    pool = [(1, 16, 32, 64), (1, 64, 32, 16), (1, 32, 32, 32), (3, 16, 32, 64), (1, 8, 8, 8)]
    for _ in range(50):
        shapes = [pool[int(k)] for k in rng.integers(0, len(pool), 9)]
        lambs = [float(x) for x in rng.choice([0.0, 0.3, 0.5, 1.0], 9)]
        a, b = slot_order(shapes), launch_order(shapes, lambs)
        assert sorted(b) == list(range(9))
        assert [shapes[i] for i in a] == [shapes[i] for i in b]
        for k in range(8):
            if shapes[b[k]] == shapes[b[k + 1]]:
                assert transform_cost(shapes[b[k]], lambs[b[k]]) >= transform_cost(shapes[b[k + 1]], lambs[b[k + 1]])


def test_general_mode_batch_plans():
    """Passes of the general arithmetic take the cluster plan's strips with
    one run per thread where the batch plan runs the two-run sweep kernel
    (one image channel, at most 1024 threads per CTA)."""
    from fastgeodis_gb300 import _lib
    from fastgeodis_gb300.batch3d import batch_general_plan_for, batch_plan_for

    for key in [(2, 256, 256), (2, 128, 256), (2, 200, 300), (2, 64, 64), (2, 40, 600)]:
        c, g = batch_plan_for(key), batch_general_plan_for(key)
        if c is None or not c[3] & _lib.FG_PLAN_RUNS2:
            assert g is None
            continue
        if g is None:
            continue
        assert g[:3] == c[:3] and g[3] & _lib.FG_PLAN_CLUSTER and not g[3] & _lib.FG_PLAN_RUNS2
        threads = g[1] * -(-key[2] // 4)
        assert threads <= 1024 and bool(g[3] & _lib.FG_PLAN_LEAN) == (threads > 512)
        assert batch_general_plan_for(key, channels=3) is None
    assert batch_general_plan_for((2, 256, 256)) == (8, 16, 256, _lib.FG_PLAN_CLUSTER | _lib.FG_PLAN_LEAN)
