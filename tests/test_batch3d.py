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
