"""Differentiable 2D transform: forward bit-identical to the plain path, and
gradients against (a) a plain PyTorch float32 autograd implementation of the
same raster scan, (b) float64 central finite differences of the scan."""
import math

import numpy as np
import pytest
import torch

import fastgeodis_gb300 as fg
from oracle import oracle

pytestmark = pytest.mark.gpu


def torch_scan(image, mask, v, lamb, iters):
    """The reference's raster scan written with PyTorch float32 ops (autograd
    through torch.min); FastGeodis/fastgeodis_cpu.cpp:53-201.  Candidate order
    (own value first, then x-1, x, x+1) matches the engine's tie rule."""
    C, H, W = image.shape[1], image.shape[2], image.shape[3]
    lg = torch.tensor(float(np.float32(lamb)))
    le = torch.tensor(float(np.float32(1.0 - lamb)))
    r2 = torch.tensor(float(np.float32(math.sqrt(2.0))))
    ld = [r2, torch.tensor(1.0), r2]
    D = v * mask[0, 0]
    I = image[0]
    inf = torch.tensor(float("inf"))

    def sweep(D, I, forward):
        L = D.shape[0]
        rows = [D[t] for t in range(L)]
        order = range(1, L) if forward else range(L - 2, -1, -1)
        for t in order:
            tp = t - 1 if forward else t + 1
            prev, cur = rows[tp], rows[t]
            cands = [cur]
            for k in (-1, 0, 1):
                n = cur.shape[0]
                idx = torch.arange(n) + k
                ok = (idx >= 0) & (idx < n)
                idc = idx.clamp(0, n - 1)
                l1 = torch.zeros(n)
                for c in range(I.shape[0]):
                    l1 = l1 + (I[c, t] - I[c, tp][idc]).abs()
                cand = (prev[idc] + le * ld[k + 1]) + lg * l1
                cands.append(torch.where(ok, cand, inf))
            rows[t] = torch.stack(cands).min(dim=0).values
        return torch.stack(rows)

    for _ in range(iters):
        D = sweep(D, I, True)
        D = sweep(D, I, False)
        Dt, It = D.t(), I.transpose(1, 2)
        Dt = sweep(Dt, It, True)
        Dt = sweep(Dt, It, False)
        D = Dt.t()
    return D


@pytest.mark.parametrize("C", [1, 3])
def test_forward_bits_and_gradients_vs_torch(C):
    torch.manual_seed(4)
    B, H, W = 2, 11, 14
    img = (torch.rand(B, C, H, W) * 10).cuda().requires_grad_(True)
    msk = torch.sigmoid(torch.randn(B, 1, H, W) * 2).cuda().requires_grad_(True)
    v, lamb, it = 3.0, 0.6, 2
    d = fg.generalised_geodesic2d_differentiable(img, msk, v, lamb, it)
    for b in range(B):
        ref = fg.generalised_geodesic2d(img[b:b + 1].detach(), msk[b:b + 1].detach(), v, lamb, it)
        assert torch.equal(d[b:b + 1].detach().view(torch.int32), ref.view(torch.int32))
    w = torch.rand(B, 1, H, W).cuda()
    (d * w).sum().backward()
    for b in range(B):
        ib = img[b:b + 1].detach().cpu().requires_grad_(True)
        mb = msk[b:b + 1].detach().cpu().requires_grad_(True)
        db = torch_scan(ib, mb, v, lamb, it)
        assert torch.equal(db.detach(), d[b, 0].detach().cpu())
        (db * w[b, 0].cpu()).sum().backward()
        torch.testing.assert_close(img.grad[b].cpu(), ib.grad[0], rtol=1e-5, atol=1e-5)
        torch.testing.assert_close(msk.grad[b].cpu(), mb.grad[0], rtol=1e-5, atol=1e-5)


def test_gradients_vs_float64_finite_differences():
    rng = np.random.default_rng(7)
    H, W = 40, 52
    img = (rng.random((1, 1, H, W)) * 20).astype(np.float32)
    msk = (1.0 / (1.0 + np.exp(-rng.normal(0, 2, (1, 1, H, W))))).astype(np.float32)
    v, lamb, it, eps = 5.0, 0.75, 2, 1e-3
    w = rng.random((H, W))
    ti = torch.from_numpy(img).cuda().requires_grad_(True)
    tm = torch.from_numpy(msk).cuda().requires_grad_(True)
    (fg.generalised_geodesic2d_differentiable(ti, tm, v, lamb, it)[0, 0] * torch.from_numpy(w).float().cuda()).sum().backward()
    gi, gm = ti.grad[0, 0].cpu().numpy(), tm.grad[0, 0].cpu().numpy()

    def loss(im, m):
        return float((oracle.geodesic2d_f64(im[0], m[0], v, lamb, it)[0] * w).sum())

    ok_i = ok_m = 0
    pts = [(int(rng.integers(0, H)), int(rng.integers(0, W))) for _ in range(16)]
    for (y, x) in pts:
        for arr, g, tag in ((img, gi, "i"), (msk, gm, "m")):
            a64 = arr.astype(np.float64)
            p, q = a64.copy(), a64.copy()
            p[0, 0, y, x] += eps
            q[0, 0, y, x] -= eps
            fd = (loss(p if tag == "i" else img.astype(np.float64), p if tag == "m" else msk.astype(np.float64))
                  - loss(q if tag == "i" else img.astype(np.float64), q if tag == "m" else msk.astype(np.float64))) / (2 * eps)
            good = abs(fd - g[y, x]) <= 1e-2 * max(1.0, abs(fd))
            if tag == "i":
                ok_i += good
            else:
                ok_m += good
    # the derivative is piecewise constant; a sample may sit within eps of a
    # change of optimal path, so most (not all) samples must agree
    assert ok_i >= 14 and ok_m >= 14, (ok_i, ok_m)


@pytest.mark.parametrize("iters,C,shape", [(1, 1, (40, 33)), (2, 1, (64, 64)), (3, 3, (37, 52))])
def test_recompute_mode_gives_the_same_bits(iters, C, shape):
    # one pass's tape plus recomputation instead of every pass's tape
    g = torch.Generator().manual_seed(11 + iters)
    B = 3
    img = (torch.rand((B, C) + shape, generator=g) * 255).cuda()
    msk = torch.sigmoid(torch.randn((B, 1) + shape, generator=g)).cuda()
    w = torch.rand((B, 1) + shape, generator=g).cuda()
    res = []
    for rec in (False, True):
        a = img.clone().requires_grad_(True)
        m = msk.clone().requires_grad_(True)
        d = fg.generalised_geodesic2d_differentiable(a, m, 10.0, 0.75, iters, recompute=rec)
        (d * w).sum().backward()
        res.append((d.detach(), a.grad, m.grad))
    for x, y in zip(res[0], res[1]):
        assert torch.equal(x.view(torch.int32), y.view(torch.int32))
    fg.check_status()


def test_wide_multichannel_images_use_the_register_adjoint():
    # 1400-wide rows with three channels: the staged adjoint's ring does not
    # fit shared memory, so the backward takes the register-prefetch path
    torch.manual_seed(9)
    B, C, H, W = 2, 3, 6, 1400
    img = (torch.rand(B, C, H, W) * 10).cuda().requires_grad_(True)
    msk = torch.sigmoid(torch.randn(B, 1, H, W) * 2).cuda().requires_grad_(True)
    v, lamb, it = 3.0, 0.6, 1
    d = fg.generalised_geodesic2d_differentiable(img, msk, v, lamb, it)
    w = torch.rand(B, 1, H, W).cuda()
    (d * w).sum().backward()
    for b in range(B):
        ib = img[b:b + 1].detach().cpu().requires_grad_(True)
        mb = msk[b:b + 1].detach().cpu().requires_grad_(True)
        db = torch_scan(ib, mb, v, lamb, it)
        assert torch.equal(db.detach(), d[b, 0].detach().cpu())
        (db * w[b, 0].cpu()).sum().backward()
        torch.testing.assert_close(img.grad[b].cpu(), ib.grad[0], rtol=1e-5, atol=1e-5)
        torch.testing.assert_close(msk.grad[b].cpu(), mb.grad[0], rtol=1e-5, atol=1e-5)
    fg.check_status()
