"""CPU tests: the C oracle against the reference's golden vectors, and the
reference's known-answer properties (tests/test_fastgeodis.py of the
reference) on the oracle."""
import math

import numpy as np
import pytest

from golden_cases import bits_equal, load_all, names
from oracle import oracle

CASES = {c["name"]: c for c in load_all()}


def run_oracle(c):
    img, m, v, lamb, it = c["image"], c["mask"], c["v"], c["lamb"], c["iter"]
    op = c["op"]
    if op == "geodesic2d":
        return oracle.geodesic2d(img, m, v, lamb, it)
    if op == "geodesic3d":
        return oracle.geodesic3d(img, m, c["spacing"], v, lamb, it)
    if op == "signed2d":
        return oracle.signed2d(img, m, v, lamb, it)
    if op == "signed3d":
        return oracle.signed3d(img, m, c["spacing"], v, lamb, it)
    if op == "gsf2d":
        return oracle.gsf2d(img, m, c["theta"], v, lamb, it)
    if op == "gsf3d":
        return oracle.gsf3d(img, m, c["theta"], c["spacing"], v, lamb, it)
    if op == "toivanen2d":
        return oracle.toivanen2d(img, m, v, lamb, it)
    if op == "toivanen3d":
        return oracle.toivanen3d(img, m, c["spacing"], v, lamb, it)
    if op == "signed_toivanen2d":
        return oracle.toivanen2d(img, m, v, lamb, it, signed=True)
    if op == "signed_toivanen3d":
        return oracle.toivanen3d(img, m, c["spacing"], v, lamb, it, signed=True)
    if op == "gsf_toivanen2d":
        return oracle.gsf_toivanen2d(img, m, c["theta"], v, lamb, it)
    if op == "gsf_toivanen3d":
        return oracle.gsf_toivanen3d(img, m, c["theta"], c["spacing"], v, lamb, it)
    raise ValueError(op)


def test_golden_set_present():
    assert len(CASES) >= 35
    ops = {c["op"] for c in CASES.values()}
    assert ops == {"geodesic2d", "geodesic3d", "signed2d", "signed3d", "gsf2d", "gsf3d",
                   "toivanen2d", "toivanen3d", "signed_toivanen2d", "signed_toivanen3d",
                   "gsf_toivanen2d", "gsf_toivanen3d"}


@pytest.mark.parametrize("name", names())
def test_oracle_matches_reference_bits(name):
    c = CASES[name]
    got = run_oracle(c)
    assert bits_equal(got, c["expected"]), f"{name}: max abs diff {np.abs(got - c['expected']).max()}"


@pytest.mark.parametrize("threads", [1, 3])
def test_oracle_thread_count_invariant(threads):
    c = CASES["g3d_cube"]
    got = oracle.geodesic3d(c["image"], c["mask"], c["spacing"], c["v"], c["lamb"], c["iter"], nthreads=threads)
    assert bits_equal(got, c["expected"])


@pytest.mark.parametrize("dims,base", [(2, 16), (2, 32), (2, 64), (3, 16), (3, 32)])
def test_oracle_known_answers(dims, base):
    shape = [1] + [base] * dims
    z = np.zeros(shape, np.float32)
    o = np.ones(shape, np.float32)
    sp = [1.0, 1.0, 1.0]
    f = (lambda i, m, v, l, it: oracle.geodesic2d(i, m, v, l, it)) if dims == 2 else \
        (lambda i, m, v, l, it: oracle.geodesic3d(i, m, sp, v, l, it))
    s = (lambda i, m, v, l, it: oracle.signed2d(i, m, v, l, it)) if dims == 2 else \
        (lambda i, m, v, l, it: oracle.signed3d(i, m, sp, v, l, it))
    # reference tests/test_fastgeodis.py:116-160, 326-371
    assert np.all(f(z, z, 1e10, 1.0, 2) == 0)
    assert np.all(f(z, o, 1e10, 1.0, 2) == np.float32(1e10))
    assert np.all(s(z, z, 1e10, 1.0, 2) == np.float32(-1e10))
    assert np.all(s(z, o, 1e10, 1.0, 2) == np.float32(1e10))
    # Euclidean distance from the corner (test_fastgeodis.py:164-210)
    m = o.copy()
    m[(0,) * (dims + 1)] = 0
    d = f(o, m, 1e10, 0.0, 2)
    exp = math.sqrt(dims * base ** 2)
    tol = 10 if dims == 2 else 100
    assert exp - tol < d.max() < exp + tol


def test_oracle_f64_close_to_f32():
    c = CASES["g2d_smooth"]
    d32 = oracle.geodesic2d(c["image"], c["mask"], c["v"], c["lamb"], c["iter"])
    d64 = oracle.geodesic2d_f64(c["image"], c["mask"], c["v"], c["lamb"], c["iter"])
    np.testing.assert_allclose(d32, d64, rtol=1e-5, atol=1e-3)
    c = CASES["g3d_cube"]
    d32 = oracle.geodesic3d(c["image"], c["mask"], c["spacing"], c["v"], c["lamb"], c["iter"])
    d64 = oracle.geodesic3d_f64(c["image"], c["mask"], c["spacing"], c["v"], c["lamb"], c["iter"])
    np.testing.assert_allclose(d32, d64, rtol=1e-5, atol=1e-4)


def test_planted_mistake_is_caught():
    """The bit-level comparison is sharp: a one-ulp change in the oracle's
    output (planted on the CPU) is detected."""
    c = CASES["g2d_c3"]
    got = run_oracle(c).copy()
    flat = got.reshape(-1)
    flat[7] = np.nextafter(flat[7], np.float32(np.inf))
    assert not bits_equal(got, c["expected"])
