"""The FP64 arithmetic the pair passes form on the integer pipes (exact
position differences from fixed-point copies, correctly rounded square root,
reciprocal and 2/y) against the IEEE operations, bit for bit.

Tolerance: none -- every result must equal numpy's (IEEE, round to nearest
even) in all 64 bits, NaNs compared as NaN."""
import numpy as np
import pytest

import sphgpu

pytestmark = pytest.mark.gpu


def same(got, want):
    g, w = np.asarray(got), np.asarray(want)
    eq = g.view(np.uint64) == w.view(np.uint64)
    return eq | (np.isnan(g) & np.isnan(w))


def positive_doubles(rng, n, e_lo=1, e_hi=2046):
    e = rng.integers(e_lo, e_hi + 1, n).astype(np.uint64)
    m = rng.integers(0, 2 ** 52, n, dtype=np.uint64)
    return ((e << np.uint64(52)) | m).view(np.float64)


def specials():
    tiny = np.finfo(np.float64).tiny
    vals = [0.0, -0.0, 5e-324, 1e-310, tiny, np.nextafter(tiny, 1.0), 1.0, 2.0, 4.0, 0.5,
            np.finfo(np.float64).max, np.inf, -np.inf, np.nan, -1.0, -2.5, 3.0, 1e300, 1e-300,
            2.0 ** 1021, 2.0 ** 1022, 2.0 ** 1023, 2.0 ** -1021, 2.0 ** -1022]
    return np.array(vals, dtype=np.float64)


def test_sqrt_reciprocal_match_ieee(gpu):
    rng = np.random.default_rng(11)
    parts = [positive_doubles(rng, 3_000_000),
             positive_doubles(rng, 1_000_000, 1000, 1050),  # around 1
             specials()]
    # exact squares and their neighbours (rounding boundaries)
    r = rng.uniform(0.5, 2.0, 500_000)
    sq = r * r
    parts += [sq, np.nextafter(sq, 0.0), np.nextafter(sq, 4.0)]
    k = rng.integers(1, 2 ** 26, 500_000).astype(np.float64)
    parts.append(k * k)
    # the values the passes see: r^2 ~ 1e-5..1e-3, r r + eta2, rho_p + rho_q ~ 2000
    parts.append(rng.uniform(1e-6, 1.5e-3, 500_000))
    parts.append(rng.uniform(1800.0, 2200.0, 500_000))
    x = np.concatenate(parts)
    with np.errstate(all="ignore"):
        refs = {"sqrt": np.sqrt(x), "rcp": 1.0 / x, "two_over": 2.0 / x}
    for op, want in refs.items():
        got = sphgpu.arith_check(op, x)
        ok = same(got, want)
        assert ok.all(), (op, x[~ok][:5], got[~ok][:5], want[~ok][:5])


@pytest.mark.parametrize("k", [59, 58, 55, 62])
def test_fixed_point_difference_matches_ieee(gpu, k):
    rng = np.random.default_rng(k)
    lim = 2.0 ** (62 - k)
    n = 1_000_000
    a = rng.uniform(-lim, lim, n)
    parts_a = [a, rng.uniform(-0.05, 0.05, n), rng.uniform(0.0, 4.0, n), specials()]
    parts_b = [a + rng.uniform(-0.07, 0.07, n), rng.uniform(-0.05, 0.05, n),
               None, specials()[::-1].copy()]
    c = parts_a[2]
    parts_b[2] = np.nextafter(c, np.where(rng.random(n) < 0.5, -1.0, 5.0))
    a = np.concatenate(parts_a)
    b = np.concatenate(parts_b)
    got = sphgpu.arith_check("sub", a, b, k=k)
    with np.errstate(all="ignore"):
        want = a - b
    ok = same(got, want)
    assert ok.all(), (a[~ok][:5], b[~ok][:5], got[~ok][:5], want[~ok][:5])
