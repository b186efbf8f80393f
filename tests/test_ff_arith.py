"""The float-float pair arithmetic of the FP64-state kernels
(utc_gb300/csrc/nb_ff.cuh), restated step by step in numpy float32 and
checked on the CPU against 80-bit long double over many random pairs:
grid splits are exact (coordinates at least 2^-16 of the scale), the pair
vector r is accurate to 2^-47 (exact for close pairs, also far from the
origin), 1/sqrt to 2^-45.5 and the weights m inv^3 to 2^-44.  Each float32 operation rounds to
nearest; an FMA is emulated by one FP64 evaluation rounded once to float32
(the product of two floats is exact in FP64).  The FP32 rsqrt seed is
emulated by a correctly rounded 1/sqrt perturbed by up to 2^-22; the
kernel refines it by one FP32 Newton step before the float-float Halley
step (without that step the Halley correction's roundings, which scale with
the seed's error, leave 2^-44 instead of 2^-46).
"""
import numpy as np
import pytest

F = np.float32
LD = np.longdouble

pytestmark = pytest.mark.skipif(np.finfo(np.longdouble).nmant < 60,
                                reason="needs an extended long double to measure 2^-48 errors")


def fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F)


def two_sum(a, b):
    s = (a + b).astype(F)
    bb = (s - a).astype(F)
    e = ((a - (s - bb).astype(F)).astype(F) + (b - bb).astype(F)).astype(F)
    return s, e


def fast_two_sum(a, b):
    s = (a + b).astype(F)
    return s, (b - (s - a).astype(F)).astype(F)


def split3(x):
    """Grid split of scaled coordinates (|x| < 1): h, m, l on 2^-20, 2^-44,
    2^-68."""
    gh = np.ldexp(np.rint(np.ldexp(x, 20)), -20)
    r1 = x - gh
    gm = np.ldexp(np.rint(np.ldexp(r1, 44)), -44)
    r2 = r1 - gm
    gl = np.ldexp(np.rint(np.ldexp(r2, 68)), -68)
    return gh.astype(F), gm.astype(F), gl.astype(F)


def split_mass(x):
    h = x.astype(F)
    return h, (x - h.astype(np.float64)).astype(F)


def ff_diff(s, p):
    A = (s[0] - p[0]).astype(F)
    B = (s[1] - p[1]).astype(F)
    C = (s[2] - p[2]).astype(F)
    s1, e1 = fast_two_sum(A, B)
    return fast_two_sum(s1, (e1 + C).astype(F))


def pair(xs, xi, ms, eps2, rng):
    """r (3 float-floats) and wj = m_s inv^3 for sources xs, targets xi."""
    r = [ff_diff(split3(xs[:, k]), split3(xi[:, k])) for k in range(3)]
    q = [(rh * rh).astype(F) for rh, _ in r]
    e = [fma(rh, rh, -qq) for (rh, _), qq in zip(r, q)]
    e = [fma((rh + rh).astype(F), rl, ee) for (rh, rl), ee in zip(r, e)]
    eh = F(eps2)
    el = F(eps2 - float(eh))
    S, t1 = two_sum(np.full_like(q[0], eh), q[0])
    S, t2 = two_sum(S, q[1])
    S, t3 = two_sum(S, q[2])
    L = (((el + e[0]).astype(F) + (e[1] + e[2]).astype(F)).astype(F) +
         ((t1 + t2).astype(F) + t3).astype(F)).astype(F)
    Dh, Dl = fast_two_sum(S, L)
    # FP32 rsqrt seed (1/sqrt within 2^-22), one FP32 Newton step
    ya = (1.0 / np.sqrt(Dh.astype(np.float64)) * (1.0 + rng.uniform(-1, 1, Dh.shape) * 2.0 ** -22)).astype(F)
    y0 = fma((ya * F(0.5)).astype(F), fma(-Dh, (ya * ya).astype(F), np.full_like(ya, F(1))), ya)
    qq = (y0 * y0).astype(F)
    qe = fma(y0, y0, -qq)
    t = (Dh * qq).astype(F)
    c = fma(Dh, qq, -t)
    c = fma(Dh, qe, c)
    c = fma(Dl, qq, c)
    u = ((F(1) - t).astype(F) - c).astype(F)
    corr = (y0 * (u * fma(np.full_like(u, F(0.375)), u, np.full_like(u, F(0.5)))).astype(F)).astype(F)
    yh, yl = fast_two_sum(y0, corr)
    p2 = (yh * yh).astype(F)
    e2 = fma(yh, yh, -p2)
    e2 = fma((yh + yh).astype(F), yl, e2)
    p3 = (p2 * yh).astype(F)
    e3 = fma(p2, yh, -p3)
    e3 = fma(p2, yl, e3)
    e3 = fma(e2, yh, e3)
    y3h, y3l = fast_two_sum(p3, e3)
    mh, mm = split_mass(ms)
    wjh = (mh * y3h).astype(F)
    we = fma(mh, y3h, -wjh)
    we = fma(mh, y3l, we)
    wjl = fma(mm, y3h, we)
    return r, (yh, yl), (wjh, wjl)


def value(ff):
    return ff[0].astype(LD) + ff[1].astype(LD)


@pytest.mark.parametrize("center,spread", [(0.0, 1.0), (3.0, 1e-2), (0.7, 1e-4)])
def test_ff_pair_terms_accuracy(center, spread):
    rng = np.random.default_rng(1)
    n = 200000
    xi = center + rng.normal(size=(n, 3)) * 0.5
    xs = xi + rng.normal(size=(n, 3)) * spread
    ms = rng.uniform(0.5, 1.5, n) / 4096
    eps2 = 1e-6
    # scale as the kernel does: largest coordinate and mass into [1/2, 1)
    kx = -np.frexp(np.abs(np.concatenate([xi, xs])).max())[1]
    km = -np.frexp(ms.max())[1]
    xi_s, xs_s, ms_s = np.ldexp(xi, kx), np.ldexp(xs, kx), np.ldexp(ms, km)
    e2_s = float(np.ldexp(eps2, 2 * kx))
    r, y, wj = pair(xs_s, xi_s, ms_s, e2_s, rng)
    rx = [xs_s[:, k].astype(LD) - xi_s[:, k].astype(LD) for k in range(3)]
    d2 = rx[0] ** 2 + rx[1] ** 2 + rx[2] ** 2 + LD(e2_s)
    inv = 1 / np.sqrt(d2)
    for k in range(3):
        err = np.abs(value(r[k]) - rx[k]) / np.maximum(np.abs(rx[k]), LD(1e-300))
        assert float(err.max()) <= 2.0 ** -47
    assert float((np.abs(value(y) - inv) / inv).max()) <= 2.0 ** -45.5
    w = ms_s.astype(LD) * inv ** 3
    assert float((np.abs(value(wj) - w) / w).max()) <= 2.0 ** -44


def test_grid_split():
    """Exact for |x| >= 2^-16 (scaled units), within 2^-69 below; each part
    exactly representable as float32."""
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(-1, 1, 100000) * 2.0 ** -rng.integers(0, 40, 100000),
                        np.array([0.0, 0.5, -0.999999999, 2.0 ** -16, -2.0 ** -30])])
    x = x[np.abs(x) < 1]
    h, m, l = split3(x)
    back = h.astype(np.float64) + m.astype(np.float64) + l.astype(np.float64)
    big = np.abs(x) >= 2.0 ** -16
    assert np.array_equal(back[big], x[big])
    assert np.abs(back - x).max() <= 2.0 ** -69
    gh = np.ldexp(np.rint(np.ldexp(x, 20)), -20)
    assert np.array_equal(h.astype(np.float64), gh)
