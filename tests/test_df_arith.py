"""The double-float accumulation of the operator kernels (benchmarks_gb300/csrc/
mfgb_common.cuh: dfacc_set, dfacc_fma, dfacc_finish, df_to_double) restated
with numpy float32 operations, and its error bound checked on the shapes the
kernels use: dot products of 3 to 15 terms whose results feed further products
unnormalised.  The claim: the error stays at the 2^-48 level of the sum of the
absolute terms, as for the renormalising form it replaced.  The reference is
numpy's extended precision (the x86 80-bit format; exact enough at 2^-64)."""
import numpy as np
import pytest

f32 = np.float32
EXT = np.longdouble


def fma32(a, b, c):
    """fma in float32: a*b is exact in float64 (48-bit product); the sums the
    kernels form this way are an error term (exact in float32) or a low-order
    accumulation, where a second rounding is immaterial."""
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def split(x):
    hi = f32(x)
    return hi, f32(np.float64(x) - np.float64(hi))


def two_sum(a, b):
    s = f32(a + b)
    z = f32(s - a)
    t = f32(f32(a - f32(s - z)) + f32(b - z))
    return s, t


def acc_set(x, y):  # dfacc_set
    s = f32(x[0] * y[0])
    c = fma32(x[0], y[0], -s)
    c = fma32(x[0], y[1], c)
    c = fma32(x[1], y[0], c)
    return [s, c]


def acc_fma(a, x, y):  # dfacc_fma
    p = f32(x[0] * y[0])
    e = fma32(x[0], y[0], -p)
    s, t = two_sum(a[0], p)
    c = f32(a[1] + f32(t + e))
    c = fma32(x[0], y[1], c)
    c = fma32(x[1], y[0], c)
    return [s, c]


def to_ext(v):
    return EXT(v[0]) + EXT(v[1])


def dot(xs, ys):
    a = acc_set(xs[0], ys[0])
    for x, y in zip(xs[1:], ys[1:]):
        a = acc_fma(a, x, y)
    return a  # dfacc_finish: the pair itself


@pytest.mark.skipif(np.finfo(np.longdouble).nmant < 60, reason="needs an extended long double")
@pytest.mark.parametrize("terms", [3, 5, 6, 15])
def test_dot_error_at_the_2_48_level(terms):
    rng = np.random.default_rng(terms)
    worst = 0.0
    for _ in range(400):
        xv = rng.uniform(-1, 1, terms) * 10.0 ** rng.integers(-3, 4, terms)
        yv = rng.uniform(-1, 1, terms)
        xs = [split(v) for v in xv]
        ys = [split(v) for v in yv]
        got = to_ext(dot(xs, ys))
        exact = sum(EXT(x[0]) * EXT(y[0]) + EXT(x[0]) * EXT(y[1]) + EXT(x[1]) * EXT(y[0]) +
                    EXT(x[1]) * EXT(y[1]) for x, y in zip(xs, ys))
        scale = sum(abs(EXT(a) * EXT(b)) for a, b in zip(xv, yv))
        worst = max(worst, float(abs(got - exact) / scale))
    assert worst < 2.0 ** -44, worst


@pytest.mark.skipif(np.finfo(np.longdouble).nmant < 60, reason="needs an extended long double")
def test_unnormalised_results_feed_the_next_contraction():
    """gradient (5 terms) -> metric (3 terms) -> integrate (15 terms), every
    intermediate used as the unnormalised pair, as in the kernels."""
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(200):
        u = [split(v) for v in rng.uniform(-1, 1, 5)]
        D = [split(v) for v in rng.uniform(-3, 3, 5)]
        grad = [dot(D, u) for _ in range(3)]
        G = [split(v) for v in rng.uniform(0.1, 1.0, 3)]
        flux = dot(G, grad)
        Dt = [split(v) for v in rng.uniform(-3, 3, 15)]
        vals = [flux] + [split(v) for v in rng.uniform(-1, 1, 14)]
        y = to_ext(dot(Dt, vals))
        # the same chain in extended precision from the same inputs
        ge = sum(to_ext(d) * to_ext(x) for d, x in zip(D, u))
        fe = sum(to_ext(g) for g in G) * ge
        ye = to_ext(Dt[0]) * fe + sum(to_ext(d) * to_ext(v) for d, v in zip(Dt[1:], vals[1:]))
        scale = abs(to_ext(Dt[0]) * fe) + sum(abs(to_ext(d) * to_ext(v))
                                              for d, v in zip(Dt[1:], vals[1:]))
        worst = max(worst, float(abs(y - ye) / scale))
    assert worst < 2.0 ** -42, worst
