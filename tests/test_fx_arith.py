"""The offset double-float arithmetic of the FP64-accurate collocation kernel
(benchmarks_gb300/csrc/mfgb_bk5fx.cuh: fx_first, fx_fma, fx_finish,
fx_from_double, fx_f2d) restated with numpy float32 operations.

Claims checked:
* with the offset C >= 2 sum |x.hi y.hi|, the two subtractions the
  accumulation relies on are exact: d = T' - T (the rounded product, Dekker's
  Fast2Sum condition |T| >= |product|) and hi = T - C (Sterbenz, since every
  partial T lies in [C/2, 3C/2]);
* the result's error stays near 2^-46 of C;
* the kernel's chain (gradient with |u| < 1, metric with the per-point bound,
  transpose with the line-maximum bound) on whole cells at p = 4 is accurate to
  about 2^-43 relative (the FP64 bar of the operator is 1e-12 ~ 2^-40);
* the per-cell exponent scaling is exact, and the pair keeps 48 bits of every
  value (relative to the cell's largest) whatever the input's binary range.
The reference values are numpy's extended precision (the x86 80-bit format).
"""
import numpy as np
import pytest

f32 = np.float32
EXT = np.longdouble
K = f32(2.0 * (1 + 2.0 ** -20))

pytestmark = pytest.mark.skipif(np.finfo(np.longdouble).nmant < 60,
                                reason="needs an extended long double")


def fma(a, b, c):
    """float32 fma: the product is exact in extended precision, then one
    rounding to float32 (after an extended rounding of the sum, immaterial here)."""
    return (np.asarray(a, EXT) * np.asarray(b, EXT) + np.asarray(c, EXT)).astype(f32)


def split(x):
    hi = np.asarray(x, np.float64).astype(f32)
    return hi, (np.asarray(x, np.float64) - hi.astype(np.float64)).astype(f32)


class Acc:
    """fxacc: value = (T - C) + S"""

    def __init__(self, C):
        self.C = np.asarray(C, f32)
        self.T = None
        self.S = None
        self.exact_ok = True

    def add(self, x, y):
        xh, xl = x
        yh, yl = y
        T = self.C if self.T is None else self.T
        t = fma(xh, yh, T)
        d = (t - T).astype(f32)
        self.exact_ok &= bool(np.all(d.astype(EXT) == t.astype(EXT) - T.astype(EXT)))
        r = fma(xh, yh, -d)
        e = fma(xl, yh, fma(xh, yl, r))
        self.S = e if self.S is None else (self.S + e).astype(f32)
        self.T = t

    def finish(self):
        hi = (self.T - self.C).astype(f32)
        self.exact_ok &= bool(np.all(hi.astype(EXT) == self.T.astype(EXT) - self.C.astype(EXT)))
        return hi, self.S


def ext(v):
    return v[0].astype(EXT) + v[1].astype(EXT)


@pytest.mark.parametrize("terms", [3, 5, 9, 15, 27])
def test_offset_dot_exact_steps_and_error(terms):
    rng = np.random.default_rng(terms)
    n = 4000
    xs = [split(rng.uniform(-1, 1, n) * 10.0 ** rng.integers(-4, 3, n)) for _ in range(terms)]
    ys = [split(rng.uniform(-1, 1, n)) for _ in range(terms)]
    B = sum(np.abs(x[0]).astype(np.float64) * np.abs(y[0]) for x, y in zip(xs, ys)).astype(f32)
    C = (K * B).astype(f32)
    a = Acc(C)
    for x, y in zip(xs, ys):
        a.add(x, y)
    got = ext(a.finish())
    exact = sum(ext(x) * ext(y) for x, y in zip(xs, ys))
    assert a.exact_ok
    err = np.abs(got - exact) / C.astype(EXT)
    assert float(err.max()) < 2.0 ** -42
    assert float(np.sqrt(np.mean(err ** 2))) < 2.0 ** -45


def fx_from_double(x, off):
    """restatement of fx_from_double by integer operations on the bits"""
    b = np.asarray(x, np.float64).view(np.uint64)
    hw = (b >> np.uint64(32)).astype(np.uint32)
    lw = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    sign = hw & np.uint32(0x80000000)
    e = ((hw >> np.uint32(20)) & np.uint32(0x7FF)).astype(np.int64)
    es = e - off
    hm = ((hw & np.uint32(0xFFFFF)) << np.uint32(3)) | (lw >> np.uint32(29))
    hi_bits = sign | (np.clip(es - 896, 0, 255).astype(np.uint32) << np.uint32(23)) | hm
    hi = np.where(es <= 896, 0, hi_bits).astype(np.uint32).view(f32)
    rem = lw & np.uint32(0x1FFFFFFF)
    fb = rem.astype(f32).view(np.uint32)
    lo_bits = (sign | (fb + ((es - 1075).astype(np.int64) << 23).astype(np.uint32))).astype(np.uint32)
    lo = np.where((rem == 0) | (es < 949), np.uint32(0), lo_bits).view(f32)
    hi = np.where(e == 0x7FF, np.float32(np.nan), hi)
    zero = (e == 0) | (es <= 896)
    return np.where(zero, f32(0), hi), np.where(zero, f32(0), lo)


@pytest.mark.parametrize("scale", [1.0, 2.0 ** -100, 1e-30, 1e30, 2.0 ** 300])
def test_scaled_conversion_keeps_48_bits(scale):
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, 5000) * scale
    emax = int(((np.abs(x).view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).max())
    off = emax - 1022
    hi, lo = fx_from_double(x, off)
    assert np.all(np.abs(hi) < 1)
    back = (hi.astype(EXT) + lo.astype(EXT)) * EXT(2.0) ** off
    rel = np.abs(back - x.astype(EXT)) / np.abs(x).max()
    assert float(rel.max()) < 2.0 ** -47  # hi: 24 bits, lo: the next 29 rounded to 24


@pytest.mark.parametrize("scale", [1.0, 1e-280, 2.0 ** -1000])
def test_zeros_convert_to_zero_in_tiny_cells(scale):
    """A cell whose largest value is below 2^-897 has a scale offset below -896:
    its exact zeros (and double subnormals) must stay zero, not take the offset
    as an exponent."""
    x = np.array([0.0, -0.0, 0.75, -0.5, 5e-324]) * np.array([1, 1, scale, scale, 1])
    emax = int(((np.abs(x).view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).max())
    off = emax - 1022
    hi, lo = fx_from_double(x, off)
    assert hi[0] == 0 and hi[1] == 0 and hi[4] == 0 and lo[4] == 0
    back = (hi[2:4].astype(EXT) + lo[2:4].astype(EXT)) * EXT(2.0) ** off
    assert np.all(np.abs(back - x[2:4].astype(EXT)) <= 2.0 ** -47 * np.abs(x[2:4]))


def gll_derivative(n):
    """GLL points of degree n-1 and the collocation derivative D[i][m] = l_m'(x_i)."""
    from numpy.polynomial import legendre as L
    p = n - 1
    x = np.concatenate([[-1.0], np.sort(np.real(L.legroots(L.legder([0] * p + [1])))), [1.0]])
    D = np.zeros((n, n))
    for m in range(n):
        c = np.zeros(n)
        c[m] = 1.0
        poly = np.polynomial.polynomial.Polynomial.fit(x, c, n - 1)
        D[:, m] = poly.deriv()(x)
    return x, D


def test_cell_chain_at_p4_matches_extended_precision():
    """The kernel's three stages with its bound rules on 200 cells of random data
    and random SPD-like G (per-cell scaled to |G| < 1), against extended
    precision: normwise relative error below 2^-42."""
    n = 5
    _, D = gll_derivative(n)
    rng = np.random.default_rng(3)
    E = 200
    u = rng.uniform(-1, 1, (E, n, n, n))
    u = u / (2.0 ** np.ceil(np.log2(np.abs(u).reshape(E, -1).max(1))))[:, None, None, None] * 0.999
    w = np.array([0.1, 0.54444, 0.71111, 0.54444, 0.1])
    W = w[:, None, None] * w[None, :, None] * w[None, None, :]
    G = np.empty((E, 6, n, n, n))
    for c, scl in enumerate((1, 0.1, 0.1, 1, 0.1, 1)):
        G[:, c] = W * scl * rng.uniform(0.5, 1.0, (E, n, n, n))
    G /= np.abs(G).reshape(E, -1).max(1)[:, None, None, None, None] * 1.001
    Dh = D.astype(f32)
    Dl = (D - Dh).astype(f32)
    cg = (K * np.abs(Dh).astype(np.float64).sum(1)).astype(f32)
    ci = (K * np.abs(Dh).astype(np.float64).sum(0)).astype(f32)
    up = split(u)
    Gp = [split(G[:, c]) for c in range(6)]

    def Dpair(a, b, shape):
        return np.full(shape, Dh[a, b], f32), np.full(shape, Dl[a, b], f32)

    def take(v, ax, m):
        sl = [slice(None)] * 4
        sl[ax] = m
        return v[0][tuple(sl)], v[1][tuple(sl)]

    def put(out, ax, i, val):
        sl = [slice(None)] * 4
        sl[ax] = i
        out[0][tuple(sl)] = val[0]
        out[1][tuple(sl)] = val[1]

    q = []
    for ax in (1, 2, 3):
        out = (np.zeros_like(up[0]), np.zeros_like(up[0]))
        for i in range(n):
            shp = take(up, ax, 0)[0].shape
            a = Acc(np.full(shp, cg[i], f32))
            for m in range(n):
                a.add(Dpair(i, m, shp), take(up, ax, m))
            put(out, ax, i, a.finish())
            assert a.exact_ok
        q.append(out)
    kq = (K * np.maximum(np.maximum(np.abs(q[0][0]), np.abs(q[1][0])), np.abs(q[2][0]))).astype(f32)
    v = []
    for rows in ((0, 1, 2), (1, 3, 4), (2, 4, 5)):
        gs = (np.abs(Gp[rows[0]][0]) + np.abs(Gp[rows[1]][0]) + np.abs(Gp[rows[2]][0])).astype(f32)
        a = Acc((gs * kq).astype(f32))
        for c, d in zip(rows, range(3)):
            a.add(Gp[c], q[d])
        v.append(a.finish())
        assert a.exact_ok
    av = [np.abs(x[0]) for x in v]
    y = np.zeros((E, n, n, n), EXT)
    for i in range(n):
        for j in range(n):
            for k in range(n):
                C = (av[0][:, :, j, k].max(1) * ci[i] + av[1][:, i, :, k].max(1) * ci[j] +
                     av[2][:, i, j, :].max(1) * ci[k]).astype(f32)
                a = Acc(C)
                for m in range(n):
                    a.add(Dpair(m, i, (E,)), (v[0][0][:, m, j, k], v[0][1][:, m, j, k]))
                    a.add(Dpair(m, j, (E,)), (v[1][0][:, i, m, k], v[1][1][:, i, m, k]))
                    a.add(Dpair(m, k, (E,)), (v[2][0][:, i, j, m], v[2][1][:, i, j, m]))
                y[:, i, j, k] = ext(a.finish())
                assert a.exact_ok
    # extended precision from the same (split) inputs
    ue = ext(up)
    De = Dh.astype(EXT) + Dl.astype(EXT)
    g = [ext(x) for x in Gp]
    qr = np.einsum('im,emjk->eijk', De, ue)
    qs = np.einsum('jm,eimk->eijk', De, ue)
    qt = np.einsum('km,eijm->eijk', De, ue)
    vr = g[0] * qr + g[1] * qs + g[2] * qt
    vs = g[1] * qr + g[3] * qs + g[4] * qt
    vt = g[2] * qr + g[4] * qs + g[5] * qt
    ye = (np.einsum('mi,emjk->eijk', De, vr) + np.einsum('mj,eimk->eijk', De, vs) +
          np.einsum('mk,eijm->eijk', De, vt))
    rel = float(np.sqrt(((y - ye) ** 2).sum() / (ye ** 2).sum()))
    assert rel < 2.0 ** -42, np.log2(rel)


def fx_f2d_fast(f, sc):
    """restatement of fx_f2d_fast: float * 2^sc to double by integer operations
    on the high word (cells with |sc| <= 896)"""
    u = np.asarray(f, np.float32).view(np.uint32).astype(np.uint64)
    a = u & np.uint64(0x7FFFFFFF)
    sgn = u & np.uint64(0x80000000)
    hi = ((a >> np.uint64(3)) + np.uint64((896 + sc) << 20)) | sgn
    lo = (u << np.uint64(29)) & np.uint64(0xFFFFFFFF)
    small = a < 0x00800000
    hi = np.where(small, sgn, hi)
    lo = np.where(small, np.uint64(0), lo)
    big = a >= 0x7F800000
    hi = np.where(big, sgn | np.uint64(0x7FF00000) | ((a & np.uint64(0x7FFFFF)) >> np.uint64(3)), hi)
    return ((hi << np.uint64(32)) | lo).view(np.float64)


@pytest.mark.parametrize("sc", [-896, -500, 0, 300, 896])
def test_fast_output_conversion_is_exact(sc):
    rng = np.random.default_rng(0)
    f = (rng.standard_normal(50000) * 10.0 ** rng.integers(-30, 30, 50000)).astype(f32)
    want = np.where(np.abs(f) < np.finfo(f32).tiny, 0.0, f.astype(np.float64) * 2.0 ** sc)
    assert np.array_equal(fx_f2d_fast(f, sc), want)
    special = fx_f2d_fast(np.array([np.inf, -np.inf, np.nan, 0.0, -0.0], f32), sc)
    assert special[0] == np.inf and special[1] == -np.inf and np.isnan(special[2])
    assert special[3] == 0.0 and special[4] == 0.0
