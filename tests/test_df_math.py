"""Double-float elementary functions of the near fill (csrc/df_math.cuh), checked
on the CPU: the split constants are read from the header and the algorithms are
replayed in NumPy FP32 arithmetic (a fused multiply-add is emulated by rounding
the exact double product-sum once to FP32), against FP64 / exact references."""
import os
import re
from fractions import Fraction

import numpy as np

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "20260722_ghost_gb300", "csrc", "df_math.cuh")
# 2 pi, pi / 128 and ln 2 / 32 to 40 digits
PI = Fraction("3.141592653589793238462643383279502884197")
LN2 = Fraction("0.6931471805599453094172321214581765680755")

f32 = np.float32


def consts():
    txt = open(HDR).read()
    out = {}
    for name, expr in re.findall(r"constexpr float (kDf\w+)\s*=\s*([^;]+);", txt):
        expr = expr.strip()
        m = re.fullmatch(r"([0-9.e+-]+)f\s*/\s*([0-9.e+-]+)f", expr)
        out[name] = f32(float(m.group(1)) / float(m.group(2))) if m else f32(float(expr.rstrip("f")))
    return out


C = consts()


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def fast(h, l):
    s = f32(h + l)
    return s, f32(l - f32(s - h))


def df_from(x):
    h = f32(x)
    return h, f32(x - np.float64(h))


def df_mul(a, b):
    p = f32(a[0] * b[0])
    e = f32(fma(a[0], b[0], -p) + fma(a[0], b[1], f32(a[1] * b[0])))
    h = f32(p + e)
    return h, f32(e - f32(h - p))


def df_add(a, b):
    s = f32(a[0] + b[0])
    bb = f32(s - a[0])
    e = f32(f32(f32(f32(a[0] - f32(s - bb)) + f32(b[0] - bb)) + a[1]) + b[1])
    h = f32(s + e)
    return h, f32(e - f32(h - s))


def value(a):
    return np.float64(a[0]) + np.float64(a[1])


TAB = [(df_from(np.sin(np.pi * (i - 128) / 128)), df_from(np.cos(np.pi * (i - 128) / 128))) for i in range(257)]
ETAB = [df_from(2.0 ** (i / 32)) for i in range(32)]


def df_reduce(ph):
    q = f32(np.rint(f32(ph[0] * C["kDfInvTwoPi"])))
    t1 = fma(-q, C["kDfTwoPiA"], ph[0])
    t2 = fma(-q, C["kDfTwoPiB"], t1)
    pc = f32(q * C["kDfTwoPiC"])
    pce = fma(q, C["kDfTwoPiC"], -pc)
    s = two_sum(t2, -pc)
    h = two_sum(s[0], ph[1])
    return fast(h[0], f32(h[1] + f32(f32(s[1] - pce) - f32(q * C["kDfTwoPiD"]))))


def df_sincos(t):
    j = int(max(-128, min(128, int(np.rint(f32(t[0] * C["kDf128ByPi"]))))))
    jf = f32(j)
    r1 = fma(-jf, C["kDfPiB128_1"], t[0])
    p2 = f32(jf * C["kDfPiB128_2"])
    p2e = fma(jf, C["kDfPiB128_2"], -p2)
    rs = two_sum(r1, -p2)
    r = fast(rs[0], f32(f32(f32(rs[1] - p2e) - f32(jf * C["kDfPiB128_3"])) + t[1]))
    rr = f32(r[0] * r[0])
    rre = f32(fma(r[0], r[0], -rr) + f32(f32(2 * r[0]) * r[1]))
    st = f32(f32(r[0] * rr) * fma(rr, fma(rr, f32(-1 / 5040), f32(1 / 120)), f32(-1 / 6)))
    sr = fast(r[0], f32(r[1] + st))
    c4 = f32(f32(rr * rr) * fma(rr, f32(-1 / 720), f32(1 / 24)))
    ch = two_sum(f32(1), f32(-f32(0.5) * rr))
    cr = fast(ch[0], f32(f32(ch[1] - f32(f32(0.5) * rre)) + c4))
    sT, cT = TAB[j + 128]
    sn = df_add(df_mul(sT, cr), df_mul(cT, sr))
    m2 = df_mul(sT, sr)
    return sn, df_add(df_mul(cT, cr), (-m2[0], -m2[1]))


def df_exp(v):
    kf = f32(np.rint(f32(v[0] * C["kDf32ByLn2"])))
    k = int(kf)
    r1 = fma(-kf, C["kDfLn2By32_1"], v[0])
    p2 = f32(kf * C["kDfLn2By32_2"])
    p2e = fma(kf, C["kDfLn2By32_2"], -p2)
    rs = two_sum(r1, -p2)
    r = fast(rs[0], f32(f32(f32(rs[1] - p2e) - f32(kf * C["kDfLn2By32_3"])) + v[1]))
    rr = f32(r[0] * r[0])
    rre = f32(fma(r[0], r[0], -rr) + f32(f32(2 * r[0]) * r[1]))
    c = f32(r[0] * fma(r[0], fma(r[0], fma(r[0], f32(1 / 720), f32(1 / 120)), f32(1 / 24)), f32(1 / 6)))
    h = two_sum(r[0], f32(f32(0.5) * rr))
    em1r = fast(h[0], f32(f32(f32(h[1] + r[1]) + f32(f32(0.5) * rre)) + f32(rr * c)))
    o = two_sum(f32(1), em1r[0])
    er = fast(o[0], f32(o[1] + em1r[1]))
    if k == 0:
        return er, em1r
    t = df_mul(ETAB[k & 31], er)
    sc = f32(2.0 ** (k >> 5))
    E = (f32(t[0] * sc), f32(t[1] * sc))
    return E, df_add(E, (f32(-1), f32(0)))


def df_rsqrt(x):
    y = f32(1.0 / np.sqrt(np.float64(x[0])) * (1 + 2e-7))   # an rsqrtf-like seed, ~2 ulp off
    y2 = f32(y * y)
    y2e = fma(y, y, -y2)
    p = f32(x[0] * y2)
    pe = fma(x[0], y2, -p)
    e = f32(f32(f32(f32(1) - p) - pe) - f32(f32(x[0] * y2e) + f32(x[1] * y2)))
    return fast(y, f32(f32(f32(0.5) * y) * e))


def test_split_constants_are_exact_enough():
    two_pi = 2 * PI
    s = sum(Fraction(float(C[n])) for n in ("kDfTwoPiA", "kDfTwoPiB", "kDfTwoPiC", "kDfTwoPiD"))
    assert abs(float((s - two_pi) / two_pi)) < 1e-21
    # three words: the last one's FP32 rounding leaves up to 2^-24 |w3| / |sum| ~ 1e-19,
    # far below the ~1e-14 the double-float results carry
    s = sum(Fraction(float(C[n])) for n in ("kDfPiB128_1", "kDfPiB128_2", "kDfPiB128_3"))
    assert abs(float((s - PI / 128) / (PI / 128))) < 1e-19
    s = sum(Fraction(float(C[n])) for n in ("kDfLn2By32_1", "kDfLn2By32_2", "kDfLn2By32_3"))
    assert abs(float((s - LN2 / 32) / (LN2 / 32))) < 1e-19

    def bits(x):
        m = Fraction(float(x))
        while m.denominator != 1:
            m *= 2
        n = abs(m.numerator)
        while n % 2 == 0:
            n //= 2
        return n.bit_length()

    # the leading words are short, so q * word is exact for the reduction counts used
    assert bits(C["kDfTwoPiA"]) <= 8 and bits(C["kDfTwoPiB"]) <= 12
    assert bits(C["kDfPiB128_1"]) <= 15 and bits(C["kDfLn2By32_1"]) <= 13


def test_phase_reduction_and_sincos():
    rng = np.random.default_rng(3)
    err_red = err_sc = 0.0
    for _ in range(3000):
        ph = df_from(rng.uniform(0.0, 1200.0))
        t = df_reduce(ph)
        pv = Fraction(float(ph[0])) + Fraction(float(ph[1]))
        q = round(float(pv / (2 * PI)))
        err_red = max(err_red, abs(value(t) - float(pv - q * 2 * PI)))
        sn, cs = df_sincos(t)
        tv = value(t)
        err_sc = max(err_sc, abs(value(sn) - np.sin(tv)), abs(value(cs) - np.cos(tv)))
    assert err_red < 1e-13, err_red
    assert err_sc < 2e-13, err_sc


def test_exp_and_rsqrt():
    rng = np.random.default_rng(4)
    err_e = err_em1 = err_r = 0.0
    for _ in range(3000):
        v = df_from(float(np.exp(rng.uniform(np.log(1e-5), np.log(4.0)))))
        E, Em1 = df_exp(v)
        vv = value(v)
        err_e = max(err_e, abs(value(E) / np.exp(vv) - 1))
        err_em1 = max(err_em1, abs(value(Em1) / np.expm1(vv) - 1))
        x = df_from(rng.uniform(1e-8, 10.0) ** 2)
        err_r = max(err_r, abs(value(df_rsqrt(x)) * np.sqrt(value(x)) - 1))
    assert err_e < 2e-13, err_e
    assert err_em1 < 1e-11, err_em1           # e^v - 1 loses bits only for v just above ln2/64
    assert err_r < 2e-13, err_r               # one Newton step from a ~2-ulp seed: 1.5 e^2
