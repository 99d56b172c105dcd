"""The Green's-function sampler of the tensor-core far fill (TcGreen in
csrc/far_fill_tc.cu), replayed on the CPU in NumPy FP32 arithmetic (a fused
multiply-add rounds the exact product-sum once), against FP64 exp(-jkR)/R.

The sampler carries R^2, R, 1/R and k R as double-float words, reduces k R by
a three-word 2 pi, and takes sin / cos by Tang's table-driven method with
sin, cos (j pi/128) as double-float table words; each part of g comes out as an
unnormalised pair hi + lo.  Its error must stay near 1e-9 of |g|, far below an
FP32 sample (the floor of the FP32 fill), including for phases k R of
thousands of radians and an rsqrt seed that is off by several ulp.
"""
import os
import re

import numpy as np

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "20260722_ghost_gb300", "csrc")
f32 = np.float32
f64 = np.float64


def _consts(fname, prefix):
    txt = open(os.path.join(CSRC, fname)).read()
    out = {}
    for name, expr in re.findall(r"constexpr float (" + prefix + r"\w+)\s*=\s*([^;]+);", txt):
        expr = expr.strip()
        m = re.fullmatch(r"([0-9.e+-]+)f\s*/\s*([0-9.e+-]+)f", expr)
        if m:
            out[name] = f32(float(m.group(1)) / float(m.group(2)))
        elif expr.startswith("(float)"):
            continue
        else:
            out[name] = f32(float(expr.rstrip("f")))
    return out


S = _consts("samplers.cuh", "k")
D = _consts("df_math.cuh", "kDf")
# kTwoPiC and kInvTwoPi are FP32 roundings of FP64 expressions in samplers.cuh
TWO_PI = 6.283185307179586476925286766559
S["kTwoPiC"] = f32(TWO_PI - 6.28125 - 4059.0 / 2097152.0)
S["kInvTwoPi"] = f32(1.0 / TWO_PI)


def fma(a, b, c):
    return (f64(a) * f64(b) + f64(c)).astype(f32)


def split(x):
    h = np.asarray(x).astype(f32)
    return h, (np.asarray(x) - f64(h)).astype(f32)


TAB = np.array([[*split(np.sin(np.pi * (i - 128) / 128)), *split(np.cos(np.pi * (i - 128) / 128))]
                for i in range(257)], dtype=f32)


def tc_green(d2, a2, k, s2, seed_ulps=0):
    """NumPy FP32 replay of TcGreen::pair (each lane of its f32x2 steps); returns
    the (hi, lo) FP32 words of re and im (the kernel carries +y sin for the
    imaginary part and negates its digit scale instead)."""
    d2h, d2l = split(d2)
    a2h, a2l = split(a2)
    kh, kl = split(np.full_like(np.asarray(d2, f64), k))
    s2h, s2l = split(s2)
    p = (a2h * s2h).astype(f32)
    pe = fma(a2h, s2h, -p)
    t = (d2h + p).astype(f32)
    bb = (t - d2h).astype(f32)
    te = ((d2h - (t - bb)) + (p - bb)).astype(f32)
    lo = (((te + pe).astype(f32) + fma(a2h, s2l, (a2l * s2h).astype(f32))).astype(f32) + d2l).astype(f32)
    R2 = (t + lo).astype(f32)
    R2l = (lo - (R2 - t)).astype(f32)
    y = (1.0 / np.sqrt(f64(R2))).astype(f32)
    if seed_ulps:
        y = (y * (1 + seed_ulps * 2.0 ** -23)).astype(f32)
    r = (R2 * y).astype(f32)
    rl = (f32(0.5) * (fma(-r, r, R2) + R2l).astype(f32) * y).astype(f32)
    eps = (fma(-r, y, f32(1.0)) - (rl * y).astype(f32)).astype(f32)
    ph = (kh * r).astype(f32)
    phl = (fma(kh, r, -ph) + fma(kh, rl, (kl * r).astype(f32))).astype(f32)
    q = np.rint((ph * S["kInvTwoPi"]).astype(f32)).astype(f32)
    t1 = fma(-q, S["kTwoPiA"], ph)
    qb = (-q * S["kTwoPiB"]).astype(f32)
    t2 = (t1 + qb).astype(f32)
    tb = (t2 - t1).astype(f32)
    t2e = ((t1 - (t2 - tb)) + (qb - tb)).astype(f32)
    dt = (fma(-q, S["kTwoPiC"], phl) + t2e).astype(f32)
    jf = np.clip(np.rint((t2 * D["kDf128ByPi"]).astype(f32)), -128, 128).astype(f32)
    r0 = fma(-jf, D["kDfPiB128_1"], t2)
    rv = fma(-jf, D["kDfPiB128_2"], (r0 + dt).astype(f32))
    r2 = (rv * rv).astype(f32)
    sr = fma((rv * r2).astype(f32), f32(-1.0 / 6.0), rv)
    c1 = (r2 * fma(r2, f32(1.0 / 24.0), f32(-0.5))).astype(f32)
    T = TAB[jf.astype(int) + 128]
    sh, sl, ch, cl = T[..., 0], T[..., 1], T[..., 2], T[..., 3]
    s_lo = (fma(ch, sr, fma(sh, c1, sl)) + (cl * sr).astype(f32)).astype(f32)
    c_lo = (fma(-sh, sr, fma(ch, c1, cl)) - (sl * sr).astype(f32)).astype(f32)
    yl = (y * eps).astype(f32)
    ya = (y + yl).astype(f32)
    gr = (y * ch).astype(f32)
    grl = (fma(y, ch, -gr) + fma(ya, c_lo, (yl * ch).astype(f32))).astype(f32)
    gi = (y * sh).astype(f32)
    gil = (fma(y, sh, -gi) + fma(ya, s_lo, (yl * sh).astype(f32))).astype(f32)
    return (gr, grl), (-gi, -gil)


def test_tc_green_matches_fp64():
    rng = np.random.default_rng(11)
    n = 200000
    rho = rng.uniform(0.0, 2.0, (2, n))
    dz = rng.uniform(-3.0, 3.0, n)
    d2 = (rho[0] - rho[1]) ** 2 + dz ** 2
    keep = d2 > 1e-6
    rho, d2 = rho[:, keep], d2[keep]
    a2 = 4.0 * rho[0] * rho[1]
    s2 = np.sin(0.5 * rng.uniform(0.0, np.pi, len(d2))) ** 2
    R = np.sqrt(d2 + a2 * s2)
    for k, ulps in ((1.0, 0), (80.0, 0), (200.0, 3), (900.0, -3)):
        (rh, rl), (ih, il) = tc_green(d2, a2, k, s2, seed_ulps=ulps)
        re, im = f64(rh) + f64(rl), f64(ih) + f64(il)
        want = np.exp(-1j * k * R) / R
        err = np.abs((re + 1j * im) - want) / np.abs(want)
        assert np.max(err) < 5e-9, (k, float(np.max(err)))
        # an FP32 sample: ~1e-7 at most, ~3e-8 typically
        fp32 = np.abs(want.real.astype(f32) + 1j * want.imag.astype(f32) - want) / np.abs(want)
        assert np.max(err) < np.max(fp32) / 10
        assert np.median(err) < np.median(fp32) / 40
