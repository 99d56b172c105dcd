"""Where the FP32 far fill's error comes from (CPU emulation on the oracle).

The far fill of the FP32+IR path samples g = e^{-jkR}/R in FP32 and forms the
orders G_n = sum_j t_jn g_j with an FP32 copy of the DCT table, summing 8-sample
FMA blocks folded in with Kahan compensation (csrc/far_fill.cu); everything
after the transform is double-float.  This test replays that arithmetic on a
small cone-sphere with NumPy FP32 rounding, assembles and solves every mode in
FP64 (oracle), and compares the monostatic far field with the all-FP64 sweep.
It pins the finding that the FP32 rounding of the table, not of the samples or
of the sums, sets the floor: an FP64 table cuts the error ~3x, an exact
transform of the FP32 samples ~10x, and an exact transform on four base-256
digits of each operand as much.  The tensor-core fill (far_fill_tc.cu) goes
further: its samples are FP32 word pairs ~50x more accurate than FP32, split
into four integer digits, with one truncating FP32 accumulator per digit
level, and its far field is ~20x closer to FP64 than an exact transform of
FP32 samples.
"""
import importlib
import math

import numpy as np

from oracle import bor_oracle as O
from test_tc_sampler import tc_green

f32 = np.float32


def _modules():
    geom = importlib.import_module("20260722_ghost_gb300.geometry")
    bodies = importlib.import_module("20260722_ghost_gb300.bodies")
    return geom, bodies


def kahan_dct(gr, gi, table, h):
    """8-sample FMA blocks (one FP32 rounding per product-sum), Kahan fold."""
    shp = gr.shape[:2] + (table.shape[1],)
    out = []
    for g in (gr, gi):
        acc = np.zeros(shp, f32)
        cmp = np.zeros(shp, f32)
        for jb in range(0, h + 1, 8):
            b = np.zeros(shp, f32)
            for j in range(jb, min(jb + 8, h + 1)):
                b = (g[..., j:j + 1].astype(np.float64) * table[j][None, None, :].astype(np.float64) + b).astype(f32)
            y = (b - cmp).astype(f32)
            t = (acc + y).astype(f32)
            cmp = ((t - acc).astype(f32) - y).astype(f32)
            acc = t
        out.append(acc.astype(np.float64) - cmp)
    return out[0] + 1j * out[1]


def _digits(t, nd=4):
    """Balanced base-256 digits of t (exact FP64 arithmetic, integers |d| <= 128)."""
    out = []
    for _ in range(nd):
        d = np.rint(t)
        out.append(d)
        t = (t - d) * 256.0
    return out


def _bf16(x):
    """x rounded to bf16 (8 significant bits, nearest-even)."""
    m, e = np.frexp(x)
    return np.ldexp(np.rint(m * 256.0) / 256.0, e)


def _digits_pair(hi, lo, sc, nd=4):
    """The digit split of far_fill_tc.cu on a pair of FP32 words hi + lo: a
    two-sum normalises hi sc + lo sc, then balanced digits; each digit must be
    an integer |d| <= 128, which bf16 holds exactly (checked)."""
    th = (hi * sc).astype(f32)
    tl = (lo * sc).astype(f32)
    t = (th + tl).astype(f32)
    bb = (t - th).astype(f32)
    te = ((th - (t - bb)).astype(f32) + (tl - bb).astype(f32)).astype(f32)
    d = np.rint(t)
    out = [d.astype(np.float64)]
    t = ((t - d).astype(f32) + te).astype(f32)
    for _ in range(nd - 1):
        t = (t * f32(256.0)).astype(f32)
        d = np.rint(t)
        out.append(d.astype(np.float64))
        t = (t - d).astype(f32)
    for d in out:
        assert np.max(np.abs(d)) <= 128.0
        assert np.array_equal(_bf16(d), d)
    return out


def _add_rz(acc, x):
    """acc + x rounded toward zero to FP32 (a truncating accumulator)."""
    s = acc.astype(np.float64) + x
    r = s.astype(f32)
    over = np.abs(r.astype(np.float64)) > np.abs(s)
    r[over] = np.nextafter(r[over], f32(0))
    return r


# digit products per accumulator: level 0 | 1 | 2 | 3
TC_LEVELS = ([(0, 0)], [(0, 1), (1, 0)], [(0, 2), (1, 1), (2, 0)], [(0, 3), (1, 2), (2, 1), (3, 0)])


def tc_dct(samples, d2, table, h, bA=7):
    """The transform of far_fill_tc.cu.  samples: ((re.hi, re.lo), (im.hi, im.lo))
    FP32 words of every Gauss-point pair's samples.  Rows on the grid
    2^(bA - e_r) of the bound |g| <= 1/|Delta|, the table on 2^sT (largest entry
    128), four integer digits each; one accumulator per digit level, each
    adding its products one 16-sample MMA step at a time in FP32 rounded toward
    zero (the worst case of a tensor core's accumulation)."""
    with np.errstate(divide="ignore"):                 # near pairs are zeroed afterwards
        v = 1.0 / np.sqrt(d2.astype(f32).astype(np.float64)) * (1.0 + 2.0 ** -10)
    e = np.frexp(v)[1][..., None]                      # v < 2^e
    sc = np.ldexp(1.0, bA - e).astype(f32)
    sT = 7 - (np.frexp(np.max(np.abs(table)))[1] - 1)
    T = _digits(np.ldexp(table, sT))
    out = []
    for hi, lo in samples:
        A = _digits_pair(hi, lo, sc)
        tot = np.zeros(hi.shape[:2] + (table.shape[1],))
        for L, grp in enumerate(TC_LEVELS):
            acc = np.zeros(tot.shape, f32)
            for k0 in range(0, h + 1, 16):
                ks = slice(k0, min(k0 + 16, h + 1))
                for sa, tb in grp:
                    acc = _add_rz(acc, np.einsum("rpj,jn->rpn", A[sa][..., ks], T[tb][ks]))
            tot += acc.astype(np.float64) * 2.0 ** (-8 * L)
        out.append(tot * np.ldexp(1.0, e - bA - sT))
    return out[0] + 1j * out[1]


class _Emulated(O.OracleSolver):
    variant = "fp64"

    def build_far(self, m_max, efie=True, mfie=False, workers=1, elem_range=None,
                  ibc_zs_pt=None):
        geom, _ = _modules()
        g = self.geo
        Nn, ne, go = g.Nn, g.ne, g.go
        nx = O.n_xi_efie(self.k, float(np.max(g.nodes[:, 0])), m_max)
        h = nx // 2
        dct, sin2 = geom.dct_tables(nx, m_max + 2, scale=1.0 / (4.0 * math.pi))
        self.Zp = np.zeros((9, m_max + 2, Nn, Nn), dtype=np.complex128)
        for e0 in range(0, ne, 4):
            e1 = min(e0 + 4, ne)
            rows = slice(e0 * go, e1 * go)
            rp, zp = g.rho[rows], g.z[rows]
            d2 = (rp[:, None] - g.rho[None, :]) ** 2 + (zp[:, None] - g.z[None, :]) ** 2
            a2 = 4.0 * rp[:, None] * g.rho[None, :]
            # coincident points belong to near pairs, which are zeroed below
            R = np.maximum(np.sqrt(d2[..., None] + a2[..., None] * sin2), 1e-30)
            g64 = np.exp(-1j * self.k * R) / R
            if self.variant == "fp64":
                Gn = np.einsum("rpj,jn->rpn", g64, dct)
            else:
                gr = np.clip(g64.real, -3e38, 3e38).astype(f32)
                gi = np.clip(g64.imag, -3e38, 3e38).astype(f32)
                if self.variant == "gpu":           # FP32 samples, FP32 table, Kahan blocks
                    Gn = kahan_dct(gr, gi, dct.astype(f32), h)
                elif self.variant == "table64":     # FP32 samples, FP64 table, Kahan blocks
                    Gn = kahan_dct(gr, gi, dct, h)
                elif self.variant == "digits4":     # 4 base-256 digits of g / 2^e and t / 2^f
                    # (the operand split of a tensor-core transform: row scale from
                    # |g| <= 1/d of the pair, table scale 2^f >= 4 max |t|)
                    with np.errstate(divide="ignore"):     # near pairs are zeroed below
                        ex = np.frexp(1.0 / np.sqrt(d2))[1][..., None]
                    sc = np.ldexp(1.0, ex)
                    q = 2.0 ** 31
                    gq = (np.rint(gr / sc * q) + 1j * np.rint(gi / sc * q)) * sc / q
                    fx = np.frexp(1.0 / h)[1]
                    tq = np.rint(dct / 2.0 ** fx * q) * 2.0 ** fx / q
                    Gn = np.einsum("rpj,jn->rpn", gq, tq)
                elif self.variant == "tc":          # the tensor-core fill (far_fill_tc.cu)
                    d2s = np.where(d2 > 0.0, d2, 1.0)[..., None]   # coincident points: near pairs
                    Gn = tc_dct(tc_green(d2s, a2[..., None], self.k, sin2[None, None, :]), d2, dct, h)
                else:                               # FP32 samples, exact transform
                    Gn = np.einsum("rpj,jn->rpn", gr.astype(np.float64) + 1j * gi.astype(np.float64), dct)
            self._zero_near(Gn, e0, e1)
            for ci, (lx, rx) in enumerate(self._COMBOS):
                self._contract(Gn, self.lv[lx][:, rows], self.lv[rx], e0, e1 - e0, self.Zp[ci])


def _far_field(pts, freq, thetas, M, variant):
    s = _Emulated(pts, freq)
    s.variant = variant
    s.prepare(M, efie=True, workers=4)
    F = np.zeros((2, len(thetas)), complex)
    for m in range(-M, M + 1):
        Z = s.assemble_efie(m, M)
        mask = s.basis_mask(m)
        V = np.stack([s.rhs_efie(m, thetas, "VV"), s.rhs_efie(m, thetas, "HH")], axis=1)
        B = V.transpose(2, 0, 1).reshape(2 * s.geo.Nn, -1)[mask]
        X = np.linalg.solve(Z[np.ix_(mask, mask)], B)
        full = np.zeros((2 * s.geo.Nn, X.shape[1]), complex)
        full[mask] = X
        xs = full.T.reshape(len(thetas), 2, -1)
        F[0] += s.farfield(m, xs[:, 0, :], thetas)[0]
        F[1] += s.farfield(m, xs[:, 1, :], thetas)[1]
    return F


def test_fp32_dct_table_sets_the_far_fill_floor():
    _, bodies = _modules()
    pts = bodies.cone_sphere_generatrix(0.5, 15.0, 80)
    freq = 10.0 * 299792458.0 / (2 * math.pi)
    thetas = np.arange(0.0, 180.0001, 2.0)
    M = 8
    ref = _far_field(pts, freq, thetas, M, "fp64")
    err = {}
    for v in ("gpu", "table64", "exact", "digits4", "tc"):
        F = _far_field(pts, freq, thetas, M, v)
        err[v] = float(np.max(np.abs(F - ref)) / np.max(np.abs(ref)))
    assert 1e-9 < err["gpu"] < 1e-7, err               # the FP32 floor (C2 on the GPU: 4.2e-8)
    assert err["table64"] < err["gpu"] / 2.5, err
    assert err["exact"] < err["gpu"] / 5.0, err
    # four digits per operand keep the exact transform's accuracy
    assert err["digits4"] < 1.2 * err["exact"], err
    # the tensor-core fill (samples as FP32 word pairs ~50x more accurate than
    # FP32, four integer digits, one truncating accumulator per digit level)
    # removes most of the FP32-sample floor as well
    assert err["tc"] < err["exact"] / 3.0, err
