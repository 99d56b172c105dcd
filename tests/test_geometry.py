"""Host-side set-up of the package (product code) against the oracle/golden."""
import math

import numpy as np
import pytest

from conftest import load_golden


def test_cells_match_golden(pkg):
    G = load_golden("kernels")
    for kind in ("diag", "corner10", "corner01"):
        s, sp, w = pkg.geometry.cell_points(kind)
        np.testing.assert_array_equal(np.stack([s, sp, w]), G[f"cells_{kind}"])


def test_nxi_rules(pkg):
    G = load_golden("kernels")
    for (k, r, m), (ne, nb) in zip(((10, 1, 20), (80, .5, 50), (200, .5, 120), (40, .6, 30), (3, .1, 2)),
                                   G["n_xi"]):
        assert pkg.geometry.n_xi_efie(k, r, m) == ne
        assert pkg.geometry.n_xi_bracket(k, r, m) == nb


@pytest.mark.parametrize("name", ["sphere_n24", "conesphere_n40", "openshell_n20"])
def test_gauss_and_masks(pkg, oracle, name):
    D = load_golden(name)
    geo = pkg.geometry
    gen = geo.Generatrix(D["points"])
    g = geo.gauss_on_generatrix(gen)
    o = oracle.Geom(D["points"])
    for a, b in ((g.rho, o.rho), (g.z, o.z), (g.w, o.w), (g.dRT0, o.dRT0), (g.dRT1, o.dRT1)):
        np.testing.assert_array_equal(a, b)
    M = int(D["m_max"])
    rows = geo.mask_rows(gen, M)
    for m in range(M + 1):
        want = np.flatnonzero(~D[f"mask_{m}"]) if f"mask_{m}" in D else np.flatnonzero(
            ~oracle.OracleSolver(D["points"], float(D["freq_hz"])).basis_mask(m))
        got = rows[m][rows[m] >= 0]
        np.testing.assert_array_equal(np.sort(got), want)


def test_dct_equals_fft(pkg):
    """The half-grid DCT tables reproduce the reference's full-grid FFT of an
    even integrand (bor_kernels.py:160-167) to rounding."""
    rng = np.random.default_rng(3)
    n_xi, M = 64, 10
    rp, rq, zp, zq = rng.uniform(0.2, 1.0, 4)
    k = 5.0
    xi = 2 * np.pi * np.arange(n_xi) / n_xi - np.pi
    R = np.sqrt((rp - rq) ** 2 + (zp - zq) ** 2 + 4 * rp * rq * np.sin(xi / 2) ** 2)
    g = np.exp(-1j * k * R) / (4 * np.pi * R)
    ref = np.fft.fft(g)[:M + 2] * np.exp(1j * np.pi * np.arange(M + 2)) * (2 * np.pi / n_xi)
    dct, sin2 = pkg.geometry.dct_tables(n_xi, M + 2)
    Rh = np.sqrt((rp - rq) ** 2 + (zp - zq) ** 2 + 4 * rp * rq * sin2)
    gh = np.exp(-1j * k * Rh) / (4 * np.pi * Rh)
    got = gh @ dct
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-14


@pytest.mark.parametrize("name", ["sphere_n24", "conesphere_n40"])
def test_near_tail_orders(pkg, oracle, name):
    """n_tail per element pair equals the order the reference's near kernel picks."""
    D = load_golden(name)
    geo = pkg.geometry
    gen = geo.Generatrix(D["points"])
    k = 2 * math.pi * float(D["freq_hz"]) / geo.C0
    M = int(D["m_max"])
    nt = geo.near_tables(gen, k, M)
    og = oracle.Geom(D["points"])
    for (e, f, _, _), n in zip(nt.pairs, nt.n_tail):
        s, sp, _ = oracle.cell_points(oracle.near_kind(int(e), int(f)))
        rp = og.points_on_element(int(e), s)[0]
        rq = og.points_on_element(int(f), sp)[0]
        rr4 = 4.0 * rp * rq
        a = np.sqrt(rr4[rr4 > 1e-30])
        osc = float(np.max(abs(complex(k)) * a)) / math.pi + (M + 2)
        assert n == int(min(1024, max(64, math.ceil(4.0 * osc))))


def test_bodies(pkg):
    b = pkg.bodies
    p = b.cone_sphere_generatrix(0.5, 15.0, 120)
    seg = np.hypot(*np.diff(p, axis=0).T)
    assert p[0, 0] == 0.0 and p[-1, 0] == 0.0 and abs(p[0, 1] - 0.5 / math.sin(math.radians(15))) < 1e-12
    assert np.all(np.diff(p[:, 1]) < 0)
    assert seg.max() / seg.min() < 1.001
    bodies = b.random_bodies(4)
    assert all(200 <= x["n"] <= 1600 for x in bodies)
    s = b.sphere_generatrix(1.0, 8)
    np.testing.assert_allclose(np.hypot(s[:, 0], s[:, 1]), 1.0)


def test_bracket_tables_reproduce_reference_brackets(pkg, oracle):
    """Three half-grid transforms of p with the per-pair constants used by the
    MFIE far kernel give the reference's four bracket transforms (full-grid
    FFT of each bracket, bins m >= 0, 2 pi Galerkin factor)."""
    D = load_golden("conesphere_n40")
    geo = pkg.geometry
    gen = geo.Generatrix(D["points"])
    g = geo.gauss_on_generatrix(gen, 4)
    k = 2 * math.pi * float(D["freq_hz"]) / geo.C0
    M = int(D["m_max"])
    nb = geo.n_xi_bracket(k, float(np.max(gen.nodes[:, 0])), M)
    tab, s2 = geo.bracket_tables(nb, M)
    xi = 2 * np.pi * np.arange(nb) / nb - np.pi
    m = np.arange(M + 1)
    rng = np.random.default_rng(3)
    for _ in range(40):
        e = int(rng.integers(0, gen.n_elems))
        f = int(np.clip(e + rng.choice([-9, -3, -2, 2, 3, 9]), 0, gen.n_elems - 1))
        p, q = 4 * e + int(rng.integers(0, 4)), 4 * f + int(rng.integers(0, 4))
        args = [np.array([v]) for v in (g.rho[p], g.z[p], g.trho[p], g.tz[p],
                                        g.rho[q], g.z[q], g.trho[q], g.tz[q])]
        F = oracle._mfie_bracket_grid(*args, k, xi[None, :])
        want = [(np.fft.fft(Fi[0])[m] * np.exp(1j * np.pi * m) * 2 * np.pi / nb) * 2 * np.pi for Fi in F]
        rp, zp, trp, tzp, rq, zq, trq, tzq = (float(a[0]) for a in args)
        dr, dz = rp - rq, zp - zq
        R = np.sqrt(dr * dr + dz * dz + 4 * rp * rq * s2)
        pt = (1 + 1j * k * R) * np.exp(-1j * k * R) / R ** 3
        Cp, Cs, S = tab[0].T @ pt, tab[1].T @ pt, tab[2].T @ pt
        X0 = trp * tzq - tzp * trq
        N0 = trp * dz - tzp * dr
        A0 = trp * dr + tzp * dz
        D0 = trp * trq + tzp * tzq
        c0 = dr * tzq - dz * trq
        c1 = 2 * (A0 * tzp * trq + trp * rq * X0 + D0 * tzp * rq + trp * trq * N0)
        e0 = rq * X0 + trq * N0
        got = [-c0 * Cp - c1 * Cs, -1j * dz * S, 1j * e0 * S, N0 * Cp - 2 * (N0 - rq * tzp) * Cs]
        scale = max(np.max(np.abs(w)) for w in want)
        for gv, wv in zip(got, want):
            assert np.max(np.abs(gv - wv)) < 1e-11 * scale


def test_element_mass(pkg, oracle):
    D = load_golden("conesphere_n40")
    geo = pkg.geometry
    gen = geo.Generatrix(D["points"])
    em = geo.element_mass(geo.gauss_on_generatrix(gen, 4), gen.n_elems)
    Mm = np.zeros((gen.n_nodes, gen.n_nodes))
    for e in range(gen.n_elems):
        for ab in range(4):
            Mm[e + ab // 2, e + ab % 2] += em[e, ab]
    ref = oracle.OracleSolver(D["points"], float(D["freq_hz"])).mass()
    assert np.max(np.abs(Mm - ref)) < 1e-14 * np.max(np.abs(ref))


def test_gauss_legendre_rule_is_numpys(pkg):
    """The cached rule (tridiagonal eigensolver, then numpy's own refinement and
    weights) returns exactly numpy's leggauss nodes and weights."""
    g = pkg.geometry
    for n in (1, 4, 48, 63, 64, 65, 100, 257, 512, 777, 1024):
        x, w = np.polynomial.legendre.leggauss(n)
        x2, w2 = g._leggauss(n)
        assert np.array_equal(x, x2) and np.array_equal(w, w2), n


def test_rule_table_equals_computed_rules():
    """The Gauss-Legendre table written by the build holds exactly what
    _leggauss_compute returns (when the table is present)."""
    import importlib
    g = importlib.import_module("20260722_ghost_gb300.geometry")
    if not g.leggauss_table_ok():
        pytest.skip("rule table not built")
    for n in (64, 65, 100, 257, 512, 1000, 1024):
        x, w = g._leg_from_table(n)
        xc, wc = g._leggauss_compute(n)
        assert np.array_equal(x, xc) and np.array_equal(w, wc), n


def test_random_batch_matches_its_definition(pkg):
    """The 64-body batch (seed 0): closed bodies drawn from +z to -z with
    rho >= 0, equal-arc segments, 12 segments per wavelength, the stated
    parameter ranges and |m| rule, and the same arrays for the same seed."""
    b = pkg.bodies
    batch = b.random_bodies(64, seed=0)
    again = b.random_bodies(64, seed=0)
    assert len(batch) == 64
    for x, y in zip(batch, again):
        assert np.array_equal(x["points"], y["points"]) and x["freq_hz"] == y["freq_hz"]
    for x in batch:
        p = x["points"]
        assert len(p) == x["n"] + 1 and 200 <= x["n"] <= 1600
        assert p[0, 0] == pytest.approx(0.0, abs=1e-12) and p[-1, 0] == pytest.approx(0.0, abs=1e-12)
        assert np.all(p[:, 0] >= -1e-12) and p[0, 1] > p[-1, 1]
        seg = np.hypot(*np.diff(p, axis=0).T)
        assert seg.max() / seg.min() < 1.01
        assert 1.0 <= x["L"] <= 4.0 and 0.2 <= x["R0"] <= 0.8
        assert all(abs(a) <= 0.1 / (i + 1) for i, a in enumerate(x["a_k"]))
        arclen = seg.sum()
        assert x["k"] * arclen / x["n"] == pytest.approx(2.0 * math.pi / 12.0, rel=1e-12)
        assert x["m_max"] == math.ceil(x["k"] * p[:, 0].max()) + 10
    assert len({x["n"] for x in batch}) > 50             # the sizes spread over the range


def test_bspline_body_definition(pkg):
    """The B-spline body of the gradient workload: clamped cubic basis (a
    partition of unity), closed on the axis from z = +1 to z = -1, radii
    bounded by the control radii, monotone in z (the control z are)."""
    b = pkg.bodies
    radii = np.random.default_rng(0).uniform(0.3, 0.6, 64)
    pts, B = b.bspline_body(radii, 600)
    assert pts.shape == (601, 2) and B.shape == (601, 66)
    np.testing.assert_allclose(B.sum(axis=1), 1.0, atol=1e-14)
    assert np.all(B >= -1e-15)
    assert pts[0, 0] == 0.0 and pts[-1, 0] == 0.0
    assert pts[0, 1] == pytest.approx(1.0) and pts[-1, 1] == pytest.approx(-1.0)
    assert np.all(np.diff(pts[:, 1]) < 0)
    assert np.all(pts[1:-1, 0] > 0.0) and pts[:, 0].max() <= radii.max() + 1e-12


def test_near_tail_orders_equal_the_pointwise_rule(pkg):
    """The tail order of every near pair (row maxima of 4 rho rho' taken
    before the square root, in row blocks) equals the pointwise rule
    clip(ceil(4 (max_points |k| sqrt(4 rho rho') / pi + m_max + 2)), 64, 1024),
    points with 4 rho rho' <= 1e-30 left out and 0 for pairs wholly on the
    axis, exactly; the pairs come sorted by (e, f)."""
    import math
    geom = pkg.geometry
    rng = np.random.default_rng(5)
    for trial in range(4):
        N = int(rng.integers(8, 300))
        t = np.linspace(0.0, 1.0, N + 1)
        rho = rng.uniform(0.2, 0.6) * np.sin(np.pi * t) * (1 + 0.1 * np.sin(5 * np.pi * t))
        gen = geom.Generatrix(np.stack([rho, 1.3 * (0.5 - t)], axis=1))
        k, M = float(rng.uniform(3, 90)), int(rng.integers(2, 60))
        nt = geom.near_tables(gen, k, M)
        x0, x1 = gen.nodes[:-1], gen.nodes[1:]
        cells = nt.cells
        for (e, f, coff, cnt), (toff, n) in zip(nt.pairs, nt.tails):
            s, sp = cells[0, coff:coff + cnt], cells[1, coff:coff + cnt]
            rp = x0[e, 0] + s * (x1[e, 0] - x0[e, 0])
            rq = x0[f, 0] + sp * (x1[f, 0] - x0[f, 0])
            rr4 = 4.0 * rp * rq
            if not np.any(rr4 > 1e-30):
                assert n == 0
                continue
            osc = np.max(k * np.sqrt(np.where(rr4 > 1e-30, rr4, 0.0))) / math.pi + (M + 2)
            assert n == min(1024, max(64, math.ceil(4.0 * osc))), (e, f)
            assert np.array_equal(nt.tail_gl[0, toff:toff + n], 0.5 * (geom._leggauss(n)[0] + 1.0))
        assert np.all(np.diff(nt.pairs[:, 0] * 4 + nt.pairs[:, 1] - nt.pairs[:, 0]) > 0)
