"""The oracle's surface-impedance (IBC-EFIE) restatement against the reference.

Pinned to tests/golden/ibc_conesphere_n40.npz, made by running the reference
(tests/golden/make_ibc_golden.py): the per-mode IBC operator additions, full
solves with a tapered and a scalar Z_s, and the impedance-sphere Mie series.
Also checks the algebra a GPU fill of the IBC brackets relies on: the four
rotated principal-value brackets are p(R) times {1, sin^2(xi/2), sin(xi)}
with per-pair coefficients -- the same three azimuth transforms of p as the
MFIE brackets, so only the coefficients and the (complex, per source element)
Z_s weight differ -- and the far field of J and the eliminated magnetic
current by reciprocity with a modified excitation.
"""
import math

import numpy as np
import pytest

from conftest import load_golden


@pytest.fixture(scope="module")
def D():
    return load_golden("ibc_conesphere_n40")


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def test_ibc_operator_matches_reference(oracle, D):
    s = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    zs = D["zs_taper"]
    zs_pt = zs[s.geo.elem]
    m_max = int(D["m_max"])
    s.prepare(m_max, efie=False, mfie=False, workers=4, ibc_zs_pt=zs_pt)
    for m in D["modes"]:
        assert _rel(s.assemble_ibc_extra(int(m), m_max, zs_pt, zs), D[f"Zi_{m}"]) < 1e-12, m


@pytest.mark.parametrize("tag", ["taper", "scalar"])
def test_ibc_solve_matches_reference(oracle, D, tag):
    zs = D["zs_taper"] if tag == "taper" else 120.0 - 80.0j
    r = oracle.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], formulation="efie",
                         zs=zs, n_modes=int(D["m_max"]), mode_tol=0.0, workers=4)
    assert _rel(r["amp_vv"], D[f"amp_vv_{tag}"]) < 1e-10
    assert _rel(r["amp_hh"], D[f"amp_hh_{tag}"]) < 1e-10


def test_impedance_mie_matches_reference(D):
    from oracle import mie
    for (a, f, zr, zi), want in zip(D["mie_cases"], D["mie_sigma"]):
        got = mie.sigma_impedance_sphere(a, f, complex(zr, zi))
        assert abs(got - want) <= 1e-14 * max(abs(want), 1e-300)
    # Weston: a Z_s = eta0 sphere has no backscatter; Z_s = 0 is the PEC sphere
    assert mie.sigma_impedance_sphere(1.0, 477.1e6, mie.ETA0) == 0.0
    assert mie.sigma_impedance_sphere(1.0, 477.1e6, 0.0) == mie.sigma_pec_sphere(1.0, 477.1e6)


def test_ibc_input_errors(oracle, D):
    with pytest.raises(ValueError):
        oracle.solve_bor(D["points"], float(D["freq_hz"]), [0.0], formulation="cfie", zs=50.0,
                         n_modes=2)
    with pytest.raises(ValueError):
        oracle.solve_bor(D["points"], float(D["freq_hz"]), [0.0], zs=np.ones(3), n_modes=2)


def test_ibc_brackets_reduce_to_three_transforms(oracle):
    """B_tt = p (-N0 - 2 s2 (t_z rho - t_rho dz)),  B_ff = p (c0 + 2 s2 (t'_z rho' + t'_rho dz)),
    B_tf = p sin(xi) (t_z t'_rho rho - t_rho t'_z rho' - t_rho t'_rho dz),  B_ft = p sin(xi) dz,
    with d = (dr, dz) = test - source, N0 = t_rho dz - t_z dr, c0 = dr t'_z - dz t'_rho,
    s2 = sin^2(xi/2); t = test tangent, t' = source tangent (unit)."""
    rng = np.random.default_rng(7)
    n = 400
    rp, rq = rng.uniform(0.05, 1.0, n), rng.uniform(0.05, 1.0, n)
    zp, zq = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    a, b = rng.uniform(0, 2 * math.pi, n), rng.uniform(0, 2 * math.pi, n)
    trp, tzp, trq, tzq = np.cos(a), np.sin(a), np.cos(b), np.sin(b)
    # near pairs too: sources a few 1e-3 away from the test point
    rq[:100] = rp[:100] + rng.uniform(-3e-3, 3e-3, 100)
    zq[:100] = zp[:100] + rng.uniform(-3e-3, 3e-3, 100)
    xi = rng.uniform(-math.pi, math.pi, (n, 64))
    xi[:100, :8] = rng.uniform(-1e-2, 1e-2, (100, 8))
    k = 30.0
    B = oracle._ibc_bracket_grid(rp, zp, trp, tzp, rq, zq, trq, tzq, k, xi)
    dr, dz = (rp - rq)[:, None], (zp - zq)[:, None]
    R = np.sqrt(dr ** 2 + dz ** 2 + 4 * (rp * rq)[:, None] * np.sin(xi / 2) ** 2)
    p = (1 + 1j * k * R) * np.exp(-1j * k * R) / (4 * np.pi * R ** 3)
    s2, sx = np.sin(xi / 2) ** 2, np.sin(xi)
    tr_p, tz_p, tr_q, tz_q = (v[:, None] for v in (trp, tzp, trq, tzq))
    N0 = tr_p * dz - tz_p * dr
    c0 = dr * tz_q - dz * tr_q
    red = (p * (-N0 - 2 * s2 * (tz_p * rp[:, None] - tr_p * dz)),
           p * sx * (tz_p * tr_q * rp[:, None] - tr_p * tz_q * rq[:, None] - tr_p * tr_q * dz),
           p * sx * dz,
           p * (c0 + 2 * s2 * (tz_q * rq[:, None] + tr_q * dz)))
    # bound: |p| times the size of the largest product term (rho ~ 1)
    scale = np.abs(p) * (1.0 + np.abs(dz) + rp[:, None] + rq[:, None])
    for got, want in zip(red, B):
        assert np.max(np.abs(got - want) / scale) < 1e-13


def test_ibc_far_field_by_reciprocity(oracle):
    """The far field of J plus the eliminated M = -Z_s n x J equals the PEC
    reciprocity form with the excitation V_E - V_H^Zs:
    F_theta = c (D (V_E,VV - V_H,VV^Zs))^T x, F_phi = -c (D (V_E,HH - V_H,HH^Zs))^T x,
    c = -j k eta0 / 4 pi, D = diag(I, -I), V_H^Zs the rotated n x H_inc
    excitation with Gauss weights w rho Z_s -- so a GPU far field needs only
    those excitation vectors, not a second projection."""
    import importlib
    bodies = importlib.import_module("20260722_ghost_gb300.bodies")
    s = oracle.OracleSolver(bodies.cone_sphere_generatrix(0.3, 15.0, 24), 20.0 * oracle.C0 / (2 * math.pi))
    g = s.geo
    rng = np.random.default_rng(3)
    zs_pt = (rng.uniform(20, 300, g.ne) + 1j * rng.uniform(-100, 100, g.ne))[g.elem]
    th = np.array([10.0, 47.0, 90.0, 133.0])
    Dg = np.concatenate([np.ones(g.Nn), -np.ones(g.Nn)])
    c = -1j * s.k * oracle.ETA0 / (4 * math.pi)

    def v_h(m, pol):                          # rhs_mfie with Gauss weights w rho Z_s
        st, ct, P, Ic, Is, I1 = s._bessel_parts(m, th, 1)
        if pol == "VV":
            et, ef = Ic, -(g.ptr * Is)
        else:
            et, ef = ct * Is, ct * g.ptr * Ic - st * g.ptz * I1
        w = g.w * g.rho * P * zs_pt / oracle.ETA0
        return np.concatenate([(w * et) @ g.BT.T, (w * ef) @ g.BT.T], axis=1)

    for m in (0, 1, -2, 3):
        x = rng.standard_normal((len(th), 2 * g.Nn)) + 1j * rng.standard_normal((len(th), 2 * g.Nn))
        fth, fph = s.farfield(m, x, th, zs_pt=zs_pt)
        rth = c * np.sum(Dg * (s.rhs_efie(m, th, "VV") - v_h(m, "VV")) * x, axis=1)
        rph = -c * np.sum(Dg * (s.rhs_efie(m, th, "HH") - v_h(m, "HH")) * x, axis=1)
        assert np.max(np.abs(rth - fth)) <= 1e-13 * np.max(np.abs(fth))
        assert np.max(np.abs(rph - fph)) <= 1e-13 * np.max(np.abs(fph))


def _pair_coefs(kind, rp, zp, trp, tzp, rq, zq, trq, tzq):
    """Per-pair coefficients (c0..c5) of the three-transform bracket fill:
    K_tt = c0 C[p] + c1 C[p s2], K_ff = c2 C[p] + c3 C[p s2], K_tf = -j c4 S,
    K_ft = -j c5 S.  "mfie": the set of csrc/mfie_fill.cu (bracket_coefs);
    "ibc": the rotated principal-value brackets of the identity above."""
    dr, dz = rp - rq, zp - zq
    if kind == "mfie":
        X0, N0 = trp * tzq - tzp * trq, trp * dz - tzp * dr
        A0, D0 = trp * dr + tzp * dz, trp * trq + tzp * tzq
        c0 = dr * tzq - dz * trq
        c1 = 2.0 * (A0 * tzp * trq + trp * rq * X0 + D0 * tzp * rq + trp * trq * N0)
        return [-c0, -c1, N0, -2.0 * (N0 - rq * tzp), dz, -(rq * X0 + trq * N0)]
    return [-(trp * dz - tzp * dr), -2.0 * (tzp * rp - trp * dz), dr * tzq - dz * trq,
            2.0 * (tzq * rq + trq * dz), tzp * trq * rp - trp * tzq * rq - trp * trq * dz, dz]


@pytest.mark.parametrize("kind", ["mfie", "ibc"])
def test_three_transform_fill_reproduces_bracket_blocks(oracle, pkg, kind):
    """The GPU bracket fill's formulation, emulated on the host: half-grid
    transforms C[p], C[p s2], S of p = (1 + jkR) e^{-jkR} / R^3 with the
    kernel's own tables (geometry.bracket_tables), per-pair coefficients, the
    -j sine convention and the T w rho Galerkin weights.  With the MFIE set it
    reproduces the oracle's FFT-of-brackets MFIE blocks, with the IBC set its
    unit-weight IBC blocks (m = 0..M)."""
    geom = pkg.geometry
    pts = pkg.bodies.cone_sphere_generatrix(0.3, 15.0, 24)
    k, M = 20.0, 6
    o = oracle.OracleSolver(pts, k * oracle.C0 / (2 * math.pi))
    o.build_far(M, efie=False, mfie=kind == "mfie",
                ibc_zs_pt=np.ones(o.geo.P) if kind == "ibc" else None)
    store = o.Kb if kind == "mfie" else o.Bb
    gen = geom.Generatrix(pts)
    geo = geom.pack_geo(geom.gauss_on_generatrix(gen, 4))
    N, P = gen.n_elems, 4 * gen.n_elems
    tab, s2 = geom.bracket_tables(geom.n_xi_bracket(k, float(np.max(gen.nodes[:, 0])), M), M)
    rho, z, tr, tz = geo[0], geo[1], geo[9], geo[10]
    e_of = np.arange(P) // 4
    pi, qi = np.meshgrid(np.arange(P), np.arange(P), indexing="ij")
    far = (np.abs(e_of[pi] - e_of[qi]) >= 2)[..., None]
    R = np.maximum(np.sqrt(((rho[pi] - rho[qi]) ** 2 + (z[pi] - z[qi]) ** 2)[..., None]
                           + (4 * rho[pi] * rho[qi])[..., None] * s2), 1e-30)
    p = (1 + 1j * k * R) * np.exp(-1j * k * R) / R ** 3
    T = np.einsum("pqj,tjm->tpqm", p, tab)
    c = [x[..., None] for x in _pair_coefs(kind, rho[pi], z[pi], tr[pi], tz[pi], rho[qi], z[qi],
                                           tr[qi], tz[qi])]
    K = [c[0] * T[0] + c[1] * T[1], -1j * c[4] * T[2], -1j * c[5] * T[2], c[2] * T[0] + c[3] * T[1]]
    W = np.zeros((N + 1, P))
    W[e_of, np.arange(P)] += geo[3]
    W[e_of + 1, np.arange(P)] += geo[4]
    scale = np.max(np.abs(store))
    for uv in range(4):
        got = np.einsum("ip,pqm,jq->mij", W, K[uv] * far, W)
        assert np.max(np.abs(got - store[uv, M:])) <= 1e-13 * scale, uv
