"""Pin the CPU oracle to golden vectors produced by the reference itself."""
import numpy as np
import pytest

from conftest import load_golden

SOLVER_CASES = ("sphere_n24", "conesphere_n40", "openshell_n20")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def test_near_kernels(oracle):
    G = load_golden("kernels")
    g = oracle.near_G(G["near_rp"], G["near_zp"], G["near_rq"], G["near_zq"],
                      float(G["near_k"]), int(G["near_m_max"]))
    ok = np.all(np.isfinite(G["near_G"]), axis=1)
    assert rel(g[ok], G["near_G"][ok]) < 1e-14
    sel = slice(6, None)
    K = oracle.near_mfie(G["near_rp"][sel], G["near_zp"][sel], G["near_trp"][sel],
                         G["near_tzp"][sel], G["near_rq"][sel], G["near_zq"][sel],
                         G["near_trq"][sel], G["near_tzq"][sel], float(G["near_k"]),
                         int(G["near_m_max"]))
    for i, n in enumerate(("tt", "tf", "ft", "ff")):
        assert rel(K[i], G[f"near_K_{n}"]) < 1e-14


def test_cells_and_nxi(oracle):
    G = load_golden("kernels")
    for kind in ("diag", "corner10", "corner01"):
        s, sp, w = oracle.cell_points(kind)
        np.testing.assert_array_equal(np.stack([s, sp, w]), G[f"cells_{kind}"])
    for (k, r, m), (ne, nb) in zip(((10, 1, 20), (80, .5, 50), (200, .5, 120), (40, .6, 30), (3, .1, 2)),
                                   G["n_xi"]):
        assert oracle.n_xi_efie(k, r, m) == ne
        assert oracle.n_xi_bracket(k, r, m) == nb


@pytest.mark.parametrize("name", SOLVER_CASES)
def test_per_mode_operators(oracle, name):
    D = load_golden(name)
    cfie = "Zm_0" in D
    s = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    M = int(D["m_max"])
    s.prepare(M, efie=True, mfie=cfie)
    th = D["thetas"]
    for m in D["modes"]:
        m = int(m)
        assert rel(s.assemble_efie(m, M), D[f"Ze_{m}"]) < 1e-13
        if cfie:
            assert rel(s.assemble_mfie(m, M), D[f"Zm_{m}"]) < 1e-13
        for pol in ("VV", "HH"):
            assert rel(s.rhs_efie(m, th, pol), D[f"Ve_{m}_{pol}"]) < 1e-13
            if cfie:
                assert rel(s.rhs_mfie(m, th, pol), D[f"Vm_{m}_{pol}"]) < 1e-13
        x = D[f"ffx_{m}"]
        fth, fph = s.farfield(m, np.tile(x, (len(th), 1)), th)
        assert rel(np.stack([fth, fph], 1), D[f"ff_{m}"]) < 1e-13
        np.testing.assert_array_equal(s.basis_mask(m), D[f"mask_{m}"])


@pytest.mark.parametrize("name", SOLVER_CASES)
def test_full_solve(oracle, name):
    D = load_golden(name)
    forms = ("efie", "cfie") if "Zm_0" in D else ("efie",)
    for form in forms:
        r = oracle.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], formulation=form,
                             n_modes=int(D["m_max"]), mode_tol=0.0, workers=2)
        assert rel(r["amp_vv"], D[f"{form}_amp_vv"]) < 1e-12
        assert rel(r["amp_hh"], D[f"{form}_amp_hh"]) < 1e-12


def test_mie(oracle):
    from oracle import mie
    M = load_golden("mie")
    for ka, s0 in zip(M["ka"], M["sigma"]):
        s = mie.sigma_pec_sphere(float(M["a"]), oracle.C0 * ka / (2 * np.pi))
        assert abs(s / s0 - 1) < 1e-13


@pytest.mark.slow
def test_c1_sphere(oracle):
    """The 240-segment sphere (ka = 10, |m| <= 20, 181 angles) against the reference."""
    D = load_golden("c1_sphere")
    r = oracle.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], n_modes=20,
                         mode_tol=0.0, workers=8)
    assert rel(r["amp_vv"], D["amp_vv"]) < 1e-12
    assert rel(r["amp_hh"], D["amp_hh"]) < 1e-12
