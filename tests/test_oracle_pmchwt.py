"""The oracle's PMCHWT restatements against the reference.

Pinned to fixtures made by tests/golden/make_pmchwt_golden.py with the
reference's own solvers: the interior EFIE operator in a lossy medium
(complex k), the PMCHWT operators P of both media and full solves for lossy,
lossless and lossy magnetic spheres (pmchwt_sphere_n24.npz); the cross-surface
T and P and the solve of a coated PEC sphere (coated_sphere.npz); a PEC
sphere under two layers through the multi-region system (layered_sphere.npz);
the dielectric- and coated-sphere Mie series.  These are the operators a GPU
PMCHWT path would be checked against.
"""
import numpy as np
import pytest

from conftest import load_golden


@pytest.fixture(scope="module")
def D():
    return load_golden("pmchwt_sphere_n24")


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def test_interior_efie_and_pmchwt_operators(oracle, D):
    M = int(D["m_max"])
    f = float(D["freq_hz"])
    se = oracle.OracleSolver(D["points"], f)
    si = oracle.OracleSolver(D["points"], f, medium=tuple(D["media"][0]))
    ones = np.ones(se.geo.P)
    for s in (se, si):
        s.prepare(M, efie=True, workers=4, ibc_zs_pt=ones)
    for m in D["modes"]:
        m = int(m)
        assert _rel(si.assemble_efie(m, M), D[f"Ti_{m}"]) < 1e-12, m
        assert _rel(se.pmchwt_P(m, M), D[f"Pe_{m}"]) < 1e-12, m
        assert _rel(si.pmchwt_P(m, M), D[f"Pi_{m}"]) < 1e-12, m


@pytest.mark.parametrize("i", [0, 1, 2])
def test_pmchwt_solve_matches_reference(oracle, D, i):
    eps, mu = D["media"][i]
    r = oracle.solve_bor_dielectric(D["points"], float(D["freq_hz"]), D["thetas"], eps, mu,
                                    n_modes=int(D["m_max"]), mode_tol=0.0, workers=4)
    assert _rel(r["amp_vv"], D[f"amp_vv_{i}"]) < 1e-10
    assert _rel(r["amp_hh"], D[f"amp_hh_{i}"]) < 1e-10
    assert r["n_unknowns"] == 4 * len(D["points"])


def test_dielectric_mie_matches_reference(D):
    from oracle import mie
    for (a, f, er, ei, ur, ui), want in zip(D["mie_cases"], D["mie_sigma"]):
        got = mie.sigma_dielectric_sphere(a, complex(er, ei), complex(ur, ui), f)
        assert abs(got - want) <= 1e-14 * want
    # a relative permittivity and permeability of 1 scatter nothing
    assert mie.sigma_dielectric_sphere(0.5, 1.0, 1.0, 3e8) < 1e-30


def test_causal_medium_branch(oracle):
    m, eta_r = oracle.causal_medium(4.0 - 1.0j, 1.0)
    assert m.imag <= 0.0 and m.real >= 0.0
    assert abs(m * m - (4.0 - 1.0j)) < 1e-14 and abs(eta_r - 1.0 / m) < 1e-15


def test_magnetic_current_far_field_by_reciprocity(oracle, D):
    """The far field of a magnetic current m (nodal, like the PMCHWT M) is the
    reciprocity dot with the OTHER polarisation's E excitation:
    F_theta^M = (j k / 4 pi) (D V_HH)^T m, F_phi^M = (j k / 4 pi) (D V_VV)^T m --
    so a GPU far field needs no second projection kernel."""
    import math
    s = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    Nn = s.geo.Nn
    th = np.array([15.0, 60.0, 90.0, 140.0])
    Dg = np.concatenate([np.ones(Nn), -np.ones(Nn)])
    pm = 1j * s.k / (4 * math.pi)
    rng = np.random.default_rng(5)
    for m in (0, 1, -3):
        x = np.zeros((len(th), 2 * Nn), complex)
        msol = rng.standard_normal((len(th), 2 * Nn)) + 1j * rng.standard_normal((len(th), 2 * Nn))
        fth, fph = s.farfield(m, x, th, msol=msol)
        want_th = pm * np.sum(Dg * s.rhs_efie(m, th, "HH") * msol, axis=1)
        want_ph = pm * np.sum(Dg * s.rhs_efie(m, th, "VV") * msol, axis=1)
        assert np.max(np.abs(fth - want_th)) <= 1e-13 * np.max(np.abs(want_th))
        assert np.max(np.abs(fph - want_ph)) <= 1e-13 * np.max(np.abs(want_ph))


@pytest.fixture(scope="module")
def Dc():
    return load_golden("coated_sphere")


def test_cross_operators_match_reference(oracle, Dc):
    """T and P between the coating and the core, both directions (the cross
    terms of the coated system), against the reference's BorCrossOperators."""
    M, f, medium = int(Dc["m_max"]), float(Dc["freq_hz"]), (complex(Dc["eps"]), complex(Dc["mu"]))
    so = oracle.OracleSolver(Dc["outer"], f, medium=medium)
    sc = oracle.OracleSolver(Dc["core"], f, medium=medium)
    for X, tag in ((oracle.CrossOperators(so, sc), "oc"), (oracle.CrossOperators(sc, so), "co")):
        assert X.near_pairs                     # the thin layer puts pairs on the near grid
        assert _rel(X.assemble_T(1, M), Dc[f"T_{tag}"]) < 1e-12, tag
        assert _rel(X.assemble_P(1, M), Dc[f"P_{tag}"]) < 1e-12, tag


def test_coated_pec_solve_matches_reference(oracle, Dc):
    r = oracle.solve_bor_coated_pec(Dc["outer"], Dc["core"], float(Dc["freq_hz"]), Dc["thetas"],
                                    complex(Dc["eps"]), complex(Dc["mu"]), n_modes=int(Dc["m_max"]),
                                    mode_tol=0.0, workers=4)
    assert _rel(r["amp_vv"], Dc["amp_vv"]) < 1e-10
    assert _rel(r["amp_hh"], Dc["amp_hh"]) < 1e-10
    assert r["n_unknowns"] == 4 * len(Dc["outer"]) + 2 * len(Dc["core"])


def test_coated_mie_matches_reference(Dc):
    from oracle import mie
    for (b, a, f, er, ei, ur, ui), want in zip(Dc["mie_cases"], Dc["mie_sigma"]):
        got = mie.sigma_coated_pec_sphere(b, a, complex(er, ei), complex(ur, ui), f)
        assert abs(got - want) <= 1e-14 * want
    with pytest.raises(ValueError):
        mie.sigma_coated_pec_sphere(0.5, 0.4, 2.0, 1.0, 3e8)


def test_cross_operators_reject_junctions(oracle):
    """Surfaces sharing an endpoint (coating terminations) are not restated."""
    import importlib
    bodies = importlib.import_module("20260722_ghost_gb300.bodies")
    a = bodies.sphere_generatrix(0.5, 8)
    b = a.copy()
    b[1:-1, 0] *= 0.8                          # same poles: the two surfaces touch on the axis
    sa, sb = oracle.OracleSolver(a, 3e8), oracle.OracleSolver(b, 3e8)
    with pytest.raises(NotImplementedError):
        oracle.CrossOperators(sa, sb)


def test_two_layer_coated_pec_matches_reference(oracle):
    """The multi-region system (no junctions): a PEC core under two full
    layers, against the reference's solve_bor_coated2_pec."""
    L = load_golden("layered_sphere")
    r = oracle.solve_bor_coated2_pec(L["outer"], L["mid"], L["core"], float(L["freq_hz"]), L["thetas"],
                                     *L["media"], n_modes=int(L["m_max"]), mode_tol=0.0, workers=4)
    assert r["n_unknowns"] == int(L["n_unknowns"])
    assert _rel(r["amp_vv"], L["amp_vv"]) < 1e-10
    assert _rel(r["amp_hh"], L["amp_hh"]) < 1e-10
