"""The oracle's homogeneous-dielectric PMCHWT restatement against the reference.

Pinned to tests/golden/pmchwt_sphere_n24.npz (tests/golden/make_pmchwt_golden.py,
the reference's own solve_bor_dielectric path): the interior EFIE operator in
a lossy medium (complex k), the PMCHWT operators P of both media, full solves
for lossy, lossless and lossy magnetic spheres, and the dielectric-sphere Mie
series.  These are the operators a GPU PMCHWT path would be checked against.
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
